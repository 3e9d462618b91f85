"""Pins the oracle to the reference's own known-answer tests (tests/golden/reference_kat.json,
read from Old/tests/*.hpp) and to the published Philox4x32-10 test vectors."""
import json
import os

import numpy as np
import pytest

from nanomagmc_gb300.sampler import interactions_file
from oracle import oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
KAT = json.load(open(os.path.join(HERE, "golden", "reference_kat.json")))


def fixture(kind, ising, periodic, D=0.0):
    off, J, Dv = O.read_interactions(interactions_file("3d_nn_bloch.dat"), 3, 1.0,
                                     0.75 if kind == "skyrm" else D)
    lat = O.Lattice.fixture(kind, 3, ising, periodic, off, J, Dv)
    lat.set_flags(useJ=True, useD=False)   # exchangeOnly (Old/tests/test.cpp:18)
    return lat


@pytest.mark.parametrize("case", KAT["cases"], ids=lambda c: c["src"] + ":" + c["fixture"])
def test_reference_kat(case):
    lat = fixture(case["fixture"], case["ising"], case["periodic"])
    if "H" in case:
        lat.set_H(*case["H"])
    if "E" in case:
        assert lat.energy() == pytest.approx(case["E"], abs=1e-9)
    if "M" in case:
        assert np.allclose(lat.mag(), case["M"], atol=1e-9)
    if "subM" in case:
        assert np.allclose(lat.submag(0), case["subM"], atol=1e-9)
    if "sub4M" in case:
        assert np.allclose(lat.sub4mag(), case["sub4M"], atol=1e-9)
    if "Q_each" in case:
        q = lat.tcharge()
        assert len(q) == 10 if case["fixture"] == "fm" else len(q) == 30
        assert np.all(np.abs(q - case["Q_each"]) <= case["Q_tol"])


@pytest.mark.parametrize("case", KAT["dE_consistency"], ids=lambda c: c["src"])
def test_dE_consistency(case):
    """E_old + dE == E_new over random proposals (the reference's *_dE_consist tests)."""
    lat = fixture(case["fixture"], case["ising"], 0)
    lat.set_H(*case["H"])
    rng = O.Rng(1, 2, 3)
    e_old = lat.energy()
    n = lat.n
    for _ in range(case["steps"]):
        pos = int(rng.uniform() * n) if case["fixture"] != "skyrm" else int(rng.uniform() * 1000)
        trial = lat.gen_rand(rng)
        dE = lat.dE(pos, trial)
        s = lat.spins()
        s[pos] = trial
        lat.set_spins(s)
        e_new = lat.energy()
        assert e_old + dE == pytest.approx(e_new, abs=case["tol"])
        e_old = e_new


def test_dmi_sign_mismatch_is_reproduced():
    """With DMI on, the reference's dE (s_j x D) is not E_new - E_old; the consistent sign
    (D x s_j) is. Neither sign is pinned by the reference's tests (they disable DMI)."""
    off, J, D = O.read_interactions(interactions_file("3d_nn_bloch.dat"), 3, 1.0, 0.7)
    lat = O.Lattice.create(3, 6, False, True, "c", off, J, D, useJ=True, useD=True)
    rng = O.Rng(5, 6, 7)
    lat.all_rand(rng)
    errs = {}
    for sign in (0, 1):
        lat.set_flags(True, True, sign)
        e0 = lat.energy()
        worst = 0.0
        for site in range(0, lat.n, 17):
            t = rng.dir3d()
            dE = lat.dE(site, t)
            s = lat.spins()
            old = s[site].copy()
            s[site] = t
            lat.set_spins(s)
            worst = max(worst, abs(lat.energy() - e0 - dE))
            s[site] = old
            lat.set_spins(s)
        errs[sign] = worst
    assert errs[1] < 1e-9
    assert errs[0] > 1e-3


def test_philox_known_answers():
    """Random123's published Philox4x32-10 vectors."""
    M = 0xFFFFFFFF
    assert list(O.philox([0, 0, 0, 0], [0, 0])) == [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]
    assert list(O.philox([M] * 4, [M, M])) == [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]
    assert list(O.philox([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0])) == \
        [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]


def test_solid_angle_of_an_octant():
    """Three orthonormal spins span one octant (solid angle pi/2); the reference's function
    returns the Berg-Luscher half angle, so the value is pi/4 (Q then divides by 2 pi)."""
    a = O.solid_angle([1, 0, 0], [0, 1, 0], [0, 0, 1])
    assert abs(abs(a) - np.pi / 4) < 1e-12


def test_neighbour_lists_follow_file_order():
    off, J, D = O.read_interactions(interactions_file("3d_nn_bloch.dat"), 3, 1.0, 0.0)
    lat = O.Lattice.create(3, 4, False, True, "c", off, J, D)
    locs = lat.locs()
    nb, ch = lat.neighbours(0)
    assert list(ch) == list(range(6))
    for j, k in zip(nb, ch):
        d = (locs[j] - locs[0] + 4) % 4
        assert np.array_equal(d, (off[k] + 4) % 4)
    # open boundary: corner site has 3 neighbours
    lat2 = O.Lattice.create(3, 4, False, False, "c", off, J, D)
    assert len(lat2.neighbours(0)[0]) == 3


def test_rng_distributions():
    """The restated GSL draws have the reference's distributions (Old/tests/rand_test.hpp)."""
    r = O.Rng(1, 2, 3)
    u = np.array([r.uniform() for _ in range(20000)])
    assert 0 <= u.min() and u.max() < 1 and abs(u.mean() - 0.5) < 0.01
    b = np.array([r.int2() for _ in range(20000)])
    assert set(np.unique(b)) == {0, 1} and abs(b.mean() - 0.5) < 0.02
    d = np.array([r.dir3d() for _ in range(5000)])
    assert np.allclose(np.linalg.norm(d, axis=1), 1, atol=1e-12)
    assert np.all(np.abs(d.mean(0)) < 0.05)
    ln = np.array([r.lognormal(0.0, 0.25) for _ in range(20000)])
    assert abs(np.log(ln).mean()) < 0.01 and abs(np.log(ln).std() - 0.25) < 0.01
