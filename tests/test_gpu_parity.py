"""GPU parity against the oracle, through libnmmc's C ABI.

Tolerances (the bar of the task):
  * Ising: bit-exact (integer energies, magnetisations).
  * Heisenberg observables: per-site terms in FP64 (NMMC_OPT_MEASURE_FP64) agree to 1e-10
    relative; the production FP32 per-site terms with FP64 sums agree to 1e-5 relative (E, M)
    and to 1e-4 absolute per slice for Q.
  * dE probes (FP32 arithmetic of the sweep kernels): |dE - dE_ref| <= 1e-5 * scale, scale =
    sum of the magnitudes of the local-field terms plus 1.
  * Sequential FP64 replay: accept/reject chain and final FP64 spins identical.
  * HBM-streaming and shared-memory resident sweep paths: bit-identical chains.
  * Ising checkerboard chain: bit-identical to the oracle's checkerboard restatement.
"""
import json
import os

import numpy as np
import pytest

from nanomagmc_gb300 import _lib as L
from oracle import oracle as O

from helpers import STENCIL, box_index, load_same, oracle_from_gpu, pair

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
KAT = json.load(open(os.path.join(HERE, "golden", "reference_kat.json")))


def compare_obs(s, o, obs, q, fp64, ising):
    e_ref, m_ref, sm_ref, s4_ref = o.energy(), o.mag(), o.submag(0), o.sub4mag()
    q_ref = o.tcharge()
    n = o.n
    if ising or fp64:
        rtol = 0 if ising else 1e-10
        assert abs(obs[L.OBS_E] - e_ref) <= rtol * max(1, abs(e_ref)), (obs[L.OBS_E], e_ref)
        assert np.allclose(obs[1:4], m_ref, rtol=0, atol=rtol * n + (0 if ising else 1e-12))
        assert np.allclose(obs[5:8], sm_ref, rtol=0, atol=rtol * n + (0 if ising else 1e-12))
        assert np.allclose(obs[9:12], s4_ref, rtol=0, atol=rtol * n + (0 if ising else 1e-12))
        if not ising:
            assert np.allclose(q, q_ref, atol=1e-10, rtol=0, equal_nan=True)
    else:
        assert abs(obs[L.OBS_E] - e_ref) <= 1e-5 * max(1, abs(e_ref)), (obs[L.OBS_E], e_ref)
        for a, b in ((obs[1:4], m_ref), (obs[5:8], sm_ref), (obs[9:12], s4_ref)):
            assert np.all(np.abs(a - b) <= 1e-5 * max(1.0, np.abs(b).max())), (a, b)
        assert np.allclose(q, q_ref, atol=1e-4, rtol=0, equal_nan=True)
    assert obs[L.OBS_ABSM] == pytest.approx(np.linalg.norm(obs[1:4]), rel=1e-15, abs=1e-15)


# ------------------------------------------------------------------------------------------
# the reference's known answers, on the GPU
# ------------------------------------------------------------------------------------------
def kat_context(kind, ising, periodic):
    edge = 30 if kind == "skyrm" else 10
    s, (o,) = pair("c", edge=edge, ising=bool(ising), periodic=bool(periodic), jfile="3d_nn_bloch.dat",
                   J=1.0, D=0.0, T=[1.0])
    off, J, D = O.read_interactions(os.path.join(os.path.dirname(HERE), "data", "Js", "3d_nn_bloch.dat"),
                                    3, 1.0, 0.75 if kind == "skyrm" else 0.0)
    f = O.Lattice.fixture(kind, 3, ising, periodic, off, J, D)
    f.set_flags(useJ=True, useD=False)
    locs = f.locs()
    full = np.zeros((s.box_sites, 3))
    full[box_index(locs, edge)] = f.spins()
    s.set_spins(0, full)
    return s, f


@pytest.mark.parametrize("fp64", [True, False])
@pytest.mark.parametrize("case", KAT["cases"], ids=lambda c: c["src"] + ":" + c["fixture"])
def test_reference_kat_on_gpu(case, fp64):
    s, f = kat_context(case["fixture"], case["ising"], case["periodic"])
    s.option(L.OPT_MEASURE_FP64, int(fp64))
    H = case.get("H", [0, 0, 0])
    s.set_point(0, 1.0, H[0] if case["ising"] else H[2])
    obs, q = s.measure()
    obs, q = obs[0], q[0]
    exact = case["ising"] or fp64
    tol = 0 if case["ising"] else (1e-9 if fp64 else 1e-5 * 3000)
    if "E" in case:
        assert abs(obs[L.OBS_E] - case["E"]) <= tol, obs[L.OBS_E]
    if "M" in case:
        assert np.all(np.abs(obs[1:4] - case["M"]) <= tol)
    if "subM" in case:
        assert np.all(np.abs(obs[5:8] - case["subM"]) <= tol)
    if "sub4M" in case:
        assert np.all(np.abs(obs[9:12] - case["sub4M"]) <= tol)
    if "Q_each" in case:
        assert np.all(np.abs(q - case["Q_each"]) <= case["Q_tol"])
        f.set_H(*H)
        assert np.allclose(q, f.tcharge(), atol=1e-10 if exact else 1e-4)
    s.close()


# ------------------------------------------------------------------------------------------
# observables on random configurations
# ------------------------------------------------------------------------------------------
LATTICES = [
    dict(shape="s", edge=12, ising=False, periodic=True, jfile="2d_nn_interfacial.dat", D=0.5),
    dict(shape="s", edge=12, ising=False, periodic=False, jfile="2d_nn_bloch.dat", D=0.3),
    dict(shape="s", edge=9, ising=False, periodic=False, jfile="2d_nn_interfacial.dat", D=0.5),
    dict(shape="c", edge=8, ising=False, periodic=True, jfile="3d_nn_bloch.dat", D=0.3),
    dict(shape="c", edge=7, ising=False, periodic=False, jfile="3d_nn_bloch.dat", D=0.3),
    dict(shape="w", size=6.0, ising=False, periodic=False, jfile="2d_nn_interfacial.dat", D=0.5),
    dict(shape="x", size=3.0, ising=False, periodic=False, jfile="3d_nn_bloch.dat", D=0.3),
    dict(shape="s", edge=16, ising=True, periodic=True, jfile="2d_nn.dat", D=0.0),
    dict(shape="s", edge=11, ising=True, periodic=False, jfile="2d_nn.dat", D=0.0),
    dict(shape="c", edge=6, ising=True, periodic=True, jfile="3d_nn_bloch.dat", D=0.0),
    dict(shape="w", size=5.0, ising=True, periodic=False, jfile="2d_nn.dat", D=0.0),
    # rows with a multiple of 4 sites per colour: the four-sites-per-thread kernels
    dict(shape="s", edge=16, ising=False, periodic=True, jfile="2d_nn_interfacial.dat", D=0.5),
    dict(shape="s", edge=8, ising=False, periodic=False, jfile="2d_nn_bloch.dat", D=0.3),
    dict(shape="c", edge=8, ising=False, periodic=False, jfile="3d_nn_bloch.dat", D=0.3),
    dict(shape="c", edge=16, ising=False, periodic=True, jfile="3d_nn_bloch.dat", D=0.0),
    # unequal couplings on +x / -x: the general DMI form of the local field
    dict(shape="s", edge=16, ising=False, periodic=True, jfile=os.path.join(HERE, "golden", "2d_asym.dat"), D=1.0),
    dict(shape="s", edge=10, ising=False, periodic=False, jfile=os.path.join(HERE, "golden", "2d_asym.dat"), D=1.0),
]


def lid(d):
    return "%s-%s-%s-%s%s" % (d["shape"], d.get("edge", d.get("size")), "I" if d["ising"] else "H",
                              "P" if d["periodic"] else "O", "-asym" if "asym" in d["jfile"] else "")


@pytest.mark.parametrize("fp64", [True, False])
@pytest.mark.parametrize("lat", LATTICES, ids=lid)
def test_measure_random_configs(lat, fp64):
    rng = np.random.default_rng(3)
    H = 0.3 if not lat["ising"] else 0.25
    s, ors = pair(T=[1.0, 1.5, 0.7], H=[H, 0.0, -H], **lat)
    s.option(L.OPT_MEASURE_FP64, int(fp64))
    for c, o in enumerate(ors):
        load_same(s, o, c, rng)
    obs, q = s.measure()
    for c, o in enumerate(ors):
        compare_obs(s, o, obs[c], q[c], fp64, lat["ising"])
    # a subset of chains, in a different order
    obs2, q2 = s.measure([2, 0])
    assert np.array_equal(obs2[0], obs[2]) and np.array_equal(obs2[1], obs[0])
    # four sites per thread item in the streaming measurement kernel (two by default): the
    # same terms in another FP32 summation order
    assert s.option(L.OPT_MEASURE_SITES) == 2
    s.option(L.OPT_MEASURE_SITES, 4)
    obs3, q3 = s.measure()
    for c, o in enumerate(ors):
        compare_obs(s, o, obs3[c], q3[c], fp64, lat["ising"])
    s.close()


def test_masks_and_counts_match_oracle():
    s, ors = pair("w", size=7.0, T=[1.0] * 4, D=0.5)
    for c, o in enumerate(ors):
        m = s.mask(c)
        ref = np.zeros_like(m)
        ref[box_index(o.locs(), s.edge)] = 1
        assert np.array_equal(m, ref)
        assert s.site_counts(c) == (o.n, o.snum, o.s4num)
    s.close()


# ------------------------------------------------------------------------------------------
# dE probes
# ------------------------------------------------------------------------------------------
@pytest.mark.parametrize("sign", [0, 1])
@pytest.mark.parametrize("lat", LATTICES, ids=lid)
def test_delta_e_matches_oracle(lat, sign):
    rng = np.random.default_rng(5)
    # integer-valued Ising energies (H = 0) must match bit for bit; Heisenberg runs with a field
    H = 0.0 if lat["ising"] else 0.2
    s, (o,) = pair(T=[1.0], H=H, **lat)
    s.option(L.OPT_DMI_SIGN, sign)
    o.set_flags(True, lat["D"] != 0 and not lat["ising"], sign)
    box = load_same(s, o, 0, rng)
    idx = rng.integers(0, o.n, size=min(o.n, 300))
    if lat["ising"]:
        trial = np.zeros((len(idx), 3))
        trial[:, 0] = rng.choice([-1.0, 1.0], size=len(idx))
    else:
        trial = rng.normal(size=(len(idx), 3))
        trial /= np.linalg.norm(trial, axis=1, keepdims=True)
        trial = trial.astype(np.float32).astype(float)
    got = s.delta_e(0, box[idx].astype(np.int32), trial)
    ref = np.array([o.dE(int(i), t) for i, t in zip(idx, trial)])
    scale = 1 + 2 * (abs(0.2) + 2 * s.dim * (1 + lat["D"]) * 2)
    if lat["ising"]:
        assert np.array_equal(got, ref)
    else:
        assert np.all(np.abs(got - ref) <= 1e-5 * scale), np.abs(got - ref).max()
    s.close()


# ------------------------------------------------------------------------------------------
# sequential FP64 replay of the oracle's random-site chain
# ------------------------------------------------------------------------------------------
@pytest.mark.parametrize("sign", [0, 1])
@pytest.mark.parametrize("lat", [LATTICES[0], LATTICES[3], LATTICES[5], LATTICES[7], LATTICES[10]], ids=lid)
def test_debug_replay_reproduces_the_chain(lat, sign):
    rng = np.random.default_rng(9)
    T = 0.9 if not lat["ising"] else 2.3
    s, (o,) = pair(T=[T], H=0.15, **lat)
    s.option(L.OPT_DMI_SIGN, sign)
    o.set_flags(True, lat["D"] != 0 and not lat["ising"], sign)
    o.set_beta(1.0 / T)
    box = load_same(s, o, 0, rng)
    start = o.spins()
    ev = o.equil(O.Rng(4, 5, 6), 20 * o.n, log=True)
    end = o.spins()
    first, acc, fin = s.debug_replay(0, ev)
    assert first == -1
    assert np.array_equal(acc, ev["accepted"].astype(np.uint8))
    assert 0.05 < acc.mean() < 0.98
    assert np.array_equal(fin[box], end)
    # the FP32 copy holds the rounded result
    got = s.get_spins(0)[box]
    assert np.array_equal(got, end.astype(np.float32).astype(float) if not lat["ising"] else end)
    # a log whose decision differs from the replay's is reported at that event
    k = int(np.nonzero(ev["u"] > 0)[0][3])
    ev2 = ev.copy()
    ev2["accepted"][k] ^= 1
    s.set_spins(0, _full(s, box, start))
    first2, _, _ = s.debug_replay(0, ev2, want_final=False)
    assert first2 == k
    s.close()


def _full(s, box, v):
    f = np.zeros((s.box_sites, 3))
    f[box] = v
    return f


# ------------------------------------------------------------------------------------------
# the two sweep paths give the same chain
# ------------------------------------------------------------------------------------------
@pytest.mark.parametrize("lat", LATTICES, ids=lid)
def test_global_and_resident_paths_identical(lat):
    spins = []
    variants = ((1, 0), (1, 1), (2, 0), (1, 2))
    for path, half in variants:
        s, _ = pair(T=[0.7, 1.3, 2.2], H=[0.2, 0.0, 0.1], seed=21, **lat)
        s.option(L.OPT_SWEEP_PATH, path)
        s.option(L.OPT_HALF_KERNEL, half)
        s.sweep(7)
        s.sweep(5, [2, 0])
        spins.append(np.stack([s.get_spins(c) for c in range(3)]))
        s.close()
    for v, sp in zip(variants[1:], spins[1:]):
        assert np.array_equal(spins[0], sp), v


@pytest.mark.parametrize("lat", [LATTICES[0], LATTICES[1], LATTICES[2], LATTICES[5], LATTICES[7], LATTICES[8],
                                 LATTICES[10], LATTICES[15]], ids=lid)
def test_drawn_ahead_resident_identical(lat):
    """The drawn-ahead resident variant (Philox words written by k_predraw) gives the same
    chain bit for bit as the resident kernel drawing its own words: on all chains, on a
    sub-list (the other chains untouched), over a call longer than the word buffer (split
    launches), with the fused observables and in graph sampling. The CTA shape is fixed, so
    that the fused observables are summed in the same FP32 order by both."""
    res = []
    for pre in (1, 2):
        s, _ = pair(T=[0.7, 1.3, 2.2], H=[0.2, 0.0, 0.1], seed=21, **lat)
        s.option(L.OPT_SWEEP_PATH, 2)
        s.option(L.OPT_RESIDENT_BINS, 2)
        s.option(L.OPT_RESIDENT_THREADS, 96)
        s.option(L.OPT_RESIDENT_PREDRAW, pre)
        s.sweep(7)
        assert s.option(L.OPT_RESIDENT_PREDRAW) == pre
        s.sweep(5, [2, 0])
        s.sweep(300, [1])
        o1, q1 = s.sweep_measure(3, accumulate=True)
        o2, q2 = s.sweep_measure(2, [2, 1], accumulate=True)
        h, hq = s.sample(2, 3, with_q=True)
        spins = np.stack([s.get_spins(c) for c in range(3)])
        res.append((spins, o1, q1, o2, q2, h, hq, s.accumulators()))
        s.close()
    for a, b in zip(res[0], res[1]):
        assert np.array_equal(a, b, equal_nan=True)


def test_fixed_resident_shape_overrides_the_tuned_one():
    """Options that fix the resident kernel's width, bins or variant take effect even when an
    automatic choice for the same model is cached."""
    lat = LATTICES[7]
    s, _ = pair(T=[1.0, 2.0], **lat)
    s.option(L.OPT_SWEEP_PATH, 2)
    s.sweep(2)   # automatic shape (cached)
    for th in (64, 96, 512):
        s.option(L.OPT_RESIDENT_THREADS, th)
        s.sweep(2)
        assert s.option(L.OPT_RESIDENT_THREADS) == th
    s.option(L.OPT_RESIDENT_BINS, 1)
    s.sweep(1)
    assert s.option(L.OPT_RESIDENT_BINS) == 1 and s.option(L.OPT_RESIDENT_THREADS) == 512
    for pre in (1, 2, 1):
        s.option(L.OPT_RESIDENT_PREDRAW, pre)
        s.sweep(1)
        assert s.option(L.OPT_RESIDENT_PREDRAW) == pre
    s.close()


# ------------------------------------------------------------------------------------------
# Ising checkerboard chain == the oracle's checkerboard restatement, bit for bit
# ------------------------------------------------------------------------------------------
@pytest.mark.parametrize("lat", [LATTICES[7], LATTICES[8], LATTICES[9], LATTICES[10]], ids=lid)
@pytest.mark.parametrize("path", [1, 2])
def test_ising_chain_bit_exact(lat, path):
    rng = np.random.default_rng(13)
    T = 2.2
    seed = 0x1234567890AB
    s, (o,) = pair(T=[T], H=0.1, seed=seed, **lat)
    s.option(L.OPT_SWEEP_PATH, path)
    o.set_beta(1.0 / T)
    box = load_same(s, o, 0, rng)
    dirs = STENCIL[: 2 * s.dim]
    Jdir = np.ones(len(dirs), np.float32)
    s.sweep(10)
    s.sweep(15)
    o.cb_ising(seed, 0, 0, 25, Jdir, dirs, hx=0.1)
    got = s.get_spins(0)[box]
    ref = o.spins()
    assert np.array_equal(got[:, 0], ref[:, 0]), np.sum(got[:, 0] != ref[:, 0])
    s.close()


# ------------------------------------------------------------------------------------------
# CUDA-graph sampling == sweep_measure calls; sweep_measure == sweep + measure
# ------------------------------------------------------------------------------------------
@pytest.mark.parametrize("lat", [LATTICES[0], LATTICES[3], LATTICES[5], LATTICES[7], LATTICES[14]], ids=lid)
def test_sample_graph_matches_calls(lat):
    a, _ = pair(T=[0.8, 1.6], H=[0.1, 0.3], seed=5, **lat)
    b, _ = pair(T=[0.8, 1.6], H=[0.1, 0.3], seed=5, **lat)
    obs_g, q_g = a.sample(3, 4, with_q=True)
    for k in range(4):
        o, q = b.sweep_measure(3, accumulate=True)
        assert np.array_equal(o, obs_g[k])
        assert np.array_equal(q, q_g[k])
    acc_a, acc_b = a.accumulators(), b.accumulators()
    assert np.array_equal(acc_a, acc_b) and acc_a[0, 0] == 4
    a.close()
    b.close()


def _obs_close(got, ref, N):
    """Observables summed in FP32 in two orders: E and the magnetisations to 2e-6 of the site
    count (relative FP32 rounding of a few thousand terms), Q to 1e-4."""
    tol = 2e-6 * max(N, 1) * 8.0
    assert np.allclose(got[:, :13], ref[:, :13], rtol=0, atol=tol), np.abs(got - ref).max()
    assert np.allclose(got[:, 13], ref[:, 13], rtol=0, atol=1e-4)


@pytest.mark.parametrize("path,sign", [(0, 0), (1, 0), (1, 1)])
@pytest.mark.parametrize("pq", [0, 1])
@pytest.mark.parametrize("lat", LATTICES, ids=lid)
def test_fused_measure_matches_separate(lat, pq, path, sign):
    """nmmc_sweep_measure: same chain as nmmc_sweep; observables as nmmc_measure (which the
    oracle tests pin) up to FP32 summation order, for every lattice, on all chains and on a
    sub-list in another order, with and without wrapped triangles in Q. Path 0 takes the
    resident kernel's fused observables where a lattice fits on chip; path 1 the HBM path,
    whose four-site kernel sums E, M, subM and sub4M in the last colour-1 half-sweep (both DMI
    sign conventions)."""
    T, H = [0.7, 1.3, 2.2], [0.2, 0.0, 0.1]
    a, _ = pair(T=T, H=H, seed=33, **lat)
    b, _ = pair(T=T, H=H, seed=33, **lat)
    for s in (a, b):
        s.option(L.OPT_PERIODIC_Q, pq)
        s.option(L.OPT_SWEEP_PATH, path)
        s.option(L.OPT_DMI_SIGN, sign)
    N = max(a.site_counts(c)[0] for c in range(3))
    for chains in (None, [2, 0], None):
        oa, qa = a.sweep_measure(4, chains, accumulate=True)
        b.sweep(4, chains)
        ob, qb = b.measure(chains, accumulate=True)
        _obs_close(oa, ob, N)
        assert np.allclose(qa, qb, rtol=0, atol=1e-4)
        for c in range(3):
            assert np.array_equal(a.get_spins(c), b.get_spins(c))
    acc_a, acc_b = a.accumulators(), b.accumulators()
    assert np.array_equal(acc_a[:, 0], acc_b[:, 0]) and acc_a[0, 0] == 3 and acc_a[1, 0] == 2
    # a measurement-only call and a zero-sweep call agree with the separate measurement
    o0, _ = a.sweep_measure(0)
    o1, _ = a.measure()
    assert np.array_equal(o0, o1)
    a.close()
    b.close()


CHARGE_LATTICES = [
    # several blocks per slice and row segments (the last one ragged), both boundary kinds
    dict(ising=False, shape="s", edge=256, periodic=True, jfile="2d_nn_interfacial.dat", D=0.5),
    dict(ising=False, shape="s", edge=200, periodic=False, jfile="2d_nn_bloch.dat", D=0.3),
    # one row per segment, 42 segments of 6 strips per block
    dict(ising=False, shape="c", edge=24, periodic=True, jfile="3d_nn_bloch.dat", D=0.3),
    dict(ising=False, shape="c", edge=24, periodic=False, jfile="3d_nn_bloch.dat", D=0.3),
]


@pytest.mark.parametrize("pq", [0, 1])
@pytest.mark.parametrize("lat", CHARGE_LATTICES, ids=lid)
def test_charge_pass_forms_agree(lat, pq):
    """nmmc_sweep_measure on the HBM four-site path: the sliding-row charge pass (strips of
    four sites walking along y) and the measurement kernel's charge-only items sum the same
    triangles (the same angles, another FP32 order): the same chains, E and magnetisations
    bit for bit (both come from the fused half-sweeps), the per-slice charge to 1e-4."""
    T, H = [0.3, 1.0, 2.5], [0.2, 0.0, 0.1]
    runs = []
    for form in (0, 1):
        s, _ = pair(T=T, H=H, seed=21, **lat)
        s.option(L.OPT_SWEEP_PATH, 1)
        s.option(L.OPT_PERIODIC_Q, pq)
        s.option(L.OPT_CHARGE_PASS, form)
        assert s.option(L.OPT_CHARGE_PASS) == form
        out = [s.sweep_measure(3, accumulate=True) for _ in range(2)]
        runs.append((out, [s.get_spins(c) for c in range(3)], s.accumulators()))
        s.close()
    (oa, sa, aa), (ob, sb, ab) = runs
    for (o1, q1), (o2, q2) in zip(oa, ob):
        assert np.array_equal(o1[:, :13], o2[:, :13])
        assert np.allclose(q1, q2, rtol=0, atol=1e-4), np.abs(q1 - q2).max()
        assert np.allclose(o1[:, 13], o2[:, 13], rtol=0, atol=1e-4 * q1.shape[1])
    for c in range(3):
        assert np.array_equal(sa[c], sb[c])
    assert np.array_equal(aa[:, :6], ab[:, :6])


@pytest.mark.parametrize("bins,threads", [(1, 32), (1, 64), (1, 1024), (3, 128), (7, 96), (40, 32)])
def test_fused_measure_multi_chain_bins(bins, threads):
    """Resident bins holding several chains of different sizes (the batched-grain layout):
    every per-slot warp grouping of the fused measurement (more warps than slots, fewer, one
    each) gives the separate measurement's observables and the same chain."""
    rng = np.random.default_rng(3)
    n = 40
    sizes = rng.uniform(3.0, 7.0, n)
    T = list(np.linspace(0.2, 2.0, n))
    kw = dict(shape="w", size=7.0, sizes=sizes, T=T, H=list(np.linspace(0, 0.5, n)), lattices=list(range(n)),
              ising=False, periodic=False, jfile="2d_nn_interfacial.dat", D=0.5, seed=8)
    a, _ = pair(**kw)
    b, _ = pair(**kw)
    for s in (a, b):
        s.option(L.OPT_SWEEP_PATH, 2)
        s.option(L.OPT_RESIDENT_BINS, bins)
        s.option(L.OPT_RESIDENT_THREADS, threads)
    N = max(a.site_counts(c)[0] for c in range(n))
    sub = list(rng.permutation(n)[:17])
    for chains in (None, sub):
        oa, qa = a.sweep_measure(3, chains, accumulate=True)
        b.sweep(3, chains)
        ob, qb = b.measure(chains, accumulate=True)
        _obs_close(oa, ob, N)
        assert np.allclose(qa, qb, rtol=0, atol=1e-4)
    for c in range(n):
        assert np.array_equal(a.get_spins(c), b.get_spins(c))
    a.close()
    b.close()


# ------------------------------------------------------------------------------------------
# summed lattices (add_to_av): running FP64 sums of the listed chains' spins
# ------------------------------------------------------------------------------------------
@pytest.mark.parametrize("lat", [LATTICES[0], LATTICES[3], LATTICES[5], LATTICES[7]], ids=lid)
def test_av_chains_sum_every_accumulating_sample(lat):
    a, _ = pair(T=[0.8, 1.6, 1.1], H=[0.1, 0.3, 0.0], seed=7, **lat)
    b, _ = pair(T=[0.8, 1.6, 1.1], H=[0.1, 0.3, 0.0], seed=7, **lat)
    c, _ = pair(T=[0.8, 1.6, 1.1], H=[0.1, 0.3, 0.0], seed=7, **lat)
    for s in (a, b, c):
        s.set_av_chains([2, 0])
    ref = {0: 0.0, 2: 0.0}
    a.sample(2, 4)                               # graph replay
    for _ in range(4):
        b.sweep_measure(2, accumulate=True)      # direct calls
        c.sweep(2)
        c.measure(accumulate=True)
        c.measure()                              # not accumulating: not summed
        for ch in ref:
            ref[ch] = ref[ch] + c.get_spins(ch)
    for ch in ref:
        assert np.array_equal(c.get_av(ch), ref[ch])
        assert np.array_equal(b.get_av(ch), ref[ch])
        assert np.array_equal(a.get_av(ch), ref[ch])
    with pytest.raises(L.NmmcError):
        a.get_av(1)
    a.set_av_chains([0])                         # resetting zeroes the sum
    assert not np.any(a.get_av(0))
    for s in (a, b, c):
        s.close()


# ------------------------------------------------------------------------------------------
# random start, forks and error codes
# ------------------------------------------------------------------------------------------
def test_random_start_and_fork():
    s, ors = pair("w", size=6.0, T=[1.0, 1.0, 2.0], H=[0.0, 0.0, 0.5], lattices=[0, 0, 1], D=0.5)
    sp = [s.get_spins(c) for c in range(3)]
    m = s.mask(0)
    n = np.linalg.norm(sp[0], axis=1)
    assert np.all(np.abs(n[m == 1] - 1) < 1e-6) and np.all(n[m == 0] == 0)
    assert np.array_equal(s.mask(0), s.mask(1)) and not np.array_equal(s.mask(0), s.mask(2))
    s.fork(2, 0)
    assert np.array_equal(s.get_spins(0), sp[2]) and np.array_equal(s.mask(0), s.mask(2))
    assert s.get_point(0) == s.get_point(2)
    s.sweep(3)   # tables rebuilt after the fork changed chain 0's particle
    s.close()


@pytest.mark.parametrize("kw", [
    dict(shape="x", size=4.0, sizes=[3.0, 4.0, 3.5], ising=False, periodic=False, jfile="3d_nn_bloch.dat", D=0.3),
    dict(shape="w", size=6.0, sizes=[4.0, 6.0, 5.0], ising=True, periodic=False, jfile="2d_nn.dat", D=0.0),
], ids=["x-heisenberg", "w-ising"])
def test_fork_moves_the_filled_site_lists(kw):
    """Masked lattices: the HBM half-sweeps and the measurement run over per-chain lists of
    filled sites. After a fork gives chain 2 the particle of chain 1, the HBM path (lists) and
    the resident path (its own tables) still give the same chains and observables, and the
    sites outside each particle stay empty."""
    res = []
    for path in (1, 2):
        s, _ = pair(T=[0.8, 1.2, 1.6], H=[0.1, 0.0, 0.2], lattices=[0, 1, 2], seed=4, **kw)
        s.option(L.OPT_SWEEP_PATH, path)
        assert not np.array_equal(s.mask(1), s.mask(2))
        s.sweep(3)
        s.fork(1, 2)
        assert np.array_equal(s.mask(2), s.mask(1))
        s.sweep(4)
        s.sweep(2, [2])
        obs, q = s.measure()
        spins = [s.get_spins(c) for c in range(3)]
        for c in range(3):
            assert np.all(spins[c][s.mask(c) == 0] == 0)
        res.append((spins, obs, q))
        s.close()
    for a, b in zip(res[0][0], res[1][0]):
        assert np.array_equal(a, b)
    assert np.array_equal(res[0][1], res[1][1]) and np.array_equal(res[0][2], res[1][2], equal_nan=True)


@pytest.mark.parametrize("lat", [LATTICES[2], LATTICES[4], LATTICES[5], LATTICES[6]], ids=lid)
def test_masked_compact_form_identical(lat):
    """Masked Heisenberg lattices on the HBM path: the compact form (filled sites gathered into
    dense planes with neighbour tables, written back after each call) gives the chains of the
    sweep over the box layout, on all chains, a sub-list, after a fork to another particle, with
    the observables, and in graph sampling."""
    kw = dict(lat)
    kw.update(lattices=[0, 1, 2], sizes=[kw.get("size", 6.0) * f for f in (1.0, 0.8, 0.9)] if "size" in kw else None)
    res = []
    for compact in (0, 1):
        s, _ = pair(T=[0.7, 1.3, 2.2], H=[0.2, 0.0, 0.1], seed=17, **kw)
        s.option(L.OPT_SWEEP_PATH, 1)
        s.option(L.OPT_MASKED_COMPACT, compact)
        s.sweep(5)
        s.sweep(3, [2, 0])
        s.fork(0, 1)
        s.sweep(2)
        o, q = s.sweep_measure(3, accumulate=True)
        h, hq = s.sample(2, 2, with_q=True)
        spins = np.stack([s.get_spins(c) for c in range(3)])
        for c in range(3):
            assert np.all(spins[c][s.mask(c) == 0] == 0)
        res.append((spins, o, q, h, hq, s.accumulators()))
        s.close()
    for a, b in zip(res[0], res[1]):
        assert np.array_equal(a, b, equal_nan=True)


def test_masked_compact_wide_table_identical():
    """A masked lattice whose +-z neighbours lie more than 32767 list entries apart (a cube of
    odd edge 257, every site filled; one colour plane holds 33,025 sites) takes the compact
    form's table of absolute indices: the same chain as the box layout, fingerprinted by the
    FP64 observables with the charge of each of the 257 slices."""
    from nanomagmc_gb300.sampler import Sampler, interactions_file, make_options, read_interactions

    res = []
    for compact in (0, 1):
        opt = make_options("c", edge=257, periodic=False, D=0.3)
        inter = read_interactions(interactions_file("3d_nn_bloch.dat"), 3, 1.0, 0.3)
        s = Sampler(opt, inter, T=[0.9], H=[0.2], seed=6)
        s.option(L.OPT_SWEEP_PATH, 1)
        s.option(L.OPT_MASKED_COMPACT, compact)
        s.sweep(2)
        s.option(L.OPT_MEASURE_FP64, 1)
        res.append(s.measure())
        s.close()
    assert np.array_equal(res[0][0], res[1][0]) and np.array_equal(res[0][1], res[1][1], equal_nan=True)


def test_error_codes():
    from nanomagmc_gb300.sampler import Sampler, interactions_file, make_options, read_interactions
    inter2 = read_interactions(interactions_file("2d_nn.dat"), 2)
    with pytest.raises(L.NmmcError) as e:
        Sampler(make_options("s", edge=8), inter2, T=[1.0, 0.0])
    assert e.value.code == 104
    with pytest.raises(L.NmmcError) as e:
        Sampler(make_options("q", edge=8), inter2, T=[1.0])
    assert e.value.code == 103
    with pytest.raises(L.NmmcError) as e:
        Sampler(make_options("s", edge=9, periodic=True), inter2, T=[1.0])
    assert e.value.code == 301
    # an offset beyond the axis neighbours runs on the multi-colour sweep ...
    inter_far = read_interactions(interactions_file("2d_nn.dat"), 2)
    inter_far.offset[0][0] = 2
    s = Sampler(make_options("s", edge=8), inter_far, T=[1.0])
    assert s.option(L.OPT_COLOURS) > 2
    s.close()
    # ... an offset along an axis the lattice does not have is refused
    inter_z = read_interactions(interactions_file("2d_nn.dat"), 2)
    inter_z.offset[0][2] = 1
    with pytest.raises(L.NmmcError) as e:
        Sampler(make_options("s", edge=8), inter_z, T=[1.0])
    assert e.value.code == 301
    s = Sampler(make_options("s", edge=8), inter2, T=[1.0])
    with pytest.raises(L.NmmcError) as e:
        s.set_point(0, -1.0, 0.0)
    assert e.value.code == 104
    with pytest.raises(L.NmmcError) as e:
        s.sweep(1, [3])
    assert e.value.code == 300
    s.close()
    # a chain listed twice would be updated by two blocks at once (or sampled twice): refused
    s = Sampler(make_options("s", edge=8), inter2, T=[1.0, 2.0])
    for call in (lambda: s.sweep(1, [1, 0, 1]), lambda: s.measure([0, 0]),
                 lambda: s.sweep_measure(1, [1, 1]), lambda: s.sample(1, 2, [0, 1, 0])):
        with pytest.raises(L.NmmcError) as e:
            call()
        assert e.value.code == 300
    s.sweep(1, [1, 0])   # a permutation is fine
    s.close()


# ------------------------------------------------------------------------------------------
# near-antiparallel neighbours: the FP32 solid angle must stay finite and close to FP64
# ------------------------------------------------------------------------------------------
@pytest.mark.parametrize("delta,tol", [(1e-2, 1e-3), (1e-5, None)])
@pytest.mark.parametrize("lat", [LATTICES[0], LATTICES[11], LATTICES[3]], ids=lid)
def test_q_near_antiparallel_pairs(lat, delta, tol):
    """Pairs `delta` rad from antiparallel. At 1e-2 rad the FP32 charge stays within 1e-3 of
    the FP64 reference; at 1e-5 rad FP32 rounds 1 + s.s' to 0 and the reference's division
    by rho would give NaN: the FP32 value must stay finite."""
    rng = np.random.default_rng(8)
    s, (o,) = pair(T=[1.0], H=0.1, **lat)
    locs = o.locs()
    E = s.edge
    v = rng.normal(size=(o.n, 3))
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    lut = {tuple(l): i for i, l in enumerate(locs)}
    for i, l in enumerate(locs):
        if l[0] % 4 == 0 and (l[0] + 1) < E:
            j = lut[(l[0] + 1, l[1], l[2])]
            perp = np.cross(v[i], [0.3, 0.5, 0.8])
            perp /= np.linalg.norm(perp)
            v[j] = -v[i] * np.cos(delta) + perp * np.sin(delta)
    v = v.astype(np.float32).astype(float)
    full = np.zeros((s.box_sites, 3))
    full[box_index(locs, E)] = v
    s.set_spins(0, full)
    o.set_spins(v)
    q_ref = o.tcharge()
    s.option(L.OPT_MEASURE_FP64, 0)
    obs32, q32 = s.measure()
    s.option(L.OPT_MEASURE_FP64, 1)
    _, q64 = s.measure()
    assert np.all(np.isfinite(q32[0])) and np.all(np.isfinite(obs32))
    assert np.allclose(q64[0], q_ref, atol=1e-9)
    if tol is not None:
        assert np.allclose(q32[0], q_ref, atol=tol)
    s.close()


def test_long_high_temperature_run_stays_finite():
    s, _ = pair("c", edge=32, periodic=True, jfile="3d_nn_bloch.dat", D=0.3, T=[2.0, 3.0, 5.0, 20.0], H=0.2)
    obs, q = s.sample(2, 60, with_q=True)
    assert np.all(np.isfinite(obs)) and np.all(np.isfinite(q))
    acc = s.accumulators()
    assert np.all(np.isfinite(acc)) and np.all(acc[:, 0] == 60)
    s.close()


# ------------------------------------------------------------------------------------------
# the ring-pipelined half-sweeps (3-D periodic, edge 128) give the chain of the other kernels,
# for every tile shape and z-segment (including ones that do not divide the edge)
# ------------------------------------------------------------------------------------------
@pytest.mark.parametrize("D,jfile", [(0.3, "3d_nn_bloch.dat"), (0.0, "3d_nn_bloch.dat")])
def test_pipelined_kernel_identical(D, jfile):
    spins = []
    variants = ((0, 0), (3, 0), (4, 0), (5, 0), (3, 7), (4, 128), (5, 1), (6, 0), (7, 0), (6, 5), (7, 128), (6, 1), (8, 0))
    for half, zseg in variants:
        s, _ = pair("c", edge=128, periodic=True, jfile=jfile, D=D, T=[0.4, 1.6], H=[0.2, 0.0], seed=4)
        s.option(L.OPT_SWEEP_PATH, 1)
        s.option(L.OPT_HALF_KERNEL, half)
        s.option(L.OPT_RING_ZSEG, zseg)
        s.sweep(3)
        s.sweep(2, [1])
        s.synchronize()
        spins.append(np.stack([s.get_spins(c) for c in range(2)]))
        s.close()
    for v, sp in zip(variants[1:], spins[1:]):
        assert np.array_equal(spins[0], sp), v


_WAVE_TABLES = {
    # +-axis pairs (J(+a) = J(-a), D(-a) = -D(+a)) with DMI vectors off the axes
    "3d_pairs": [((1, 0, 0), 1.0, (0, 0.4, 0.1)), ((-1, 0, 0), 1.0, (0, -0.4, -0.1)),
                 ((0, 1, 0), 0.9, (0.2, 0, 0.3)), ((0, -1, 0), 0.9, (-0.2, 0, -0.3)),
                 ((0, 0, 1), 1.1, (0.1, 0.2, 0)), ((0, 0, -1), 1.1, (-0.1, -0.2, 0))],
    # per-direction couplings with no pair structure
    "3d_asym": [((1, 0, 0), 1.0, (0.2, 0.3, 0.1)), ((-1, 0, 0), 0.8, (-0.1, 0.4, 0.0)),
                ((0, 1, 0), 1.1, (0.0, 0.0, 0.5)), ((0, -1, 0), 0.9, (0.3, -0.2, 0.0)),
                ((0, 0, 1), 1.0, (0.1, 0.0, 0.0)), ((0, 0, -1), 0.7, (0.0, 0.2, -0.3))],
}

WAVE_LATTICES = [
    dict(edge=16, periodic=True, jfile="3d_nn_bloch.dat", D=0.3),   # one tile; runs end inside a column
    dict(edge=48, periodic=True, jfile="3d_nn_bloch.dat", D=0.3),   # two tiles of 24 rows
    dict(edge=64, periodic=True, jfile="3d_nn_bloch.dat", D=0.0),   # no DMI, two tiles of 32 rows
    dict(edge=24, periodic=False, jfile="3d_nn_bloch.dat", D=0.3),  # open boundaries, 72 threads per tile
    dict(edge=48, periodic=False, jfile="3d_nn_bloch.dat", D=0.3),
    dict(edge=16, periodic=True, jfile="3d_pairs", D=1.0),
    dict(edge=24, periodic=False, jfile="3d_asym", D=1.0),
]


@pytest.mark.parametrize("lat", WAVE_LATTICES, ids=lambda d: "%s-e%d-%s" % (d["jfile"], d["edge"],
                                                                             "per" if d["periodic"] else "open"))
def test_wave_sweeps_identical(lat, tmp_path):
    """Wavefront sweeps (both colours of a sweep in one out-of-place pass) give the chain of the
    two half-sweeps bit for bit: spins, observables (fused into a sample step or not) and
    accumulators, for even and odd sweep counts and chain lists in any order. The launch
    counts show that the wavefront kernel ran."""
    kw = dict(lat)
    if kw["jfile"] in _WAVE_TABLES:
        path = tmp_path / (kw["jfile"] + ".dat")
        with open(path, "w") as f:
            for off, J, D in _WAVE_TABLES[kw["jfile"]]:
                f.write("%d %d %d %.17g %.17g %.17g %.17g\n" % (*off, J, *D))
        kw["jfile"] = str(path)
    res = []
    for wave in (1, 0):
        s, _ = pair("c", T=[0.5, 1.1, 2.0], H=[0.2, 0.0, 0.5], seed=5, **kw)
        s.option(L.OPT_SWEEP_PATH, 1)
        s.option(L.OPT_WAVE, wave)
        s.option(L.OPT_TIMING, 1)
        s.timing()
        s.sweep(4)
        _, launches, _ = s.timing()
        assert launches == (4 if wave else 8)
        s.sweep(3, [2, 0])
        s.sweep(1)
        o1, q1 = s.sweep_measure(5, accumulate=True)
        o2, q2 = s.sweep_measure(2, [1], accumulate=True)
        s.sweep(6, [1, 2])
        spins = np.stack([s.get_spins(c) for c in range(3)])
        res.append((spins, o1, q1, o2, q2, s.accumulators()))
        s.close()
    for a, b, name in zip(res[0], res[1], ("spins", "obs", "q", "obs list", "q list", "accumulators")):
        assert np.array_equal(a, b), name


PF_LATTICES = WAVE_LATTICES + [
    dict(edge=16, periodic=True, jfile="2d_nn_interfacial.dat", D=0.5, shape="s"),
    dict(edge=24, periodic=False, jfile="2d_nn_interfacial.dat", D=0.5, shape="s"),
]


@pytest.mark.parametrize("lat", PF_LATTICES, ids=lambda d: "%s-%s-e%d-%s" % (d.get("shape", "c"), d["jfile"], d["edge"],
                                                                               "per" if d["periodic"] else "open"))
def test_prefetching_half_sweep_identical(lat, tmp_path):
    """The four-site half-sweep with the next quad prefetched into shared memory
    (NMMC_OPT_HALF_KERNEL 8) gives the chain of the four-site kernel bit for bit, over 2-D and
    3-D, periodic and open lattices, every DMI structure and chain lists in any order."""
    kw = dict(lat)
    shape = kw.pop("shape", "c")
    if kw["jfile"] in _WAVE_TABLES:
        path = tmp_path / (kw["jfile"] + ".dat")
        with open(path, "w") as f:
            for off, J, D in _WAVE_TABLES[kw["jfile"]]:
                f.write("%d %d %d %.17g %.17g %.17g %.17g\n" % (*off, J, *D))
        kw["jfile"] = str(path)
    res = []
    for half in (8, 0):
        s, _ = pair(shape, T=[0.5, 1.1, 2.0], H=[0.2, 0.0, 0.5], seed=6, **kw)
        s.option(L.OPT_SWEEP_PATH, 1)
        s.option(L.OPT_HALF_KERNEL, half)
        s.sweep(3)
        s.sweep(2, [2, 0])
        o, q = s.sweep_measure(3, accumulate=True)
        res.append((np.stack([s.get_spins(c) for c in range(3)]), o, q))
        s.close()
    for a, b in zip(res[0], res[1]):
        assert np.array_equal(a, b)


STENCIL_LATTICES = [
    dict(shape="s", edge=16, periodic=True, jfile="2d_nn_interfacial.dat", D=0.5),
    dict(shape="s", edge=64, periodic=True, jfile="2d_nn_interfacial.dat", D=0.5),   # the C2 lattice
    dict(shape="s", edge=24, periodic=False, jfile="2d_nn_bloch.dat", D=0.3),
    dict(shape="s", edge=32, periodic=True, jfile="2d_nn_interfacial.dat", D=0.0),
    dict(shape="s", edge=16, periodic=True, jfile=os.path.join(HERE, "golden", "2d_asym.dat"), D=1.0),
    dict(shape="s", edge=16, periodic=False, jfile=os.path.join(HERE, "golden", "2d_asym.dat"), D=1.0),
]


@pytest.mark.parametrize("lat", STENCIL_LATTICES, ids=lambda d: "e%d-%s-%s" % (d["edge"], os.path.basename(d["jfile"]),
                                                                                "per" if d["periodic"] else "open"))
def test_stencil_resident_identical(lat):
    """The stencil resident kernel (whole unmasked 2-D chains in shared memory, four sites per
    thread item; NMMC_OPT_RESIDENT_STENCIL 2) gives the record kernel's chain bit for bit:
    sweeps of every chain and of lists in another order, fused sample steps and the sampling
    graph; its fused observables agree with the record kernel's to FP32 summation order."""
    T, H = [0.4, 0.9, 1.6, 2.5, 0.7], [0.2, 0.0, 0.5, 0.1, 0.3]
    res = []
    for st in (2, 1):
        s, _ = pair(T=T, H=H, seed=21, **lat)
        s.option(L.OPT_SWEEP_PATH, 2)
        s.option(L.OPT_RESIDENT_STENCIL, st)
        s.sweep(5)
        assert s.option(L.OPT_RESIDENT_STENCIL) == st   # the kernel the shape resolved to
        s.sweep(3, [3, 0, 4])
        o1, q1 = s.sweep_measure(4, accumulate=True)
        o2, q2 = s.sweep_measure(2, [4, 1], accumulate=True)
        h = s.sample(3, 2, [2, 0], with_q=True)
        res.append(dict(spins=np.stack([s.get_spins(c) for c in range(len(T))]), obs=(o1, o2, h[0]),
                        q=(q1, q2, h[1]), acc=s.accumulators()))
        s.close()
    a, b = res
    assert np.array_equal(a["spins"], b["spins"])
    N = lat["edge"] ** 2
    for oa, ob in zip(a["obs"], b["obs"]):
        _obs_close(oa.reshape(-1, L.OBS_N), ob.reshape(-1, L.OBS_N), N)
    for qa, qb in zip(a["q"], b["q"]):
        assert np.allclose(qa, qb, rtol=0, atol=1e-4)
    assert np.array_equal(a["acc"][:, 0], b["acc"][:, 0])


@pytest.mark.parametrize("half", [3, 6])
def test_pipelined_wait_gives_up_and_context_recovers(half):
    """A bounded wait that runs out: with the poll limit at 0 every wait of the ring kernel
    gives up at once, the kernel lets the copies it issued land and returns, and
    nmmc_synchronize reports NMMC_ERR_TIMEOUT. The context then sweeps on: given the spins of
    a context that made the same sweep with the four-site kernel, it produces that context's
    chain bit for bit."""
    mk = lambda: pair("c", edge=128, periodic=True, jfile="3d_nn_bloch.dat", D=0.3, T=[0.6, 1.5], H=0.2,
                      seed=12)[0]
    a, b = mk(), mk()
    a.option(L.OPT_SWEEP_PATH, 1)
    b.option(L.OPT_SWEEP_PATH, 1)
    a.option(L.OPT_HALF_KERNEL, half)
    start = np.stack([a.get_spins(c) for c in range(2)])
    a.option(L.OPT_WAIT_LIMIT, 0)
    a.sweep(1)
    with pytest.raises(L.NmmcError) as e:
        a.synchronize()
    assert e.value.code == L.ERR_TIMEOUT
    assert np.array_equal(np.stack([a.get_spins(c) for c in range(2)]), start)   # no site was updated
    a.synchronize()                     # the error word was cleared
    a.option(L.OPT_WAIT_LIMIT, 1 << 26)
    b.sweep(1)                          # both contexts' sweep counters now stand at one sweep
    for c in range(2):
        a.set_spins(c, b.get_spins(c))
    a.sweep(3)
    b.sweep(3)
    a.synchronize()
    for c in range(2):
        assert np.array_equal(a.get_spins(c), b.get_spins(c))
    a.close()
    b.close()


# ------------------------------------------------------------------------------------------
# degenerate inputs: empty chain lists, zero sweeps, the smallest lattices, near-empty grains
# ------------------------------------------------------------------------------------------
SMALL = [
    dict(shape="s", edge=2, ising=False, periodic=True, jfile="2d_nn_interfacial.dat", D=0.5),
    dict(shape="s", edge=3, ising=False, periodic=False, jfile="2d_nn_bloch.dat", D=0.3),
    dict(shape="c", edge=2, ising=False, periodic=True, jfile="3d_nn_bloch.dat", D=0.3),
    dict(shape="s", edge=2, ising=True, periodic=True, jfile="2d_nn.dat", D=0.0),
    dict(shape="w", size=0.6, ising=False, periodic=False, jfile="2d_nn_interfacial.dat", D=0.5),
]


@pytest.mark.parametrize("lat", SMALL, ids=lid)
def test_smallest_lattices_match_oracle(lat):
    """Edge 2 (periodic: both x neighbours are the same site, counted twice as in the
    reference's neighbour lists), edge 3 open, and a grain of a few sites: site counts,
    observables and dE against the oracle, and the same chain on both sweep paths."""
    rng = np.random.default_rng(21)
    s, ors = pair(T=[0.9, 1.7], H=0.2, seed=5, **lat)
    for c, o in enumerate(ors):
        assert s.site_counts(c)[0] == o.n
        if o.n:
            load_same(s, o, c, rng)
    obs, q = s.measure()
    for c, o in enumerate(ors):
        compare_obs(s, o, obs[c], q[c], False, lat["ising"])
    o = ors[0]
    if o.n:
        o.set_flags(True, lat["D"] != 0 and not lat["ising"], 0)
        box = box_index(o.locs(), s.edge)
        trial = np.zeros((o.n, 3))
        if lat["ising"]:
            trial[:, 0] = -o.spins()[:, 0]
        else:
            trial = rng.normal(size=(o.n, 3))
            trial /= np.linalg.norm(trial, axis=1, keepdims=True)
            trial = trial.astype(np.float32).astype(float)
        got = s.delta_e(0, box.astype(np.int32), trial)
        ref = np.array([o.dE(i, t) for i, t in enumerate(trial)])
        assert np.all(np.abs(got - ref) <= 1e-5 * (1 + np.abs(ref))), np.abs(got - ref).max()
    s.close()
    spins = []
    for path in (1, 2):
        s, _ = pair(T=[0.9, 1.7], H=0.2, seed=5, **lat)
        s.option(L.OPT_SWEEP_PATH, path)
        s.sweep(6)
        spins.append(np.stack([s.get_spins(c) for c in range(2)]))
        s.close()
    assert np.array_equal(spins[0], spins[1])
    assert np.all(np.isfinite(spins[0]))


def test_empty_lists_and_zero_sweeps_are_no_ops():
    s, _ = pair("c", edge=8, periodic=True, jfile="3d_nn_bloch.dat", D=0.3, T=[0.8, 1.6], H=0.1, seed=2)
    before = np.stack([s.get_spins(c) for c in range(2)])
    s.sweep(0)
    s.sweep(5, [])
    obs, q = s.sweep_measure(0, [])
    assert obs.shape == (0, L.OBS_N)
    obs, q = s.measure([])
    assert obs.shape == (0, L.OBS_N)
    assert s.sample(2, 3, []).shape == (3, 0, L.OBS_N)
    assert s.sample(2, 0).shape == (0, 2, L.OBS_N)
    after = np.stack([s.get_spins(c) for c in range(2)])
    assert np.array_equal(before, after)
    o0, _ = s.measure()
    o1, _ = s.sweep_measure(0)   # zero sweeps, then the observables of the unchanged state
    assert np.array_equal(o0, o1)
    s.close()


# ------------------------------------------------------------------------------------------
# record order of an interaction file: the shipped 3d_nn_bloch.dat lists its six records
# z, y, x as the reference's file does (Old/Js/3d_nn_bloch.dat:1-6); the oracle sums the
# neighbours in file order (Old/lib/field_type.cpp:49-71,104-141), the library maps the
# records onto its stencil. Both orders must give the oracle's dE and E for that order and
# the same GPU chain.
# ------------------------------------------------------------------------------------------
def test_interaction_record_order(tmp_path):
    from nanomagmc_gb300.sampler import interactions_file
    rows = [r for r in open(interactions_file("3d_nn_bloch.dat")).read().splitlines() if r.strip()]
    assert [tuple(int(v) for v in r.split()[:3]) for r in rows] == \
        [(0, 0, 1), (0, 0, -1), (0, 1, 0), (0, -1, 0), (1, 0, 0), (-1, 0, 0)]
    xyz = tmp_path / "3d_nn_bloch_xyz.dat"
    xyz.write_text("\n".join(rows[4:6] + rows[2:4] + rows[0:2]) + "\n")
    chains, energies = [], []
    for path in (interactions_file("3d_nn_bloch.dat"), str(xyz)):
        rng = np.random.default_rng(8)
        s, ors = pair("c", edge=8, periodic=True, jfile=path, D=0.3, T=[0.7, 1.4], H=0.2, seed=3)
        for c, o in enumerate(ors):
            box = load_same(s, o, c, rng)
        # dE probes (FP32 sweep arithmetic) and E, M, Q in both measurement modes
        idx = rng.integers(0, ors[0].n, size=200)
        trial = rng.normal(size=(200, 3))
        trial = (trial / np.linalg.norm(trial, axis=1, keepdims=True)).astype(np.float32).astype(float)
        got = s.delta_e(0, box[idx].astype(np.int32), trial)
        ref = np.array([ors[0].dE(int(i), t) for i, t in zip(idx, trial)])
        assert np.all(np.abs(got - ref) <= 1e-5 * (1 + 2 * (0.2 + 6 * 1.3 * 2)))
        for fp64 in (True, False):
            s.option(L.OPT_MEASURE_FP64, int(fp64))
            obs, q = s.measure()
            for c, o in enumerate(ors):
                compare_obs(s, o, obs[c], q[c], fp64, False)
        energies.append([o.energy() for o in ors])
        s.sweep(6)
        chains.append(np.stack([s.get_spins(c) for c in range(2)]))
        s.close()
    assert np.array_equal(chains[0], chains[1])
    # the two summation orders differ only by FP64 rounding
    assert np.allclose(energies[0], energies[1], rtol=1e-13, atol=0)
