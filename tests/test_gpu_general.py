"""General interaction tables on the GPU (multi-colour gather sweep) against the oracle.

The oracle builds its neighbour lists from the same records in file order, exactly as the
reference's set_neigh does, so every check here is against the reference's arithmetic:
  * dE probes (FP32 field of the sweep): within 1e-5 of the local-field scale; Ising exact;
  * observables on random configurations: FP64 per-site mode to 1e-10, FP32 mode to 1e-5;
  * the FP64 sequential replay reproduces the oracle's random-site chain exactly;
  * the Ising colour-class chain equals the oracle's restatement of that order bit for bit;
  * Heisenberg equilibrium E, |M|, Q agree with the oracle's random-site chain within 3 sigma.
"""
import ctypes as C

import numpy as np
import pytest

from nanomagmc_gb300 import _lib as L
from oracle import oracle as O

from general_tables import write_table
from helpers import load_same, pair
from stats import binned_error
from test_gpu_stats import oracle_series

pytestmark = pytest.mark.gpu

CASES = [
    dict(shape="s", edge=12, ising=False, periodic=True, table="2d_j1j2", D=0.5),
    dict(shape="s", edge=10, ising=False, periodic=False, table="2d_j1j3", D=0.5),
    dict(shape="w", size=6.0, ising=False, periodic=False, table="2d_j1j2", D=0.5),
    dict(shape="c", edge=8, ising=False, periodic=True, table="3d_j1j2", D=0.3),
    dict(shape="c", edge=7, ising=False, periodic=False, table="3d_j1j2", D=0.3),
    dict(shape="s", edge=12, ising=True, periodic=True, table="2d_j1j2", D=0.0),
    dict(shape="w", size=5.0, ising=True, periodic=False, table="2d_j1j2", D=0.0),
    dict(shape="s", edge=20, ising=False, periodic=True, table="2d_long", D=0.0),
    dict(shape="s", edge=16, ising=False, periodic=False, table="2d_long", D=0.0),
]


def cid(c):
    return "%s%s-%s-%s-%s" % (c["shape"], c.get("edge", c.get("size")), "I" if c["ising"] else "H",
                              "P" if c["periodic"] else "O", c["table"])


@pytest.fixture(scope="module")
def tables(tmp_path_factory):
    d = str(tmp_path_factory.mktemp("js"))
    return {n: write_table(d, n) for n in ("2d_j1j2", "2d_j1j3", "3d_j1j2", "2d_long")}


def make(tables, case, **kw):
    c = dict(case)
    c["jfile"] = tables[c.pop("table")]
    c.update(kw)
    return pair(**c)


def field_scale(tables, case):
    """1 + twice the largest possible local field: |H| + sum over records of |J| + |D|."""
    rec = np.loadtxt(tables[case["table"]])
    dim = 3 if case["shape"] in "cx" else 2
    J, D = np.abs(rec[:, dim]), np.abs(rec[:, dim + 1:]).sum(1) * case["D"]
    return 1 + 2 * (0.3 + J.sum() + D.sum())


def compare_general(o, obs, q, fp64, ising):
    e_ref = o.energy()
    tol = 1e-10 if fp64 else 1e-5
    assert abs(obs[L.OBS_E] - e_ref) <= tol * max(1, abs(e_ref)), (obs[L.OBS_E], e_ref)
    for a, b in ((obs[1:4], o.mag()), (obs[5:8], o.submag(0)), (obs[9:12], o.sub4mag())):
        if ising:   # sums of +-1: exact in either mode
            assert np.array_equal(a, b[:3])
        else:
            assert np.all(np.abs(a - b[:3]) <= tol * max(1.0, np.abs(b).max())), (a, b)
    if not ising:
        assert np.allclose(q, o.tcharge(), atol=1e-10 if fp64 else 1e-4, rtol=0)


@pytest.mark.parametrize("sign", [0, 1])
@pytest.mark.parametrize("case", CASES, ids=cid)
def test_general_delta_e_matches_oracle(tables, case, sign):
    rng = np.random.default_rng(5)
    H = 0.0 if case["ising"] else 0.2
    s, (o,) = make(tables, case, T=[1.0], H=H)
    assert s.option(L.OPT_COLOURS) > 2
    s.option(L.OPT_DMI_SIGN, sign)
    o.set_flags(True, case["D"] != 0 and not case["ising"], sign)
    box = load_same(s, o, 0, rng)
    idx = rng.integers(0, o.n, size=min(o.n, 300))
    if case["ising"]:
        trial = np.zeros((len(idx), 3))
        trial[:, 0] = rng.choice([-1.0, 1.0], size=len(idx))
    else:
        trial = rng.normal(size=(len(idx), 3))
        trial /= np.linalg.norm(trial, axis=1, keepdims=True)
        trial = trial.astype(np.float32).astype(float)
    got = s.delta_e(0, box[idx].astype(np.int32), trial)
    ref = np.array([o.dE(int(i), t) for i, t in zip(idx, trial)])
    if case["ising"]:
        # J2 = -0.3 is not a small integer: FP32 field vs FP64, a few ulps
        assert np.all(np.abs(got - ref) <= 1e-5 * (1 + np.abs(ref))), np.abs(got - ref).max()
    else:
        assert np.all(np.abs(got - ref) <= 1e-5 * field_scale(tables, case)), np.abs(got - ref).max()
    s.close()


@pytest.mark.parametrize("fp64", [True, False])
@pytest.mark.parametrize("case", CASES, ids=cid)
def test_general_measure_matches_oracle(tables, case, fp64):
    rng = np.random.default_rng(3)
    H = 0.3 if not case["ising"] else 0.25
    s, ors = make(tables, case, T=[1.0, 1.5, 0.7], H=[H, 0.0, -H])
    s.option(L.OPT_MEASURE_FP64, int(fp64))
    for c, o in enumerate(ors):
        load_same(s, o, c, rng)
    obs, q = s.measure()
    for c, o in enumerate(ors):
        # Ising energies with J2 = -0.3 are not integers: FP32 terms are compared to 1e-5
        compare_general(o, obs[c], q[c], fp64, case["ising"])
    s.close()


@pytest.mark.parametrize("sign", [0, 1])
@pytest.mark.parametrize("case", [CASES[0], CASES[2], CASES[3], CASES[5], CASES[7]], ids=cid)
def test_general_replay_reproduces_the_chain(tables, case, sign):
    rng = np.random.default_rng(9)
    T = 0.9 if not case["ising"] else 2.0
    s, (o,) = make(tables, case, T=[T], H=0.15)
    s.option(L.OPT_DMI_SIGN, sign)
    o.set_flags(True, case["D"] != 0 and not case["ising"], sign)
    o.set_beta(1.0 / T)
    box = load_same(s, o, 0, rng)
    ev = o.equil(O.Rng(4, 5, 6), 20 * o.n, log=True)
    end = o.spins()
    first, acc, fin = s.debug_replay(0, ev)
    assert first == -1
    assert np.array_equal(acc, ev["accepted"].astype(np.uint8))
    assert 0.05 < acc.mean() < 0.98
    assert np.array_equal(fin[box], end)
    s.close()


def _colouring(s, case, tables):
    from nanomagmc_gb300.sampler import read_interactions
    dim = 3 if case["shape"] in "cx" else 2
    inter = read_interactions(tables[case["table"]], dim, 1.0, case["D"])
    out = (C.c_int * 5)()
    L.check(L.load().nmmc_colouring(dim, s.edge, int(case["periodic"]), int(case["ising"]), C.byref(inter), out))
    return list(out)


@pytest.mark.parametrize("case", [CASES[5], CASES[6]], ids=cid)
def test_general_ising_chain_bit_exact(tables, case):
    rng = np.random.default_rng(13)
    T = 2.0
    seed = 0x1234567890AB
    s, (o,) = make(tables, case, T=[T], H=0.1, seed=seed)
    o.set_beta(1.0 / T)
    o.set_H(0.1, 0, 0)
    box = load_same(s, o, 0, rng)
    col = _colouring(s, case, tables)
    assert col[1] == s.option(L.OPT_COLOURS)
    s.sweep(10)
    s.sweep(15)
    o.colour_ising(seed, 0, 0, 25, col, hx=float(np.float32(0.1)))
    got = s.get_spins(0)[box]
    ref = o.spins()
    assert np.array_equal(got[:, 0], ref[:, 0]), np.sum(got[:, 0] != ref[:, 0])
    s.close()


EQ_CASES = [
    dict(shape="s", edge=8, ising=False, periodic=True, table="2d_j1j2", D=0.5, H=0.2, T=0.8),
    dict(shape="s", edge=12, ising=False, periodic=True, table="2d_j1j3", D=0.5, H=0.2, T=1.2),
    dict(shape="c", edge=4, ising=False, periodic=True, table="3d_j1j2", D=0.3, H=0.2, T=1.0),
]


@pytest.mark.parametrize("case", EQ_CASES, ids=lambda c: "%s%d-%s-T%.1f" % (c["shape"], c["edge"], c["table"], c["T"]))
def test_general_heisenberg_equilibrium_against_reference_chain(tables, case):
    T, H = case["T"], case["H"]
    nchain = 256
    c = {k: v for k, v in case.items() if k not in ("H", "T")}
    s, ors = make(tables, c, T=[T] * nchain, H=H, seed=17)
    s.sweep(2000)
    obs = s.sample(1, 1000)
    N = s.box_sites
    g = {k: obs[:, :, i].mean(0) / N for k, i in (("E", L.OBS_E), ("M", L.OBS_ABSM))}
    g["Q"] = obs[:, :, L.OBS_QTOT].mean(0)
    E, M, Q = oracle_series(ors[0], T, 2000, 40000, 31)
    r = {"E": E / N, "M": M / N, "Q": Q}
    for k in ("E", "M", "Q"):
        gm, ge = g[k].mean(), g[k].std(ddof=1) / np.sqrt(nchain)
        cm, ce = r[k].mean(), binned_error(r[k])
        assert abs(gm - cm) <= 3 * np.hypot(ge, ce) + 1e-9, (k, gm, ge, cm, ce)
    s.close()


@pytest.mark.parametrize("case", [CASES[0], CASES[3], CASES[6]], ids=cid)
def test_general_sample_graph_and_fused_call_match(tables, case):
    a, _ = make(tables, case, T=[0.8, 1.6], H=[0.1, 0.3], seed=5)
    b, _ = make(tables, case, T=[0.8, 1.6], H=[0.1, 0.3], seed=5)
    c, _ = make(tables, case, T=[0.8, 1.6], H=[0.1, 0.3], seed=5)
    obs_g, q_g = a.sample(3, 4, with_q=True)
    for k in range(4):
        o, q = b.sweep_measure(3, accumulate=True)
        assert np.array_equal(o, obs_g[k]) and np.array_equal(q, q_g[k])
        c.sweep(3)
        o2, q2 = c.measure(accumulate=True)
        assert np.array_equal(o2, o) and np.array_equal(q2, q)
    assert np.array_equal(a.accumulators(), b.accumulators())
    for x in (a, b, c):
        x.close()
