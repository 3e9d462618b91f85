"""Equilibrium statistics of the production checkerboard chains.

* 2-D Ising, L = 32 periodic (the Ising configuration of the benchmark set): energy per site
  against the exact finite-lattice value (Kaufman), |M| per site against Yang's spontaneous
  magnetisation below T_c; 3 sigma, sigma from the scatter of independent chains.
* Heisenberg with DMI and field (2-D interfacial, 3-D bulk): E, |M| and Q of the GPU
  checkerboard chain against the oracle's random-site chain (the reference's algorithm) within
  3 sigma combined, sigma of the oracle series from binning.
"""
import numpy as np
import pytest

from nanomagmc_gb300 import _lib as L
from oracle import oracle as O

from helpers import pair
from onsager import energy_per_site_torus, spontaneous_m
from stats import binned_error

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("T", [2.0, 2.6])
@pytest.mark.parametrize("path", [1, 2])
def test_ising_32_against_exact(T, path):
    nchain, edge = 256, 32
    s, _ = pair("s", edge=edge, ising=True, periodic=True, jfile="2d_nn.dat", T=[T] * nchain, H=0.0, seed=3)
    s.option(L.OPT_SWEEP_PATH, path)
    s.sweep(1500)
    obs = s.sample(2, 500)                 # (samples, chains, obs)
    N = edge * edge
    e = obs[:, :, L.OBS_E].mean(0) / N     # per-chain means
    m = obs[:, :, L.OBS_ABSM].mean(0) / N
    e_mean, e_err = e.mean(), e.std(ddof=1) / np.sqrt(nchain)
    exact = energy_per_site_torus(T, edge)
    assert abs(e_mean - exact) <= 3 * e_err + 1e-12, (e_mean, exact, e_err)
    if T < 2.2:
        m_mean, m_err = m.mean(), m.std(ddof=1) / np.sqrt(nchain)
        # finite-size offset of <|M|> at L = 32, T = 2.0 is far below 2e-3
        assert abs(m_mean - spontaneous_m(T)) <= 3 * m_err + 2e-3, (m_mean, spontaneous_m(T))
    s.close()


def oracle_series(o, T, n_eq, n_samp, seed):
    rng = O.Rng(seed, seed + 1, seed + 2)
    o.set_beta(1.0 / T)
    o.all_rand(rng)
    o.equil(rng, n_eq * o.n)
    E, M, Q = [], [], []
    for _ in range(n_samp):
        o.equil(rng, o.n)
        E.append(o.energy())
        M.append(np.linalg.norm(o.mag()))
        Q.append(o.tcharge().sum())
    return np.array(E), np.array(M), np.array(Q)


CASES = [
    dict(shape="s", edge=8, jfile="2d_nn_interfacial.dat", D=0.5, H=0.2, T=0.6),
    dict(shape="s", edge=8, jfile="2d_nn_interfacial.dat", D=0.5, H=0.2, T=1.5),
    dict(shape="c", edge=4, jfile="3d_nn_bloch.dat", D=0.3, H=0.2, T=1.0),
]


@pytest.mark.parametrize("case", CASES, ids=lambda c: "%s%d-T%.1f" % (c["shape"], c["edge"], c["T"]))
def test_heisenberg_against_reference_chain(case):
    T, H = case["T"], case["H"]
    nchain = 256
    s, ors = pair(case["shape"], edge=case["edge"], periodic=True, jfile=case["jfile"], D=case["D"],
                  T=[T] * nchain, H=H, seed=17)
    s.sweep(2000)
    obs = s.sample(1, 1000)
    N = s.box_sites
    g = {k: obs[:, :, i].mean(0) / N for k, i in (("E", L.OBS_E), ("M", L.OBS_ABSM))}
    g["Q"] = obs[:, :, L.OBS_QTOT].mean(0)
    o = ors[0]
    E, M, Q = oracle_series(o, T, 2000, 40000, 31)
    c = {"E": E / N, "M": M / N, "Q": Q}
    for k in ("E", "M", "Q"):
        gm, ge = g[k].mean(), g[k].std(ddof=1) / np.sqrt(nchain)
        cm, ce = c[k].mean(), binned_error(c[k])
        assert abs(gm - cm) <= 3 * np.hypot(ge, ce) + 1e-9, (k, gm, ge, cm, ce)
    s.close()
