"""Equilibrium parity of the production checkerboard chains against the oracle's random-site
chain (the reference's algorithm, Old/lib/state.cpp:171-203) on the lattices and Hamiltonians
of every benchmark configuration's path:

  * C2 physics: 2-D L = 64 periodic, interfacial DMI 0.5, a skyrmion-phase point (T 0.5,
    B 0.15, Q about 20) and a paramagnetic one (T 1.2, B 0.2); resident and HBM paths;
  * C3: one open Weibull grain of about 1.4k sites (scale radius 20, box 90), on the resident
    kernel and on the HBM path both in the compact form and over the box layout's lists;
  * the C4 Hamiltonian (3-D cubic, bulk DMI 0.3, B_z 0.2) at L = 16 for T = 0.8 and 1.6 (HBM
    four-site kernel and resident) and at L = 12 (HBM one-site kernel);
  * a 3-D Weibull sphere (resident, HBM compact, HBM box layout);
  * 2-D Ising L = 32 with open boundaries at T = 2.0 and 2.3 (resident and HBM).

The oracle side is tests/golden/equilibrium_oracle.json, made by make_equilibrium.py beside it
(32 independent FP64 oracle chains per case). The GPU side: 256 chains at the case's point,
the same number of equilibration sweeps, then one sample per sweep accumulated on the
device. E/N, |M|/N and Q must agree within 3 sigma, sigma = hypot(GPU error, oracle error),
each the standard error of independent chain means; the sigmas used are printed.
"""
import json
import os

import numpy as np
import pytest

from nanomagmc_gb300 import _lib as L
from nanomagmc_gb300.sampler import Sampler, interactions_file, make_options, read_interactions

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
FIX = json.load(open(os.path.join(HERE, "golden", "equilibrium_oracle.json")))

NCHAIN = 256
SAMPLES = 2000

# (case, sweep path, masked compact option or None)
RUNS = [
    ("c2_skyrmion", 2, None), ("c2_skyrmion", 1, None),
    ("c2_para", 2, None), ("c2_para", 1, None),
    ("c3_grain", 2, None), ("c3_grain", 1, 0), ("c3_grain", 1, 1),
    ("c4h_T08", 1, None), ("c4h_T08", 2, None),
    ("c4h_T16", 1, None), ("c4h_T16", 2, None),
    ("c4h_L12", 1, None),
    ("x_sphere", 2, None), ("x_sphere", 1, 0), ("x_sphere", 1, 1),
    ("ising_open_T23", 2, None), ("ising_open_T23", 1, None),
    ("ising_open_T20", 2, None), ("ising_open_T20", 1, None),
]


def rid(r):
    name, path, compact = r
    return "%s-%s%s" % (name, {1: "hbm", 2: "resident"}[path], "" if compact is None else "-compact%d" % compact)


def sampler_for(f, seed=11):
    dim = 3 if f["shape"] in "cx" else 2
    opt = make_options(f["shape"], edge=f["edge"], size=f.get("size"), ising=f["ising"], periodic=f["periodic"],
                       J=1.0, D=f["D"], weibull=3.0)
    inter = read_interactions(interactions_file(f["jfile"]), dim, 1.0, f["D"])
    # every chain on particle 0 of the seed the oracle's mask used
    return Sampler(opt, inter, T=[f["T"]] * NCHAIN, H=f["H"], sizes=f.get("size"), lattices=0, seed=seed)


@pytest.mark.parametrize("run", RUNS, ids=rid)
def test_checkerboard_chain_matches_oracle_chain(run):
    name, path, compact = run
    f = FIX[name]
    s = sampler_for(f)
    s.option(L.OPT_SWEEP_PATH, path)
    if compact is not None:
        s.option(L.OPT_MASKED_COMPACT, compact)
    N = s.site_counts(0)[0]
    assert N == f["sites"]
    s.sweep(f["eq"])
    s.reset_accumulators()
    lib = L.load()
    for _ in range(SAMPLES):
        L.check(lib.nmmc_sweep_measure(s.h, None, NCHAIN, 1, None, None, 1))
    acc = s.accumulators()
    s.close()
    assert np.all(acc[:, 0] == SAMPLES)
    g = {"E": acc[:, 1] / SAMPLES / N, "M": acc[:, 3] / SAMPLES / N, "Q": acc[:, 6] / SAMPLES}
    report = []
    for k in ("E", "M", "Q"):
        if k not in f:
            continue
        gm, ge = g[k].mean(), g[k].std(ddof=1) / np.sqrt(NCHAIN)
        om, oe = f[k]["mean"], f[k]["err"]
        sigma = np.hypot(ge, oe)
        report.append("%s gpu %.5f+-%.5f oracle %.5f+-%.5f dev %.2f sigma" % (k, gm, ge, om, oe, (gm - om) / sigma))
        assert abs(gm - om) <= 3 * sigma, (name, path, compact, report[-1])
    print("%s: %s" % (rid(run), "; ".join(report)))
