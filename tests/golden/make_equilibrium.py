"""Generates tests/golden/equilibrium_oracle.json: equilibrium E, |M| and Q of the oracle's
random-site Metropolis chain (the reference's algorithm, Old/lib/state.cpp:171-203, FP64)
for the configurations the GPU chain-parity tests compare against.

For each case, `chains` independent oracle chains start from random spins
(Old/lib/field_type.cpp:197-204), run `eq` sweeps of N random-site attempts, then record
E/N, |M|/N and the total topological charge Q after each of `samples` further sweeps. The
fixture keeps, per observable, the mean over chains of the per-chain means and its standard
error from the scatter of those chain means (independent chains, each far longer than its
autocorrelation time), plus the per-chain binning error for reference.

Run from the repository root (several minutes on 8 cores):
    python tests/golden/make_equilibrium.py [--only NAME] [--quick]
"""
from __future__ import annotations

import argparse
import json
import multiprocessing as mp
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

OUT = os.path.join(HERE, "equilibrium_oracle.json")

# name: lattice and point. size = Weibull scale radius (LATTSHAPE w / x); the box edge of a
# Weibull particle is 3 * size as the reference derives it (Old/lib/param_read.cpp:55-70)
CASES = {
    # 2-D Heisenberg, interfacial DMI D = 0.5, L = 64 periodic (the C2 lattice): a skyrmion
    # phase point (Q about 20) and a paramagnetic one
    "c2_skyrmion": dict(shape="s", edge=64, periodic=True, ising=False, jfile="2d_nn_interfacial.dat", D=0.5,
                        T=0.5, H=0.15, chains=32, eq=6000, samples=20000),
    "c2_para": dict(shape="s", edge=64, periodic=True, ising=False, jfile="2d_nn_interfacial.dat", D=0.5,
                    T=1.2, H=0.2, chains=32, eq=3000, samples=15000),
    # one open Weibull-masked grain of the C3 ensemble (scale radius 20 in a box of edge 90,
    # about 1.4k filled sites), Heisenberg, interfacial DMI 0.5
    "c3_grain": dict(shape="w", edge=90, size=20.0, periodic=False, ising=False, jfile="2d_nn_interfacial.dat",
                     D=0.5, T=0.8, H=0.5, chains=32, eq=3000, samples=20000),
    # the C4 Hamiltonian (3-D cubic, bulk DMI 0.3, B_z = 0.2) at L = 16 periodic, below and
    # above the ordering temperature
    "c4h_T08": dict(shape="c", edge=16, periodic=True, ising=False, jfile="3d_nn_bloch.dat", D=0.3,
                    T=0.8, H=0.2, chains=32, eq=3000, samples=15000),
    "c4h_T16": dict(shape="c", edge=16, periodic=True, ising=False, jfile="3d_nn_bloch.dat", D=0.3,
                    T=1.6, H=0.2, chains=32, eq=3000, samples=15000),
    # the same Hamiltonian at L = 12 (rows of 6 sites per colour: the one-site-per-thread kernel)
    "c4h_L12": dict(shape="c", edge=12, periodic=True, ising=False, jfile="3d_nn_bloch.dat", D=0.3,
                    T=1.2, H=0.2, chains=32, eq=3000, samples=15000),
    # a 3-D Weibull sphere (LATTSHAPE x, scale radius 6, box edge 18, about 1.2k sites)
    "x_sphere": dict(shape="x", edge=18, size=6.0, periodic=False, ising=False, jfile="3d_nn_bloch.dat", D=0.3,
                     T=1.0, H=0.2, chains=32, eq=3000, samples=20000),
    # 2-D Ising, L = 32 with open boundaries, zero field, near and below T_c
    "ising_open_T23": dict(shape="s", edge=32, periodic=False, ising=True, jfile="2d_nn.dat", D=0.0,
                           T=2.3, H=0.0, chains=32, eq=3000, samples=20000),
    "ising_open_T20": dict(shape="s", edge=32, periodic=False, ising=True, jfile="2d_nn.dat", D=0.0,
                           T=2.0, H=0.0, chains=32, eq=3000, samples=20000),
}


def oracle_lattice(case):
    from nanomagmc_gb300.sampler import interactions_file
    from oracle import oracle as O
    dim = 3 if case["shape"] in "cx" else 2
    off, J, Dv = O.read_interactions(interactions_file(case["jfile"]), dim, 1.0, case["D"])
    o = O.Lattice.create(dim, case["edge"], case["ising"], case["periodic"], case["shape"], off, J, Dv,
                         size=case.get("size", 0.0), wbeta=3.0, seed=case.get("mask_seed", 11), chain=0,
                         useJ=True, useD=(case["D"] != 0 and not case["ising"]))
    o.set_beta(1.0 / case["T"])
    if case["ising"]:
        o.set_H(case["H"], 0.0, 0.0)
    else:
        o.set_H(0.0, 0.0, case["H"])
    return o


def run_chain(args):
    """One oracle chain: per-sweep E/N, |M|/N, Q after `eq` sweeps."""
    from oracle import oracle as O
    case, k = args
    o = oracle_lattice(case)
    seed = 1000 * (k + 1) + 7
    rng = O.Rng(seed, seed + 1, seed + 2)
    o.all_rand(rng)
    o.equil(rng, case["eq"] * o.n)
    n = o.n
    E = np.empty(case["samples"])
    M = np.empty(case["samples"])
    Q = np.empty(case["samples"])
    for i in range(case["samples"]):
        o.equil(rng, n)
        E[i] = o.energy() / n
        M[i] = np.linalg.norm(o.mag()) / n
        Q[i] = 0.0 if case["ising"] else o.tcharge().sum()
    return n, E, M, Q


def summarise(case, results):
    from stats import binned_error
    n = results[0][0]
    out = {"sites": int(n)}
    for j, name in ((1, "E"), (2, "M"), (3, "Q")):
        if name == "Q" and case["ising"]:
            continue
        means = np.array([r[j].mean() for r in results])
        out[name] = {"mean": float(means.mean()), "err": float(means.std(ddof=1) / np.sqrt(len(means))),
                     "binned_err": float(np.sqrt(sum(binned_error(r[j]) ** 2 for r in results)) / len(results))}
    return out


def generate(names, quick=False, processes=None):
    cases = {k: dict(CASES[k]) for k in names}
    if quick:
        for c in cases.values():
            c.update(chains=2, eq=200, samples=300)
    jobs = [(c, k) for c in cases.values() for k in range(c["chains"])]
    with mp.get_context("spawn").Pool(processes or os.cpu_count()) as pool:
        res = pool.map(run_chain, jobs)
    out, i = {}, 0
    for name, c in cases.items():
        out[name] = dict(c)
        out[name].update(summarise(c, res[i:i + c["chains"]]))
        i += c["chains"]
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--only", default=None)
    ap.add_argument("--quick", action="store_true")
    a = ap.parse_args()
    names = [a.only] if a.only else list(CASES)
    out = generate(names, a.quick)
    if a.quick:
        print(json.dumps(out, indent=1))
        return
    old = json.load(open(OUT)) if os.path.exists(OUT) else {}
    old.update(out)
    json.dump(old, open(OUT, "w"), indent=1, sort_keys=True)
    for k, v in out.items():
        print(k, v["sites"], {o: (round(v[o]["mean"], 5), round(v[o]["err"], 5)) for o in ("E", "M", "Q") if o in v})


if __name__ == "__main__":
    main()
