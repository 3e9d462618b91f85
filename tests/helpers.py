"""Shared set-up for the parity tests: one libnmmc context and the oracle's lattice built
from the same options, interaction file and seed."""
from __future__ import annotations

import numpy as np

from nanomagmc_gb300 import _lib as L
from nanomagmc_gb300.sampler import Sampler, interactions_file, make_options, read_interactions
from oracle import oracle as O

STENCIL = np.array([[1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0], [0, 0, 1], [0, 0, -1]], np.int32)


def box_index(locs, edge):
    return locs[:, 0] + edge * (locs[:, 1] + edge * locs[:, 2])


def pair(shape="s", edge=8, ising=False, periodic=True, jfile=None, J=1.0, D=0.0, size=None,
         wbeta=3.0, seed=11, T=(1.0,), H=0.0, lattices=None, sizes=None):
    """(sampler, [oracle lattice per chain]) for the same model."""
    dim = 3 if shape in "cCxX" else 2
    if jfile is None:
        jfile = "3d_nn_bloch.dat" if dim == 3 else "2d_nn_interfacial.dat"
    path = jfile if "/" in jfile else interactions_file(jfile)
    opt = make_options(shape, edge=edge, size=size, ising=ising, periodic=periodic, J=J, D=D,
                       weibull=wbeta)
    inter = read_interactions(path, dim, J, D)
    T = np.atleast_1d(np.asarray(T, float))
    s = Sampler(opt, inter, T=T, H=H, sizes=sizes, lattices=lattices, seed=seed)
    edge = s.edge
    off, Jv, Dv = O.read_interactions(path, dim, J, D)
    ors = []
    lat = np.arange(len(T)) if lattices is None else np.broadcast_to(np.asarray(lattices), (len(T),))
    sz = np.broadcast_to(np.asarray(opt.size if sizes is None else sizes, float), (len(T),))
    Hs = np.broadcast_to(np.asarray(H, float), (len(T),))
    for c in range(len(T)):
        o = O.Lattice.create(dim, edge, ising, periodic, shape, off, Jv, Dv, size=float(sz[c]),
                             wbeta=wbeta, seed=seed, chain=int(lat[c]), useJ=(J != 0),
                             useD=(D != 0 and not ising))
        o.set_beta(1.0 / T[c])
        if ising:
            o.set_H(float(Hs[c]), 0, 0)
        else:
            o.set_H(0, 0, float(Hs[c]))
        ors.append(o)
    return s, ors


def random_spins(n, ising, rng):
    if ising:
        v = np.zeros((n, 3))
        v[:, 0] = rng.choice([-1.0, 1.0], size=n)
        return v
    v = rng.normal(size=(n, 3))
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    return v.astype(np.float32).astype(np.float64)   # representable in the FP32 store


def load_same(s, o, chain, rng):
    """Random configuration set identically on the GPU chain and the oracle lattice."""
    locs = o.locs()
    box = box_index(locs, s.edge)
    v = random_spins(len(locs), s.ising, rng)
    full = np.zeros((s.box_sites, 3))
    full[box] = v
    s.set_spins(chain, full)
    o.set_spins(v)
    return box


def oracle_from_gpu(s, o, chain):
    locs = o.locs()
    box = box_index(locs, s.edge)
    o.set_spins(s.get_spins(chain)[box])
    return box
