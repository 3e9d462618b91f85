"""Python face of libnmmc: a batch of Metropolis chains on one GPU.

``Sampler`` holds many chains (the reference's ``state`` objects) in one device context;
``State`` is the single-chain view with the reference's method names
(Old/includes/state.hpp:12-52): ``equil``, ``energy``, ``magnetisation``, ``submag``,
``sub4mag``, ``tcharge``, ``change_temp``, ``change_field``, ``change_v1``, ``change_v2``.
Every call goes through the C ABI; nothing here computes physics.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import _lib as L

DATA_DIR = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "data")


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def read_input(path: str) -> L.Options:
    """read_all_vars (Old/lib/param_read.cpp:35-82)."""
    o = L.Options()
    L.check(L.load().nmmc_read_input(path.encode(), C.byref(o)))
    return o


def load_lists(opt: L.Options, workdir: str = "."):
    """load_Hs_Ts (Old/lib/param_read.cpp:84-151) -> (Ts, Hs)."""
    T = np.zeros(65536)
    H = np.zeros(65536)
    nT = C.c_int()
    nH = C.c_int()
    L.check(L.load().nmmc_load_lists(C.byref(opt), workdir.encode(), _p(T), len(T), C.byref(nT),
                                     _p(H), len(H), C.byref(nH)))
    return T[:nT.value].copy(), H[:nH.value].copy()


def read_interactions(path: str, dim: int, J: float = 1.0, D: float = 0.0) -> L.Interactions:
    """Js/ file reader (Old/lib/field_type.cpp:39-73)."""
    it = L.Interactions()
    L.check(L.load().nmmc_read_interactions(path.encode(), dim, J, D, C.byref(it)))
    return it


def interactions_file(name: str) -> str:
    return os.path.join(DATA_DIR, "Js", name)


def make_options(shape="s", edge=None, size=None, ising=False, periodic=True, J=1.0, D=0.0,
                 k_b=1.0, weibull=3.0, asd=0.0) -> L.Options:
    """Options for programmatic use (the fields read_all_vars would fill)."""
    o = L.Options()
    o.shape_code = shape.encode()[:1]
    o.is_ising = int(ising)
    o.is_perio = int(periodic)
    o.J = J
    o.K = D
    o.k_b = k_b
    o.beta_w = weibull
    amean = float(size if size is not None else edge)
    o.amean = amean
    o.asd = asd
    o.size = amean
    if edge is not None:
        o.edge_size = float(edge)
    elif shape in "wWxX":
        o.edge_size = (amean + 2 * asd) * 3
    else:
        o.edge_size = amean + 2 * asd
    return o


class Sampler:
    """A batch of chains sharing one lattice model (one device context)."""

    def __init__(self, opt: L.Options, inter: L.Interactions, T, H=0.0, sizes=None, lattices=None,
                 seed: int = 1):
        T = np.atleast_1d(np.asarray(T, np.float64))
        n = len(T)
        H = np.broadcast_to(np.asarray(H, np.float64), (n,))
        sizes = np.broadcast_to(np.asarray(opt.size if sizes is None else sizes, np.float64), (n,))
        lattices = np.arange(n) if lattices is None else np.broadcast_to(np.asarray(lattices), (n,))
        descs = (L.ChainDesc * n)()
        for i in range(n):
            descs[i].lattice = int(lattices[i])
            descs[i].size = float(sizes[i])
            descs[i].T = float(T[i])
            descs[i].H = float(H[i])
        self.lib = L.load()
        h = C.c_void_p()
        L.check(self.lib.nmmc_create(C.byref(opt), C.byref(inter), descs, n, seed, C.byref(h)))
        self.h = h
        info = L.Info()
        L.check(self.lib.nmmc_get_info(self.h, C.byref(info)))
        self.dim, self.edge, self.nchains, self.nslices = info.dim, info.edge, info.nchains, info.nslices
        self.box_sites = info.box_sites
        self.ising = bool(info.is_ising)

    def close(self):
        if getattr(self, "h", None):
            self.lib.nmmc_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # ---- helpers ----
    def _list(self, chains):
        if chains is None:
            return None, self.nchains
        a = np.ascontiguousarray(np.atleast_1d(chains), np.int32)
        return a, len(a)

    def option(self, key, value=None):
        if value is None:
            v = C.c_int64()
            L.check(self.lib.nmmc_get_option(self.h, key, C.byref(v)))
            return v.value
        L.check(self.lib.nmmc_set_option(self.h, key, int(value)))

    # ---- the reference's verbs ----
    def site_counts(self, chain=0):
        n, s, s4 = C.c_int(), C.c_int(), C.c_int()
        L.check(self.lib.nmmc_site_counts(self.h, chain, C.byref(n), C.byref(s), C.byref(s4)))
        return n.value, s.value, s4.value

    def set_point(self, chain, T, H):
        L.check(self.lib.nmmc_set_point(self.h, chain, T, H))

    def get_point(self, chain):
        T, H = C.c_double(), C.c_double()
        L.check(self.lib.nmmc_get_point(self.h, chain, C.byref(T), C.byref(H)))
        return T.value, H.value

    def set_points(self, chains, T, H):
        c = np.ascontiguousarray(chains, np.int32)
        T = np.ascontiguousarray(T, np.float64)
        H = np.ascontiguousarray(H, np.float64)
        L.check(self.lib.nmmc_set_points(self.h, _p(c), _p(T), _p(H), len(c)))

    def change_v1(self, chain, protocol, v):
        L.check(self.lib.nmmc_change_v1(self.h, chain, protocol, v))

    def change_v2(self, chain, protocol, v):
        L.check(self.lib.nmmc_change_v2(self.h, chain, protocol, v))

    def fork(self, src, dst):
        L.check(self.lib.nmmc_fork(self.h, src, dst))

    def sweep(self, nsweeps, chains=None):
        a, n = self._list(chains)
        L.check(self.lib.nmmc_sweep(self.h, _p(a), n, int(nsweeps)))

    def measure(self, chains=None, accumulate=False, with_q=True):
        a, n = self._list(chains)
        obs = np.zeros((n, L.OBS_N))
        q = np.zeros((n, self.nslices)) if with_q else None
        L.check(self.lib.nmmc_measure(self.h, _p(a), n, _p(obs), _p(q), int(accumulate)))
        return (obs, q) if with_q else obs

    def set_av_chains(self, chains):
        """Chains whose spins are summed at every accumulating measurement (add_to_av)."""
        a = np.ascontiguousarray(chains if chains is not None else [], np.int32)
        L.check(self.lib.nmmc_set_av_chains(self.h, _p(a) if len(a) else None, len(a)))

    def get_av(self, chain):
        out = np.zeros((self.box_sites, 3))
        L.check(self.lib.nmmc_get_av(self.h, chain, _p(out), self.box_sites))
        return out

    def sweep_measure(self, nsweeps, chains=None, accumulate=False, with_q=True):
        """nsweeps sweeps then the observables, in one launch where the lattice is held on chip."""
        a, n = self._list(chains)
        obs = np.zeros((n, L.OBS_N))
        q = np.zeros((n, self.nslices)) if with_q else None
        L.check(self.lib.nmmc_sweep_measure(self.h, _p(a), n, int(nsweeps), _p(obs), _p(q), int(accumulate)))
        return (obs, q) if with_q else obs

    def sample(self, nsweeps, nsamples, chains=None, with_q=False):
        a, n = self._list(chains)
        obs = np.zeros((nsamples, n, L.OBS_N))
        q = np.zeros((nsamples, n, self.nslices)) if with_q else None
        L.check(self.lib.nmmc_sample(self.h, _p(a), n, int(nsweeps), int(nsamples), _p(obs), _p(q)))
        return (obs, q) if with_q else obs

    def accumulators(self, chains=None):
        a, n = self._list(chains)
        out = np.zeros((n, L.ACC_N))
        L.check(self.lib.nmmc_get_accumulators(self.h, _p(a), n, _p(out)))
        return out

    def reset_accumulators(self):
        L.check(self.lib.nmmc_reset_accumulators(self.h))

    def get_spins(self, chain=0):
        out = np.zeros((self.box_sites, 3))
        L.check(self.lib.nmmc_get_spins(self.h, chain, _p(out), self.box_sites))
        return out

    def set_spins(self, chain, xyz):
        a = np.ascontiguousarray(xyz, np.float64).reshape(self.box_sites, 3)
        L.check(self.lib.nmmc_set_spins(self.h, chain, _p(a), self.box_sites))

    def mask(self, chain=0):
        out = np.zeros(self.box_sites, np.uint8)
        L.check(self.lib.nmmc_get_mask(self.h, chain, _p(out), self.box_sites))
        return out

    def delta_e(self, chain, sites, trial):
        s = np.ascontiguousarray(sites, np.int32)
        t = np.ascontiguousarray(trial, np.float64).reshape(len(s), 3)
        out = np.zeros(len(s))
        L.check(self.lib.nmmc_delta_e(self.h, chain, _p(s), _p(t), len(s), _p(out)))
        return out

    def debug_replay(self, chain, events, want_final=True):
        ev = np.ascontiguousarray(events)
        acc = np.zeros(len(ev), np.uint8)
        first = C.c_int64(-2)
        fin = np.zeros((self.box_sites, 3)) if want_final else None
        L.check(self.lib.nmmc_debug_replay(self.h, chain, _p(ev), len(ev), _p(acc), C.byref(first), _p(fin)))
        return first.value, acc, fin

    def timing(self):
        ms, la, up = C.c_double(), C.c_longlong(), C.c_longlong()
        L.check(self.lib.nmmc_get_timing(self.h, C.byref(ms), C.byref(la), C.byref(up)))
        return ms.value, la.value, up.value

    def stream(self):
        return self.lib.nmmc_stream(self.h)

    def synchronize(self):
        L.check(self.lib.nmmc_synchronize(self.h))


class State:
    """One chain with the reference's `state` interface (Old/includes/state.hpp:12-52)."""

    def __init__(self, sampler: Sampler, chain: int = 0):
        self.s = sampler
        self.chain = chain
        self._n = sampler.site_counts(chain)

    def num_spins(self):
        return self._n[0]

    def sub_num(self, sub=0):
        return self._n[1]

    def sub4_num(self):
        return self._n[2]

    def equil(self, iters):
        """equil(iter): iter = sweeps * num_spins attempts (checkerboard sweeps here)."""
        n = self.num_spins()
        if iters % n:
            raise ValueError("iter must be a multiple of num_spins() (whole sweeps)")
        self.s.sweep(iters // n, [self.chain])

    def _obs(self):
        obs, q = self.s.measure([self.chain])
        return obs[0], q[0]

    def energy(self):
        return self._obs()[0][L.OBS_E]

    def magnetisation(self):
        return list(self._obs()[0][1:4]) + [0.0]

    def submag(self, sub=0):
        return list(self._obs()[0][5:8]) + [0.0]

    def sub4mag(self):
        return list(self._obs()[0][9:12]) + [0.0]

    def tcharge(self):
        return list(self._obs()[1])

    def change_temp(self, T):
        L.check(self.s.lib.nmmc_set_point(self.s.h, self.chain, T, self._H()))

    def change_field(self, H):
        L.check(self.s.lib.nmmc_set_point(self.s.h, self.chain, self._T(), H))

    def change_v1(self, protocol, v):
        self.s.change_v1(self.chain, protocol, v)

    def change_v2(self, protocol, v):
        self.s.change_v2(self.chain, protocol, v)

    def _point(self):
        T, H = C.c_double(), C.c_double()
        L.check(self.s.lib.nmmc_get_point(self.s.h, self.chain, C.byref(T), C.byref(H)))
        return T.value, H.value

    def _T(self):
        return self._point()[0]

    def _H(self):
        return self._point()[1]
