"""ORACLE — test infrastructure only.

Python handle on the CPU restatement in ``nmmc_oracle.cpp`` of NanoMagMC's hot path
(Old/lib/thermodynamics.cpp, Old/lib/state.cpp, Old/lib/field_type.cpp,
Old/lib/shape.cpp). Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` may use it, and only as the checker: the product never imports it.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

_lib = None

EVENT_DTYPE = np.dtype([("site_box", "<i4"), ("accepted", "<i4"), ("trial", "<f8", (3,)),
                        ("u", "<f8"), ("dE", "<f8")])


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = C.CDLL(path)
        vp, i32, u32, u64, dbl = C.c_void_p, C.c_int, C.c_uint32, C.c_uint64, C.c_double
        P = C.POINTER
        L.orc_create.restype = vp
        L.orc_create.argtypes = [i32, i32, i32, i32, C.c_char, dbl, dbl, u64, u32, vp,
                                 i32, vp, vp, vp, i32, i32]
        L.orc_fixture.restype = vp
        L.orc_fixture.argtypes = [i32, i32, i32, i32, i32, vp, vp, vp]
        L.orc_destroy.argtypes = [vp]
        for f in ("orc_num_sites", "orc_snum", "orc_s4num"):
            getattr(L, f).restype = i32
            getattr(L, f).argtypes = [vp]
        L.orc_set_flags.argtypes = [vp, i32, i32, i32]
        L.orc_set_H.argtypes = [vp, dbl, dbl, dbl]
        L.orc_set_beta.argtypes = [vp, dbl]
        L.orc_locs.argtypes = [vp, vp]
        L.orc_get_spins.argtypes = [vp, vp]
        L.orc_set_spins.argtypes = [vp, vp]
        L.orc_all_rand.argtypes = [vp, vp]
        L.orc_neighbours.restype = i32
        L.orc_neighbours.argtypes = [vp, i32, vp, vp, i32]
        L.orc_adj.argtypes = [vp, vp]
        L.orc_energy.restype = dbl
        L.orc_energy.argtypes = [vp]
        L.orc_dE.restype = dbl
        L.orc_dE.argtypes = [vp, i32, vp]
        L.orc_mag.argtypes = [vp, vp]
        L.orc_submag.argtypes = [vp, i32, vp]
        L.orc_sub4mag.argtypes = [vp, vp]
        L.orc_tcharge.restype = i32
        L.orc_tcharge.argtypes = [vp, vp]
        L.orc_solid_angle.restype = dbl
        L.orc_solid_angle.argtypes = [vp, vp, vp]
        L.orc_rng_create.restype = vp
        L.orc_rng_create.argtypes = [C.c_ulong, C.c_ulong, C.c_ulong]
        L.orc_rng_destroy.argtypes = [vp]
        L.orc_rng_uniform.restype = dbl
        L.orc_rng_uniform.argtypes = [vp]
        L.orc_rng_int2.restype = i32
        L.orc_rng_int2.argtypes = [vp]
        L.orc_rng_dir3d.argtypes = [vp, vp]
        L.orc_rng_lognormal.restype = dbl
        L.orc_rng_lognormal.argtypes = [vp, dbl, dbl]
        L.orc_gen_rand.argtypes = [vp, vp, vp]
        L.orc_equil.argtypes = [vp, vp, C.c_long, vp]
        L.orc_replay.restype = C.c_long
        L.orc_replay.argtypes = [vp, vp, C.c_long, vp]
        L.orc_event_size.restype = i32
        L.orc_cb_ising.argtypes = [vp, u64, u32, u64, i32, vp, i32, vp, C.c_float]
        L.orc_colour_ising.argtypes = [vp, u64, u32, u64, i32, i32, i32, i32, i32, i32, C.c_float]
        L.orc_philox.argtypes = [vp, vp, vp]
        L.orc_philox_boxes.argtypes = [u64, u32, u64, u32, u32, C.c_long, vp]
        L.orc_rng_fill.argtypes = [vp, i32, C.c_long, dbl, dbl, vp]
        L.orc_mask_uniform.restype = dbl
        L.orc_mask_uniform.argtypes = [u64, u32, u32]
        L.orc_read_interactions.restype = i32
        L.orc_read_interactions.argtypes = [C.c_char_p, i32, dbl, dbl, i32, vp, vp, vp]
        L.orc_bench_equil.restype = C.c_long
        L.orc_bench_equil.argtypes = [vp, vp, C.c_long]
        assert L.orc_event_size() == EVENT_DTYPE.itemsize
        _lib = L
    return _lib


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


def read_interactions(path: str, d: int, jmod: float, dmod: float, cap: int = 4096):
    """Interaction file reader (Old/lib/field_type.cpp:39-73)."""
    off = np.zeros((cap, 3), np.int32)
    J = np.zeros(cap, np.float64)
    D = np.zeros((cap, 3), np.float64)
    n = lib().orc_read_interactions(path.encode(), d, jmod, dmod, cap, _ptr(off), _ptr(J), _ptr(D))
    if n < 0:
        raise FileNotFoundError(path)
    return off[:n].copy(), J[:n].copy(), D[:n].copy()


def philox(ctr, key):
    c = np.asarray(ctr, np.uint32)
    k = np.asarray(key, np.uint32)
    out = np.zeros(4, np.uint32)
    lib().orc_philox(_ptr(c), _ptr(k), _ptr(out))
    return out


class Rng:
    """The reference's three MT19937 generators (int, double, sphere)."""

    def __init__(self, seed_int=1, seed_double=2, seed_sphere=3):
        self.h = lib().orc_rng_create(seed_int, seed_double, seed_sphere)

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_rng_destroy(self.h)
            self.h = None

    def uniform(self):
        return lib().orc_rng_uniform(self.h)

    def int2(self):
        return lib().orc_rng_int2(self.h)

    def dir3d(self):
        out = np.zeros(3)
        lib().orc_rng_dir3d(self.h, _ptr(out))
        return out

    def lognormal(self, zeta, sigma):
        return lib().orc_rng_lognormal(self.h, zeta, sigma)

    def fill(self, kind, n, a=0.0, b=0.0):
        """n bulk draws: kind "uniform", "int2", "lognormal" (a=zeta, b=sigma) or "dir3d" (n x 3)."""
        k = ("uniform", "int2", "lognormal", "dir3d").index(kind)
        out = np.zeros(3 * n if k == 3 else n)
        lib().orc_rng_fill(self.h, k, n, a, b, _ptr(out))
        return out.reshape(n, 3) if k == 3 else out


def philox_boxes(seed, chain, sweep, nbox, box0=0, stream=0):
    """Sweep-stream Philox words of nbox consecutive boxes, shape (nbox, 4) uint32."""
    out = np.zeros((nbox, 4), np.uint32)
    lib().orc_philox_boxes(seed, chain, sweep, stream, box0, nbox, _ptr(out))
    return out


class Lattice:
    """One reference `field_type` + `state` (spins, neighbours, H, beta)."""

    def __init__(self, h):
        self.h = h
        self.n = lib().orc_num_sites(h)

    @classmethod
    def create(cls, d, edge, ising, periodic, shape, offsets, J, D, size=0.0, wbeta=0.0,
               seed=0, chain=0, mask=None, useJ=True, useD=False):
        off = np.ascontiguousarray(offsets, np.int32).reshape(-1, 3)
        J = np.ascontiguousarray(J, np.float64)
        D = np.ascontiguousarray(D, np.float64).reshape(-1, 3)
        m = None if mask is None else np.ascontiguousarray(mask, np.uint8)
        h = lib().orc_create(d, edge, int(ising), int(periodic), shape.encode()[:1], size, wbeta,
                             seed, chain, _ptr(m), len(J), _ptr(off), _ptr(J), _ptr(D),
                             int(useJ), int(useD))
        return cls(h)

    @classmethod
    def fixture(cls, kind, d, ising, periodic, offsets, J, D):
        """kind: 'fm' | 'afm' | 'skyrm' (Old/tests/test_functions.hpp:19-128)."""
        k = {"fm": 0, "afm": 1, "skyrm": 2}[kind]
        off = np.ascontiguousarray(offsets, np.int32).reshape(-1, 3)
        J = np.ascontiguousarray(J, np.float64)
        D = np.ascontiguousarray(D, np.float64).reshape(-1, 3)
        return cls(lib().orc_fixture(k, d, int(ising), int(periodic), len(J), _ptr(off),
                                     _ptr(J), _ptr(D)))

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_destroy(self.h)
            self.h = None

    # configuration ------------------------------------------------------------------
    def set_flags(self, useJ=True, useD=False, dmi_sign=0):
        lib().orc_set_flags(self.h, int(useJ), int(useD), int(dmi_sign))

    def set_H(self, hx=0.0, hy=0.0, hz=0.0):
        lib().orc_set_H(self.h, hx, hy, hz)

    def set_beta(self, beta):
        lib().orc_set_beta(self.h, beta)

    def locs(self):
        out = np.zeros((self.n, 3), np.int32)
        lib().orc_locs(self.h, _ptr(out))
        return out

    def spins(self):
        out = np.zeros((self.n, 3))
        lib().orc_get_spins(self.h, _ptr(out))
        return out

    def set_spins(self, s):
        s = np.ascontiguousarray(s, np.float64).reshape(self.n, 3)
        lib().orc_set_spins(self.h, _ptr(s))

    def all_rand(self, rng: Rng):
        lib().orc_all_rand(self.h, rng.h)

    def adj(self):
        out = np.zeros((self.n, 4), np.int32)
        lib().orc_adj(self.h, _ptr(out))
        return out

    def neighbours(self, site, cap=4096):
        nb = np.zeros(cap, np.int32)
        ch = np.zeros(cap, np.int32)
        k = lib().orc_neighbours(self.h, site, _ptr(nb), _ptr(ch), cap)
        return nb[:k].copy(), ch[:k].copy()

    @property
    def snum(self):
        return lib().orc_snum(self.h)

    @property
    def s4num(self):
        return lib().orc_s4num(self.h)

    # observables --------------------------------------------------------------------
    def energy(self):
        return lib().orc_energy(self.h)

    def dE(self, site, trial):
        t = np.ascontiguousarray(trial, np.float64)
        return lib().orc_dE(self.h, int(site), _ptr(t))

    def mag(self):
        out = np.zeros(3)
        lib().orc_mag(self.h, _ptr(out))
        return out

    def submag(self, sub=0):
        out = np.zeros(3)
        lib().orc_submag(self.h, sub, _ptr(out))
        return out

    def sub4mag(self):
        out = np.zeros(3)
        lib().orc_sub4mag(self.h, _ptr(out))
        return out

    def tcharge(self):
        out = np.zeros(4096)
        k = lib().orc_tcharge(self.h, _ptr(out))
        return out[:k].copy()

    def gen_rand(self, rng: Rng):
        out = np.zeros(3)
        lib().orc_gen_rand(self.h, rng.h, _ptr(out))
        return out

    # chains -------------------------------------------------------------------------
    def equil(self, rng: Rng, iters: int, log: bool = False):
        ev = np.zeros(iters, EVENT_DTYPE) if log else None
        lib().orc_equil(self.h, rng.h, int(iters), _ptr(ev))
        return ev

    def replay(self, events):
        acc = np.zeros(len(events), np.uint8)
        first = lib().orc_replay(self.h, _ptr(events), len(events), _ptr(acc))
        return first, acc

    def cb_ising(self, seed, chain, sweep0, nsweeps, Jdir, dirs, hx=0.0):
        Jd = np.ascontiguousarray(Jdir, np.float32)
        dd = np.ascontiguousarray(dirs, np.int32).reshape(-1, 3)
        lib().orc_cb_ising(self.h, seed, chain, sweep0, nsweeps, _ptr(Jd), len(Jd), _ptr(dd), hx)

    def colour_ising(self, seed, chain, sweep0, nsweeps, colouring, hx=0.0):
        """The general-table sweep's class-by-class order; colouring = nmmc_colouring's output."""
        kind, q, p, b, c = (int(v) for v in colouring[:5])
        lib().orc_colour_ising(self.h, seed, chain, sweep0, nsweeps, kind, q, p, b, c, hx)

    def bench_equil(self, rng: Rng, iters: int):
        return lib().orc_bench_equil(self.h, rng.h, int(iters))


def solid_angle(a, b, c):
    a, b, c = (np.ascontiguousarray(x, np.float64) for x in (a, b, c))
    return lib().orc_solid_angle(_ptr(a), _ptr(b), _ptr(c))


def mask_uniform(seed, chain, box):
    return lib().orc_mask_uniform(seed, chain, box)
