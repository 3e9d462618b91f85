"""ctypes binding of libnmmc's C ABI (include/nmmc.h).

This module loads the in-tree ``_build/libnmmc.so`` and raises if it is missing: there is no
CPU fallback. Struct layouts mirror the header exactly.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libnmmc.so")

MAX_PATH = 256
MAX_OFFSETS = 2048
MAX_CHAINS = 65535

OK = 0
ERR_SHAPE = 103
ERR_TEMP = 104
ERR_INPUT = 105
ERR_PROTOCOL = 207
ERR_ARG = 300
ERR_UNSUPPORTED = 301
ERR_CUDA = 302
ERR_TIMEOUT = 303
ERR_NOMEM = 304
ERR_IO = 305

OBS_E, OBS_M, OBS_ABSM, OBS_SUBM, OBS_ABSSUBM, OBS_SUB4M, OBS_ABSSUB4M, OBS_QTOT, OBS_N = \
    0, 1, 4, 5, 8, 9, 12, 13, 14
ACC_N = 8
GEN_OPT_TENSOR_CORES = 1
GEN_OPT_TILE_ROWS = 2
GEN_OPT_WEIGHT_IMAGE = 3
GEN_OPT_SCHEDULE = 4
STATIC_SCRATCH_DOUBLES = 262144

OPT_SWEEP_PATH, OPT_DMI_SIGN, OPT_MEASURE_FP64, OPT_PERIODIC_Q, OPT_TIMING, \
    OPT_RESIDENT_THREADS, OPT_RESIDENT_BINS, OPT_HALF_KERNEL, OPT_COLOURS, OPT_MEASURE_SITES, \
    OPT_RESIDENT_PREDRAW, OPT_MASKED_COMPACT, OPT_WAIT_LIMIT, OPT_RING_ZSEG, OPT_L2_PREFETCH, OPT_WAVE, \
    OPT_RESIDENT_STENCIL, OPT_CHARGE_PASS = 1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12, 13, 14, 15, 16, 17, 18


class Options(C.Structure):
    _fields_ = [
        ("size", C.c_double), ("edge_size", C.c_double), ("is_perio", C.c_int),
        ("is_ising", C.c_int), ("shape_code", C.c_char), ("J", C.c_double), ("K", C.c_double),
        ("H", C.c_double), ("k_b", C.c_double), ("T", C.c_double), ("beta_w", C.c_double),
        ("int_file", C.c_char * MAX_PATH), ("temp_file", C.c_char * MAX_PATH),
        ("field_file", C.c_char * MAX_PATH), ("out_file", C.c_char * MAX_PATH),
        ("samp_sweeps", C.c_int), ("n_samp", C.c_int), ("eq_sweeps", C.c_int),
        ("n_latts", C.c_int), ("protocol", C.c_int), ("distrib", C.c_int),
        ("amean", C.c_double), ("asd", C.c_double), ("lmean", C.c_double), ("lsd", C.c_double),
    ]


class Interactions(C.Structure):
    _fields_ = [("dim", C.c_int), ("n", C.c_int), ("offset", (C.c_int * 3) * MAX_OFFSETS),
                ("J", C.c_double * MAX_OFFSETS), ("D", (C.c_double * 3) * MAX_OFFSETS)]


class ChainDesc(C.Structure):
    _fields_ = [("lattice", C.c_int), ("size", C.c_double), ("T", C.c_double), ("H", C.c_double)]


class Info(C.Structure):
    _fields_ = [("dim", C.c_int), ("edge", C.c_int), ("is_ising", C.c_int), ("is_perio", C.c_int),
                ("nchains", C.c_int), ("nslices", C.c_int), ("box_sites", C.c_longlong),
                ("shape_code", C.c_char)]


class Event(C.Structure):
    _fields_ = [("site_box", C.c_int32), ("accepted", C.c_int32), ("trial", C.c_double * 3),
                ("u", C.c_double), ("dE", C.c_double)]


# name -> (restype, argtypes); every function declared in include/nmmc.h
vp, i32, i64, u64, dbl, sz = C.c_void_p, C.c_int, C.c_int64, C.c_uint64, C.c_double, C.c_size_t
P = C.POINTER
SIGNATURES = {
    "nmmc_read_input": (i32, [C.c_char_p, P(Options)]),
    "nmmc_load_lists": (i32, [P(Options), C.c_char_p, vp, i32, P(i32), vp, i32, P(i32)]),
    "nmmc_read_interactions": (i32, [C.c_char_p, i32, dbl, dbl, P(Interactions)]),
    "nmmc_colouring": (i32, [i32, i32, i32, i32, P(Interactions), P(C.c_int)]),
    "nmmc_protocol_plan": (i32, [i32, i32, i32] + [P(i32)] * 7),
    "nmmc_lognormal_size": (dbl, [u64, i32, dbl, dbl]),
    "nmmc_binning": (i32, [vp, i32, P(dbl), P(dbl), P(dbl)]),
    "nmmc_shape_mask": (i32, [C.c_char, i32, dbl, dbl, u64, i32, vp, P(i32), P(i32), P(i32)]),
    "nmmc_create": (i32, [P(Options), P(Interactions), vp, i32, u64, P(vp)]),
    "nmmc_destroy": (None, [vp]),
    "nmmc_get_info": (i32, [vp, P(Info)]),
    "nmmc_site_counts": (i32, [vp, i32, P(i32), P(i32), P(i32)]),
    "nmmc_set_point": (i32, [vp, i32, dbl, dbl]),
    "nmmc_set_points": (i32, [vp, vp, vp, vp, i32]),
    "nmmc_get_point": (i32, [vp, i32, P(dbl), P(dbl)]),
    "nmmc_change_v1": (i32, [vp, i32, i32, dbl]),
    "nmmc_change_v2": (i32, [vp, i32, i32, dbl]),
    "nmmc_fork": (i32, [vp, i32, i32]),
    "nmmc_sweep": (i32, [vp, vp, i32, i32]),
    "nmmc_measure": (i32, [vp, vp, i32, vp, vp, i32]),
    "nmmc_sweep_measure": (i32, [vp, vp, i32, i32, vp, vp, i32]),
    "nmmc_sample": (i32, [vp, vp, i32, i32, i32, vp, vp]),
    "nmmc_measure_static": (i32, [vp, vp, i32, vp, vp]),
    "nmmc_get_accumulators": (i32, [vp, vp, i32, vp]),
    "nmmc_reset_accumulators": (i32, [vp]),
    "nmmc_get_spins": (i32, [vp, i32, vp, sz]),
    "nmmc_set_spins": (i32, [vp, i32, vp, sz]),
    "nmmc_set_av_chains": (i32, [vp, vp, i32]),
    "nmmc_get_av": (i32, [vp, i32, vp, sz]),
    "nmmc_get_mask": (i32, [vp, i32, vp, sz]),
    "nmmc_delta_e": (i32, [vp, i32, vp, vp, i32, vp]),
    "nmmc_debug_replay": (i32, [vp, i32, vp, sz, vp, P(i64), vp]),
    "nmmc_set_option": (i32, [vp, i32, i64]),
    "nmmc_get_option": (i32, [vp, i32, P(i64)]),
    "nmmc_get_timing": (i32, [vp, P(dbl), P(C.c_longlong), P(C.c_longlong)]),
    "nmmc_timer_mark": (i32, [vp, i32]),
    "nmmc_timer_elapsed": (i32, [vp, i32, i32, P(dbl)]),
    "nmmc_host_alloc": (i32, [sz, P(vp)]),
    "nmmc_host_free": (i32, [vp]),
    "nmmc_stream": (vp, [vp]),
    "nmmc_synchronize": (i32, [vp]),
    "nmmc_last_error": (C.c_char_p, []),
    "nmmc_run": (i32, [C.c_char_p, C.c_char_p, C.c_char_p, u64, i32]),
    "nmmc_gen_create": (i32, [i32, i32, u64, P(vp)]),
    "nmmc_gen_destroy": (None, [vp]),
    "nmmc_gen_param_count": (i32, [vp]),
    "nmmc_gen_get_params": (i32, [vp, vp, i32]),
    "nmmc_gen_set_params": (i32, [vp, vp, i32]),
    "nmmc_gen_add_snapshots": (i32, [vp, vp, vp, i32, vp]),
    "nmmc_gen_dataset_size": (i32, [vp]),
    "nmmc_gen_train_step": (i32, [vp, vp, vp, i32, C.c_float, P(dbl)]),
    "nmmc_gen_get_grads": (i32, [vp, vp, i32]),
    "nmmc_gen_get_input": (i32, [vp, i32, vp]),
    "nmmc_gen_warm_start": (i32, [vp, vp, vp, i32, vp, i32, i32]),
    "nmmc_gen_set_option": (i32, [vp, i32, C.c_int64]),
    "nmmc_gen_probe_conv": (i32, [vp, i32, i32, vp, vp, i32]),
    "nmmc_gen_probe_wgrad": (i32, [vp, i32, vp, vp, vp, i32]),
    "nmmc_reference_stats": (i32, [vp, vp, i32, i32, i32, i32, vp]),
    "nmmc_gen_gated_warm_start": (i32, [vp, vp, vp, i32, vp, i32, i32, i32, i32, vp, u64, P(i32)]),
    "nmmc_gen_save": (i32, [vp, C.c_char_p]),
    "nmmc_gen_load": (i32, [vp, C.c_char_p]),
}

_lib = None


class NmmcError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("nmmc error %d: %s" % (code, msg))
        self.code = code


def load(path: str | None = None):
    """Loads libnmmc; raises FileNotFoundError when it has not been built."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise FileNotFoundError(
            "libnmmc is not built (%s); run `python -c \"import __graft_entry__ as g; g.build()\"`" % p)
    lib = C.CDLL(p)
    for name, (res, args) in SIGNATURES.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    if path is None:
        _lib = lib
    return lib


def check(rc: int):
    if rc != OK:
        raise NmmcError(rc, load().nmmc_last_error().decode(errors="replace"))
    return rc
