"""libnmmc loads and exports every function include/nmmc.h declares (no GPU calls)."""
import ctypes
import os
import re

from nanomagmc_gb300 import _lib as L

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared(header):
    text = open(os.path.join(ROOT, "include", header)).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(nmmc_[a-z0-9_]+)\s*\(", text)))


def test_every_declared_symbol_is_exported():
    lib = ctypes.CDLL(L.LIB_PATH)
    names = declared("nmmc.h")
    assert len(names) >= 30
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_covers_the_header():
    names = set(declared("nmmc.h"))
    assert names == set(L.SIGNATURES), names ^ set(L.SIGNATURES)


def test_struct_sizes_match_the_header_layout():
    # nmmc_event is written by the oracle and read by the library: 48 bytes, 8-aligned
    assert ctypes.sizeof(L.Event) == 48
    assert ctypes.sizeof(L.ChainDesc) == 32
    # nmmc_interactions: dim, n, then NMMC_MAX_OFFSETS records of 3 ints, J and 3 doubles
    assert L.MAX_OFFSETS == int(re.search(r"#define NMMC_MAX_OFFSETS (\d+)",
                                          open(os.path.join(ROOT, "include", "nmmc.h")).read()).group(1))
    assert ctypes.sizeof(L.Interactions) == 8 + L.MAX_OFFSETS * (12 + 8 + 24)


def header_enum_values():
    """NAME = value pairs of the header's enums and #defines (comments removed)."""
    text = open(os.path.join(ROOT, "include", "nmmc.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    vals = {k: int(v) for k, v in re.findall(r"\b(NMMC_[A-Z0-9_]+)\s*=\s*(-?\d+)", text)}
    vals.update({k: int(v) for k, v in re.findall(r"#define\s+(NMMC_[A-Z0-9_]+)\s+(-?\d+)\b", text)})
    return vals


def test_binding_constants_match_the_header():
    """Every option, observable index and size constant of the binding has the header's value,
    and every option of the header has a binding constant."""
    vals = header_enum_values()
    checked = 0
    for name, v in vals.items():
        short = name[len("NMMC_"):]
        if hasattr(L, short):
            assert getattr(L, short) == v, (name, getattr(L, short), v)
            checked += 1
    options = [k for k in vals if k.startswith("NMMC_OPT_")]
    missing = [k for k in options if not hasattr(L, k[len("NMMC_"):])]
    assert not missing, missing
    assert checked >= len(options) + 8
