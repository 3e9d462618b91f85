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


def test_integration_guide_lists_every_entry_point():
    text = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    missing = [n for n in declared("nmmc.h") if "`%s`" % n not in text]
    assert not missing, missing


def test_struct_sizes_match_the_header_layout():
    # nmmc_event is written by the oracle and read by the library: 48 bytes, 8-aligned
    assert ctypes.sizeof(L.Event) == 48
    assert ctypes.sizeof(L.ChainDesc) == 32
    # nmmc_interactions: dim, n, then NMMC_MAX_OFFSETS records of 3 ints, J and 3 doubles
    assert L.MAX_OFFSETS == int(re.search(r"#define NMMC_MAX_OFFSETS (\d+)",
                                          open(os.path.join(ROOT, "include", "nmmc.h")).read()).group(1))
    assert ctypes.sizeof(L.Interactions) == 8 + L.MAX_OFFSETS * (12 + 8 + 24)
