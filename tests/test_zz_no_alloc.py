"""nmmc_measure_static: the measurement entry point for callers that cannot allocate device
memory (stream-capture regions, pool-only frameworks, latency-critical loops). It must give
the observables of nmmc_measure, call after call, with caller-owned device outputs.

Kept in its own file, collected last, so a stop-at-first-failure run has already run every
other test; it also passes alone in a fresh process (the first call on the device sets up
the scratch address)."""
import ctypes as C

import numpy as np
import pytest

from nanomagmc_gb300 import _lib as L

from helpers import pair

pytestmark = pytest.mark.gpu

CASES = [
    dict(shape="c", edge=16, ising=False, periodic=True, jfile="3d_nn_bloch.dat", D=0.3),   # quad kernel
    dict(shape="w", size=6.0, ising=False, periodic=False, jfile="2d_nn_interfacial.dat", D=0.5),
    dict(shape="s", edge=12, ising=True, periodic=True, jfile="2d_nn.dat", D=0.0),
    # a 2-D lattice of several measurement blocks: the per-block FP32 sums must stay those of
    # nmmc_measure (the same block split), not one block per slice
    dict(shape="s", edge=256, ising=False, periodic=True, jfile="2d_nn_interfacial.dat", D=0.5),
]


def check_close(a, b, ising):
    # the tolerances of the parity tests: Ising exact; Heisenberg FP32 per-site terms 1e-5
    if ising:
        assert np.array_equal(a[:, :13], b[:, :13])
        return
    scale = np.maximum(1.0, np.abs(b[:, 0:1]))
    assert np.all(np.abs(a[:, 0] - b[:, 0]) <= 1e-5 * scale[:, 0])
    assert np.all(np.abs(a[:, 1:13] - b[:, 1:13]) <= 1e-5 * np.maximum(1.0, np.abs(b[:, 1:13]).max()))
    assert np.allclose(a[:, 13], b[:, 13], atol=1e-4)


@pytest.mark.parametrize("case", CASES, ids=lambda c: c["shape"] + str(c.get("edge", "")) + ("I" if c["ising"] else "H"))
def test_static_measure_matches_measure(case):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    lib = L.load()
    s, _ = pair(T=[0.6, 1.2, 2.5], H=[0.2, 0.0, 0.1], seed=9, **case)
    n, ns = s.nchains, s.nslices
    d_obs = torch.full((n, L.OBS_N), float("nan"), dtype=torch.float64, device="cuda")
    d_q = torch.full((n, ns), float("nan"), dtype=torch.float64, device="cuda")
    for call in range(2):   # two calls in a row, with sweeps and a new field in between
        s.sweep(3 + call)
        if call == 1:
            s.set_point(1, 1.2, 0.35)   # a changed field reaches the static call first
        rc = lib.nmmc_measure_static(s.h, None, n, C.c_void_p(d_obs.data_ptr()), C.c_void_p(d_q.data_ptr()))
        L.check(rc)
        s.synchronize()
        torch.cuda.synchronize()
        got, q_got = d_obs.cpu().numpy(), d_q.cpu().numpy()
        ref, q_ref = s.measure()
        check_close(got, ref, case["ising"])
        if not case["ising"]:
            assert np.allclose(q_got, q_ref, atol=1e-4)
    # a subset of chains given as a device array, results in list order
    idx = torch.tensor([2, 0], dtype=torch.int32, device="cuda")
    out = torch.zeros((2, L.OBS_N), dtype=torch.float64, device="cuda")
    L.check(lib.nmmc_measure_static(s.h, C.c_void_p(idx.data_ptr()), 2, C.c_void_p(out.data_ptr()), None))
    s.synchronize()
    ref, _ = s.measure([2, 0])
    check_close(out.cpu().numpy(), ref, case["ising"])
    s.close()


def test_static_measure_device_list_edges():
    """Out-of-range device-list entries are not read and give NaN rows; repeated entries are
    measured twice; an empty list does nothing."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    lib = L.load()
    s, _ = pair("c", edge=12, periodic=True, jfile="3d_nn_bloch.dat", D=0.3, T=[0.7, 1.4], H=0.2, seed=5)
    s.sweep(4)
    ref, q_ref = s.measure()
    idx = torch.tensor([1, -1, 0, 2, 1, 1 << 30], dtype=torch.int32, device="cuda")
    out = torch.zeros((6, L.OBS_N), dtype=torch.float64, device="cuda")
    q = torch.zeros((6, s.nslices), dtype=torch.float64, device="cuda")
    L.check(lib.nmmc_measure_static(s.h, C.c_void_p(idx.data_ptr()), 6, C.c_void_p(out.data_ptr()),
                                    C.c_void_p(q.data_ptr())))
    s.synchronize()
    got, qg = out.cpu().numpy(), q.cpu().numpy()
    for row, chain in ((0, 1), (2, 0), (4, 1)):
        check_close(got[row:row + 1], ref[chain:chain + 1], False)
        assert np.allclose(qg[row], q_ref[chain], atol=1e-4)
    for row in (1, 3, 5):
        assert np.all(np.isnan(got[row])) and np.all(np.isnan(qg[row]))
    before = out.clone()
    assert lib.nmmc_measure_static(s.h, C.c_void_p(idx.data_ptr()), 0, C.c_void_p(out.data_ptr()), None) == 0
    s.synchronize()
    assert torch.equal(torch.nan_to_num(out, 7.0), torch.nan_to_num(before, 7.0))
    s.close()


def test_static_measure_rejects_oversized_requests():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    lib = L.load()
    # a 2-D lattice of edge 4 is one measurement block: 11 doubles of scratch per chain, and a
    # device list adds half a double per entry (groups of 64 entries)
    limit = L.STATIC_SCRATCH_DOUBLES // 11
    s, _ = pair("s", edge=4, ising=True, periodic=True, jfile="2d_nn.dat", T=[2.0] * (limit + 1))
    out = torch.zeros((limit + 1, L.OBS_N), dtype=torch.float64, device="cuda")
    rc = lib.nmmc_measure_static(s.h, None, limit + 1, C.c_void_p(out.data_ptr()), None)
    assert rc == L.ERR_ARG
    assert b"static scratch" in lib.nmmc_last_error()
    listed = limit
    while (listed + 63) // 64 * 32 + listed * 11 > L.STATIC_SCRATCH_DOUBLES:
        listed -= 1
    first = torch.arange(listed + 1, dtype=torch.int32, device="cuda")
    assert lib.nmmc_measure_static(s.h, C.c_void_p(first.data_ptr()), listed + 1, C.c_void_p(out.data_ptr()),
                                   None) == L.ERR_ARG
    assert lib.nmmc_measure_static(s.h, C.c_void_p(first.data_ptr()), listed, C.c_void_p(out.data_ptr()),
                                   None) == 0
    s.synchronize()
    assert np.all(np.isfinite(out[:listed].cpu().numpy()))
    s.close()
