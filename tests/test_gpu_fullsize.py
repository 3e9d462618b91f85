"""Full-size parity: the benchmark configurations at their full lattice sizes, checked through
properties that do not depend on a CPU reference finishing at that size.

  * C4 (3-D Heisenberg L = 128, 40 chains): the four-sites-per-thread, one-site-per-thread and
    TMA-pipelined half-sweeps give the same chains bit for bit; spins stay unit vectors; the
    production FP32 observables agree with the FP64 per-site mode (E 1e-6 relative,
    magnetisations 1e-6 x N, total charge 1e-3).
  * C2 (2-D L = 64, 420 chains) and C3 (512 Weibull grains): the shared-memory resident path and
    the HBM path (filled-site lists for the grains) give the same chains bit for bit; the fused
    observables agree with the separate measurement to FP32 summation order.
  * C1 (2-D Ising L = 32, 13 temperatures): every chain equals the oracle's checkerboard
    restatement bit for bit.
  * x3 (96 3-D Weibull spheres of radius 30 in 90^3 boxes): sweeping the chains in two lists
    gives the chains of one call over all of them; sites outside each particle stay empty and
    the filled ones unit vectors; FP32 and FP64 observables agree.
"""
import numpy as np
import pytest

from nanomagmc_gb300 import _lib as L
from nanomagmc_gb300.sampler import Sampler, interactions_file, make_options, read_interactions

from helpers import STENCIL, oracle_from_gpu, pair

pytestmark = pytest.mark.gpu


def sampler(shape, edge=None, size=None, asd=0.0, ising=False, periodic=True, jfile="3d_nn_bloch.dat", D=0.0,
            T=(1.0,), H=0.0, sizes=None, seed=1):
    dim = 3 if shape in "cx" else 2
    opt = make_options(shape, edge=edge, size=size, ising=ising, periodic=periodic, J=1.0, D=D, weibull=3.0,
                       asd=asd)
    inter = read_interactions(interactions_file(jfile), dim, 1.0, D)
    return Sampler(opt, inter, T=np.asarray(T, float), H=H, sizes=sizes, seed=seed)


def fp32_vs_fp64(s, N):
    s.option(L.OPT_MEASURE_FP64, 1)
    o64, q64 = s.measure()
    s.option(L.OPT_MEASURE_FP64, 0)
    o32, q32 = s.measure()
    assert np.all(np.abs(o32[:, L.OBS_E] - o64[:, L.OBS_E]) <= 1e-6 * np.maximum(1.0, np.abs(o64[:, L.OBS_E])))
    assert np.max(np.abs(o32[:, 1:13] - o64[:, 1:13])) <= 1e-6 * N
    assert np.max(np.abs(np.nansum(q32, 1) - np.nansum(q64, 1))) <= 1e-3
    return o64


def test_c4_full_kernels_identical():
    T = np.linspace(0.2, 2.0, 40)
    picks = (0, 17, 39)
    ref = None
    for half, wave in ((0, 0), (1, 0), (3, 0), (0, 1), (8, 0)):
        s = sampler("c", edge=128, periodic=True, jfile="3d_nn_bloch.dat", D=0.3, T=T, H=0.2, seed=9)
        s.option(L.OPT_SWEEP_PATH, 1)
        s.option(L.OPT_HALF_KERNEL, half)
        s.option(L.OPT_WAVE, wave)
        s.sweep(4)
        s.sweep(2, [39, 3, 17])
        if ref is None:
            o64 = fp32_vs_fp64(s, 128 ** 3)
            ref = (o64, [s.get_spins(c) for c in picks])
            for sp in ref[1]:
                assert np.all(np.abs(np.linalg.norm(sp, axis=1) - 1.0) < 1e-6)
        else:
            s.option(L.OPT_MEASURE_FP64, 1)
            o64, _ = s.measure()
            assert np.array_equal(o64, ref[0]), half
            for c, sp in zip(picks, ref[1]):
                assert np.array_equal(s.get_spins(c), sp), (half, c)
        s.close()


def test_c4_fused_step_matches_separate():
    """The benchmark step (10 sweeps, then the observables) on 128^3 lattices: E, M, subM and
    sub4M summed inside the last colour-1 half-sweep and the charge pass give the observables of
    nmmc_measure on the same chain, to FP32 summation order."""
    T = np.linspace(0.2, 2.0, 4)
    a = sampler("c", edge=128, periodic=True, jfile="3d_nn_bloch.dat", D=0.3, T=T, H=0.2, seed=9)
    b = sampler("c", edge=128, periodic=True, jfile="3d_nn_bloch.dat", D=0.3, T=T, H=0.2, seed=9)
    for s in (a, b):
        s.option(L.OPT_SWEEP_PATH, 1)
    N = 128 ** 3
    for _ in range(2):
        oa, qa = a.sweep_measure(10, accumulate=True)
        b.sweep(10)
        ob, qb = b.measure(accumulate=True)
        assert np.all(np.abs(oa[:, L.OBS_E] - ob[:, L.OBS_E]) <= 1e-6 * np.abs(ob[:, L.OBS_E]))
        assert np.max(np.abs(oa[:, 1:13] - ob[:, 1:13])) <= 1e-6 * N
        assert np.allclose(qa, qb, rtol=0, atol=1e-4)   # the same angles in another FP32 order
    for c in range(4):
        assert np.array_equal(a.get_spins(c), b.get_spins(c))
    acc_a, acc_b = a.accumulators(), b.accumulators()
    assert np.allclose(acc_a, acc_b, rtol=1e-6, atol=0)
    a.close()
    b.close()


def test_c2_full_resident_equals_hbm():
    Tg, Bg = np.meshgrid(np.linspace(0.05, 1.5, 20), np.linspace(0.0, 1.0, 21))
    res = []
    for path in (2, 1):
        s = sampler("s", edge=64, periodic=True, jfile="2d_nn_interfacial.dat", D=0.5, T=Tg.ravel(), H=Bg.ravel(),
                    seed=3)
        s.option(L.OPT_SWEEP_PATH, path)
        s.sweep(5)
        fused, fq = s.sweep_measure(2, accumulate=True)
        sep, sq = s.measure()
        spins = np.stack([s.get_spins(c) for c in range(s.nchains)])
        res.append((spins, sep, sq))
        if path == 2:   # fused observables against the separate measurement: FP32 order only
            assert np.max(np.abs(fused[:, :13] - sep[:, :13])) <= 2e-6 * 4096 * 8
            assert np.allclose(fq, sq, rtol=0, atol=1e-4)
        s.close()
    assert np.array_equal(res[0][0], res[1][0])
    assert np.array_equal(res[0][1], res[1][1]) and np.array_equal(res[0][2], res[1][2])


def test_c3_full_resident_equals_hbm_lists():
    Tg, Bg = np.meshgrid(np.linspace(0.05, 1.5, 32), np.linspace(0.0, 1.0, 16))
    am, sd = 20.0, 5.0
    lm, ls = np.log(am * am / np.sqrt(sd * sd + am * am)), np.sqrt(np.log(1 + sd * sd / (am * am)))
    sizes = [L.load().nmmc_lognormal_size(7, k, lm, ls) for k in range(512)]
    res = []
    for path in (2, 1):
        s = sampler("w", size=am, asd=sd, periodic=False, jfile="2d_nn_interfacial.dat", D=0.5, T=Tg.ravel(),
                    H=Bg.ravel(), sizes=sizes, seed=5)
        assert s.edge == 90
        s.option(L.OPT_SWEEP_PATH, path)
        s.sweep(5)
        s.sweep(3, list(range(511, -1, -3)))
        obs, q = s.measure()
        spins = np.stack([s.get_spins(c) for c in range(s.nchains)])
        masks = np.stack([s.mask(c) for c in range(s.nchains)])
        if path == 1:
            assert np.all(spins[masks == 0] == 0)
            assert np.all(np.abs(np.linalg.norm(spins[masks == 1], axis=1) - 1.0) < 1e-6)
            fp32_vs_fp64(s, 4600)
        res.append((spins, obs, q))
        s.close()
    assert np.array_equal(res[0][0], res[1][0])
    assert np.array_equal(res[0][1], res[1][1]) and np.array_equal(res[0][2], res[1][2])


def test_c1_full_matches_oracle_checkerboard():
    T = np.linspace(2.0, 2.6, 13)
    seed = 0xC1C1
    s, ors = pair("s", edge=32, ising=True, periodic=True, jfile="2d_nn.dat", D=0.0, T=T, H=0.0, seed=seed)
    boxes = [oracle_from_gpu(s, o, c) for c, o in enumerate(ors)]
    s.sweep(10)
    s.sweep_measure(15)
    dirs = STENCIL[:4]
    Jdir = np.ones(4, np.float32)
    for c, (o, box) in enumerate(zip(ors, boxes)):
        o.set_beta(1.0 / T[c])
        o.cb_ising(seed, c, 0, 25, Jdir, dirs, hx=0.0)
        assert np.array_equal(s.get_spins(c)[box][:, 0], o.spins()[:, 0]), c
    s.close()


def test_x3_full_chain_lists_and_invariants():
    T = np.linspace(0.2, 2.0, 96)
    outs = []
    for split in (False, True):
        s = sampler("x", edge=90, size=30.0, periodic=False, jfile="3d_nn_bloch.dat", D=0.3, T=T, H=0.2, seed=2)
        if split:
            s.sweep(3, list(range(0, 96, 2)))
            s.sweep(3, list(range(1, 96, 2)))
        else:
            s.sweep(3)
        s.option(L.OPT_MEASURE_FP64, 1)
        o64, q64 = s.measure()
        s.option(L.OPT_MEASURE_FP64, 0)
        outs.append((o64, q64, [s.get_spins(c) for c in (0, 50, 95)]))
        if not split:
            for c in (0, 50, 95):
                sp, mk = s.get_spins(c), s.mask(c)
                assert np.all(sp[mk == 0] == 0)
                assert np.all(np.abs(np.linalg.norm(sp[mk == 1], axis=1) - 1.0) < 1e-6)
            fp32_vs_fp64(s, 2e5)
        s.close()
    assert np.array_equal(outs[0][0], outs[1][0]) and np.array_equal(outs[0][1], outs[1][1], equal_nan=True)
    for a, b in zip(outs[0][2], outs[1][2]):
        assert np.array_equal(a, b)
