"""Learned warm start on the GPU: the generator's forward/backward against the FP64 oracle
(oracle/gen_oracle.py), training, and what a trained generator gains over random starts."""
import numpy as np
import pytest

from oracle import gen_oracle as G

pytestmark = pytest.mark.gpu


def small_dataset(L=16, n=4, D=0.5):
    from nanomagmc_gb300.warmstart import Generator, heisenberg_sampler
    gen = Generator(L, capacity=n, seed=5)
    T = np.linspace(0.3, 1.2, n)
    B = np.linspace(0.0, 0.3, n)
    s = heisenberg_sampler(L, D, T, B, seed=3)
    s.sweep(50)
    cond = np.stack([T, B, np.full(n, D)], 1)
    gen.add_snapshots(s, np.arange(n), cond)
    spins = np.stack([s.get_spins(c) for c in range(n)]).reshape(n, L, L, 3)
    s.close()
    return gen, spins, cond


@pytest.mark.parametrize("tensor", [1, 2, 0], ids=["tcgen05", "tcgen05-ws", "fma"])
@pytest.mark.parametrize("layer", [1, 4, 6])
def test_hidden_convolution_matches_fp64(tensor, layer):
    """One hidden layer (48 -> 48, 3x3 periodic) of BF16 data against an FP64 convolution of
    the same BF16 operands: every output within 1e-5 of the sum of its terms' magnitudes."""
    from nanomagmc_gb300.warmstart import Generator
    L, n = 32, 3
    gen = Generator(L, 0, seed=4)
    rng = np.random.default_rng(layer)
    x = G.bf16(np.maximum(rng.normal(size=(n, L, L, 48)), 0).astype(np.float32))
    w, b = G.unpack(gen.params().astype(np.float64))[layer]
    wb = G.bf16(w)
    ref = G.conv(x, wb) + b
    mag = G.conv(np.abs(x), np.abs(wb)) + np.abs(b)
    gen.tensor_cores(tensor)
    got = gen.probe_conv(layer, x, tensor != 0)
    assert np.all(np.abs(got - ref) <= 1e-5 * mag + 1e-30), np.max(np.abs(got - ref) / mag)
    gen.close()


@pytest.mark.parametrize("tensor", [1, 3, 4], ids=["tma", "cp-async", "tma-ws"])
def test_hidden_convolution_l128_matches_fp64(tensor):
    """At L = 128 a tile is one image row whose window TMA stages (periodic x edges copied in
    shared memory): option 1 in the single-role kernel, 4 in the warp-specialised kernel (ring
    of windows, two TMEM accumulators), 3 with cp.async staging. Each against an FP64
    convolution of the same BF16 operands as above, and bit for bit against the cp.async
    kernel (same MMAs in the same order)."""
    from nanomagmc_gb300.warmstart import Generator
    L, n = 128, 2
    gen = Generator(L, 0, seed=4)
    rng = np.random.default_rng(11)
    x = G.bf16(np.maximum(rng.normal(size=(n, L, L, 48)), 0).astype(np.float32))
    w, b = G.unpack(gen.params().astype(np.float64))[3]
    wb = G.bf16(w)
    ref = G.conv(x, wb) + b
    mag = G.conv(np.abs(x), np.abs(wb)) + np.abs(b)
    gen.tensor_cores(tensor)
    got = gen.probe_conv(3, x, True)
    assert np.all(np.abs(got - ref) <= 1e-5 * mag + 1e-30), np.max(np.abs(got - ref) / mag)
    gen.tensor_cores(1 if tensor == 3 else 3)
    assert np.array_equal(gen.probe_conv(3, x, True), got)
    gen.close()


@pytest.mark.parametrize("layer", [0, 7])
@pytest.mark.parametrize("L_edge", [128, 32])
def test_first_and_last_layers_match_fp64(layer, L_edge):
    """The first (8 -> 48) and last (48 -> 4) convolutions: on the tensor cores at L = 128 (K
    padded with a zero chunk for the 8 inputs; N = 16 for the 4 outputs), on the FMA pipes
    otherwise; against an FP64 convolution of the same BF16 operands, to 1e-5 of the sum of
    the terms' magnitudes."""
    from nanomagmc_gb300.warmstart import Generator
    n = 2
    gen = Generator(L_edge, 0, seed=4)
    rng = np.random.default_rng(layer + 3)
    cin = 8 if layer == 0 else 48
    x = G.bf16(rng.normal(size=(n, L_edge, L_edge, cin)).astype(np.float32))
    if layer:
        x = np.maximum(x, 0)
    w, b = G.unpack(gen.params().astype(np.float64))[layer]
    wb = G.bf16(w)
    ref = G.conv(x, wb) + b
    mag = G.conv(np.abs(x), np.abs(wb)) + np.abs(b)
    for tensor in (1, 0):
        got = gen.probe_conv(layer, x, tensor)
        assert got.shape == ref.shape
        assert np.all(np.abs(got - ref) <= 1e-5 * mag + 1e-30), (tensor, np.max(np.abs(got - ref) / mag))
    gen.close()


def test_l128_training_gradients_same_for_every_window_staging():
    """Forward (BF16) and data-gradient (TF32) convolutions of a training step at L = 128: the
    warp-specialised and single-role TMA kernels give identical loss and gradients; with
    cp.async staging (the first and last layers then on the FMA pipes) the loss agrees to FP32
    rounding and the gradients to the tensor-core bar of test_gradients_match_oracle."""
    res = []
    for tensor in (1, 4, 3):
        gen, _, _ = small_dataset(L=128, n=2)
        gen.tensor_cores(tensor)
        loss = gen.train_step(np.array([0, 1], np.int32), np.array([0.4, 0.7], np.float32), lr=0.0)
        res.append((loss, gen.grads().astype(np.float64)))
        gen.close()
    assert res[1][0] == res[0][0]
    assert np.array_equal(res[1][1], res[0][1])
    assert res[2][0] == pytest.approx(res[0][0], rel=1e-4)
    err = np.linalg.norm(res[2][1] - res[0][1]) / np.linalg.norm(res[0][1])
    assert err < 3e-2, err


def test_l128_two_row_tiles_identical():
    """The TMA-staged forward convolutions at L = 128 take tiles of two output rows (a window of
    four input rows, two TMEM accumulators) and their weights as one bulk copy of an operand
    image by default: each row gets the same MMAs on the same operands in the same order as
    with one-row tiles or thread-staged weights, so every layer's output, a training step's
    loss and gradients and a warm start are identical."""
    from nanomagmc_gb300.warmstart import Generator, heisenberg_sampler
    outs = []
    for rows, image in ((2, 1), (1, 1), (2, 0)):
        gen, _, _ = small_dataset(L=128, n=2)
        gen.tile_rows(rows)
        gen.weight_image(image)
        conv = []
        for layer, cin in ((0, 8), (3, 48), (7, 48)):
            x = G.bf16(np.maximum(np.random.default_rng(layer).normal(size=(2, 128, 128, cin)), 0).astype(np.float32))
            conv.append(gen.probe_conv(layer, x, True))
        loss = gen.train_step(np.array([0, 1], np.int32), np.array([0.4, 0.7], np.float32), lr=0.0)
        s = heisenberg_sampler(128, 0.5, [0.6, 0.9], [0.25, 0.0], seed=3)
        gen.warm_start(s, [0, 1], [[0.6, 0.25, 0.5], [0.9, 0.0, 0.5]], steps=4)
        outs.append((conv, loss, gen.grads(), [s.get_spins(c) for c in range(2)]))
        s.close()
        gen.close()
    for other in outs[1:]:
        for a, b in zip(outs[0][0], other[0]):
            assert np.array_equal(a, b)
        assert outs[0][1] == other[1]
        assert np.array_equal(outs[0][2], other[2])
        for a, b in zip(outs[0][3], other[3]):
            assert np.array_equal(a, b)


@pytest.mark.parametrize("tensor", [1, 2, 0], ids=["tcgen05", "tcgen05-ws", "fma"])
def test_gradients_match_oracle(tensor):
    """End to end against the FP64 oracle with the GPU's BF16 rounding points. The oracle's
    FP64 sums and the GPU's FP32 sums round a few activations to neighbouring BF16 values;
    at random initialisation the v/|v| head amplifies such flips, so the per-layer gradient
    error measures the accumulation order rather than the kernels (the FMA path shows 4e-3 on
    a 32x32 batch). Bars: 5e-3 for the FMA path, 3e-2 for the tensor-core path, whose FP32
    accumulation differs more from sequential FMA; the kernels themselves are checked to 1e-5
    by test_hidden_convolution_matches_fp64."""
    gen, spins, _ = small_dataset()
    gen.tensor_cores(tensor)
    idx = np.array([0, 3], np.int32)
    sig = np.array([0.3, 0.8], np.float32)
    loss = gen.train_step(idx, sig, lr=0.0)          # loss and gradients only
    g_gpu = gen.grads().astype(np.float64)
    inp = gen.last_input(2).astype(np.float64)
    target = G.bf16(spins[idx].astype(np.float32))   # the dataset stores BF16 snapshots
    p = gen.params().astype(np.float64)
    loss_ref, g_ref = G.loss_and_grads(p, inp, target)
    assert loss == pytest.approx(loss_ref, rel=2e-4)
    # per layer: relative L2 error of the gradient (FP32 accumulation vs FP64)
    o = 0
    for cin, cout in G.LAYERS:
        n = 9 * cin * cout + cout
        a, b = g_gpu[o:o + n], g_ref[o:o + n]
        o += n
        err = np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30)
        assert err < (3e-2 if tensor else 5e-3), (cin, cout, err)
    gen.close()


def test_training_step_lowers_the_loss_and_round_trips(tmp_path):
    gen, _, _ = small_dataset()
    rng = np.random.default_rng(0)
    idx = np.array([0, 1, 2, 3], np.int32)
    sig = np.array([0.5, 0.5, 0.5, 0.5], np.float32)
    l0 = gen.train_step(idx, sig, lr=0.0)
    for _ in range(60):
        gen.train_step(rng.integers(0, 4, 4), np.full(4, 0.5, np.float32), lr=3e-3)
    l1 = gen.train_step(idx, sig, lr=0.0)
    assert l1 < 0.7 * l0, (l0, l1)
    p = gen.params()
    path = str(tmp_path / "gen.bin")
    gen.save(path)
    gen2 = type(gen)(16, 0, seed=99)
    assert not np.array_equal(gen2.params(), p)
    gen2.load(path)
    assert np.array_equal(gen2.params(), p)
    gen.close()
    gen2.close()


def test_equilibrium_test_and_reference_check():
    """The equilibrium test of the sweeps-to-equilibrium figure: long chains already in
    equilibrium meet it at once with sigma = one chain's equilibrium spread; random spins do
    not (their energy is far from the equilibrium value); relaxation() resolves every sweep up
    to `fine`. checked_reference finds a paramagnetic point converged from the random and the
    ordered start."""
    from nanomagmc_gb300 import warmstart as W
    L, D, T, B, n = 32, 0.5, 1.5, 0.2, 16
    ref, info = W.checked_reference(L, T, B, D, n, eq_sweeps=2000, nsamp=100, gap=5, every=10)
    assert info["converged"]
    assert info["control_t_eq"]["spread"] == 0
    s = W.heisenberg_sampler(L, D, [T] * n, [B] * n, seed=5)
    rel = W.relaxation(s, np.arange(n), 200, every=10, fine=20)
    assert list(rel.t[:21]) == list(range(21)) and list(rel.t[21:]) == list(range(30, 201, 10))
    assert abs(rel.E[0] - ref["E"][0]) > ref["E"][1]   # random spins: far from equilibrium
    teq = W.sweeps_to_equilibrium(rel, ref, n)
    assert teq is not None and 0 < teq <= 200
    s.close()


def test_warm_start_writes_unit_spins():
    from nanomagmc_gb300 import _lib as L
    from nanomagmc_gb300.warmstart import Generator, heisenberg_sampler
    gen = Generator(32, 0, seed=2)
    s = heisenberg_sampler(32, 0.5, [0.3, 0.6], [0.1, 0.2])
    for mode in (0, 1, 2):   # fresh noise, DDIM-style, DDPM-style passes
        gen.warm_start(s, [0, 1], [[0.3, 0.1, 0.5], [0.6, 0.2, 0.5]], steps=3, reuse_noise=mode)
        for c in range(2):
            n = np.linalg.norm(s.get_spins(c), axis=1)
            assert np.allclose(n, 1.0, atol=1e-5)
    for sched in (1, 2, 0):   # quadratic and cosine noise levels
        gen.schedule(sched)
        gen.warm_start(s, [0, 1], [[0.3, 0.1, 0.5], [0.6, 0.2, 0.5]], steps=3)
        for c in range(2):
            assert np.allclose(np.linalg.norm(s.get_spins(c), axis=1), 1.0, atol=1e-5)
    with pytest.raises(L.NmmcError):
        gen.schedule(3)
    s.sweep(5)
    s.close()
    gen.close()


def _deviation(rel, ref, n):
    """Mean over the relaxation of |observable - long-chain mean| in units of the n-chain
    standard error, summed over E, |M| and Q."""
    tot = 0.0
    for k, series in (("E", rel.E), ("M", rel.M), ("Q", rel.Q)):
        mean, sd = ref[k][:2]
        tot += float(np.mean(np.abs(series - mean)) / (sd / np.sqrt(n)))
    return tot


def test_trained_generator_gains_over_random_starts():
    """L = 32, D = 0.5: a generator trained for 3000 steps on 3840 snapshots of the plain
    sampler starts 32 chains at (T, B) = (0.6, 0.1), with 128 DDPM-style passes, closer to
    equilibrium than random spins:
    the mean deviation of E, |M|, Q from long plain chains over the first 500 sweeps is at
    least 30 % below that of random starts (about half in the runs recorded); the 3-sigma gate
    keeps the learned start, and an untrained generator's start is rejected and replaced by
    random spins."""
    from nanomagmc_gb300 import warmstart as W
    L, D, T, B, M = 32, 0.5, 0.6, 0.1, 32
    gen = W.Generator(L, capacity=4096, seed=1)
    pts = [(t, b, D) for t in (0.15, 0.3, 0.45, 0.6, 0.9) for b in (0.0, 0.1, 0.2, 0.3)]
    W.make_dataset(gen, pts, replicas=8, eq_sweeps=8000, snap_every=50, snaps=24)
    hist = W.train(gen, 3000, batch=32, lr=2e-3)
    assert hist[-50:].mean() < 0.5 * hist[:50].mean()
    ref_s = W.heisenberg_sampler(L, D, [T] * M, [B] * M, seed=77)
    ref = W.reference(ref_s, np.arange(M), 16000, 400)
    rnd = W.heisenberg_sampler(L, D, [T] * M, [B] * M, seed=78)
    r_rel = W.relaxation(rnd, np.arange(M), 500, every=5)
    lrn = W.heisenberg_sampler(L, D, [T] * M, [B] * M, seed=79)
    gen.warm_start(lrn, np.arange(M), np.tile([T, B, D], (M, 1)), steps=128)
    l_rel = W.relaxation(lrn, np.arange(M), 500, every=5)
    dev_r, dev_l = _deviation(r_rel, ref, M), _deviation(l_rel, ref, M)
    assert dev_l < 0.7 * dev_r, (dev_l, dev_r)
    # the gate judges the learned start with the plain chain and keeps it
    g = W.heisenberg_sampler(L, D, [T] * M, [B] * M, seed=80)
    assert W.gated_warm_start(gen, g, np.arange(M), np.tile([T, B, D], (M, 1)), ref, steps=128,
                              check_sweeps=500)
    # an untrained generator's start, judged before any sweep, falls back to random spins
    raw = W.Generator(L, 0, seed=3)
    f = W.heisenberg_sampler(L, D, [T] * M, [B] * M, seed=81)
    assert not W.gated_warm_start(raw, f, np.arange(M), np.tile([T, B, D], (M, 1)), ref, steps=128,
                                  check_sweeps=0, nsamp=5)
    obs = f.measure(with_q=False)
    assert np.all(np.abs(obs[:, 4] / f.box_sites) < 0.2)   # random spins: |M|/N ~ N^-1/2
    for s in (ref_s, rnd, lrn, g, f):
        s.close()
    gen.close()
    raw.close()


# ------------------------------------------------------------------------------------------
# the 3-sigma gate and random-start fallback through the C ABI, and nmmc_run's GENERATOR key
# ------------------------------------------------------------------------------------------
def _gate(gen, s, chains, cond, ref, check_sweeps=200, seed=5):
    import ctypes as C

    from nanomagmc_gb300 import _lib as L
    lib = L.load()
    ch = np.ascontiguousarray(chains, np.int32)
    cd = np.ascontiguousarray(cond, np.float64)
    kept = C.c_int(-1)
    r = None if ref is None else np.ascontiguousarray(ref, np.float64)
    L.check(lib.nmmc_gen_gated_warm_start(gen.h, s.h, ch.ctypes.data_as(C.c_void_p), len(ch),
                                          cd.ctypes.data_as(C.c_void_p), 8, check_sweeps, 40, 2,
                                          None if r is None else r.ctypes.data_as(C.c_void_p), seed, C.byref(kept)))
    return kept.value


def test_gated_warm_start_keeps_or_falls_back():
    """nmmc_reference_stats of long plain chains is the reference. At T = 1.5 (paramagnetic:
    200 check sweeps equilibrate any start) the learned start is kept; against a reference
    shifted by far more than its error it is rejected and the chains are back at uniform
    random spins (unit vectors, |M|/N near 0)."""
    import ctypes as C

    from nanomagmc_gb300 import _lib as L
    from nanomagmc_gb300.warmstart import heisenberg_sampler
    lib = L.load()
    gen, _, _ = small_dataset(L=16, n=4)
    for _ in range(50):
        gen.train_step(np.arange(4), np.full(4, 0.7, np.float32), 2e-3)
    n, T, B, D = 16, 1.5, 0.1, 0.5
    s = heisenberg_sampler(16, D, [T] * (2 * n), [B] * (2 * n), seed=21)
    ref = np.zeros(9)
    refc = np.arange(n, 2 * n, dtype=np.int32)
    L.check(lib.nmmc_reference_stats(s.h, refc.ctypes.data_as(C.c_void_p), n, 500, 200, 2,
                                     ref.ctypes.data_as(C.c_void_p)))
    assert np.all(np.isfinite(ref)) and np.all(ref[2::3] > 0)
    cond = np.tile([T, B, D], (n, 1))
    assert _gate(gen, s, np.arange(n), cond, ref) == 1
    bad = ref.copy()
    bad[0] += 100 * ref[1]                      # an energy no chain can reach
    assert _gate(gen, s, np.arange(n), cond, bad, check_sweeps=10) == 0
    for c in range(n):
        sp = s.get_spins(c)
        assert np.allclose(np.linalg.norm(sp, axis=1), 1.0, atol=1e-6)
        assert np.linalg.norm(sp.sum(0)) / len(sp) < 0.2
    # the drift form (no reference) runs and reports a decision
    assert _gate(gen, s, np.arange(n), cond, None) in (0, 1)
    s.close()
    gen.close()


def test_nmmc_run_with_a_generator(tmp_path):
    """nmmc_run with GENERATOR (WSSCHED 1: quadratic noise schedule): the base chains start from
    the gated learned warm start; the
    run completes with the output of a plain run's shapes, records its gate decision, and its
    samples agree with a plain run's (same model, many samples) within 4 sigma per point."""
    import os
    import shutil

    from nanomagmc_gb300 import _lib as L
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    gen, _, _ = small_dataset(L=16, n=4)
    for _ in range(50):
        gen.train_step(np.arange(4), np.full(4, 0.7, np.float32), 2e-3)
    runs = {}
    for name in ("plain", "learned"):
        wd = tmp_path / name
        for d in ("Temps", "Fields", "Js"):
            (wd / d).mkdir(parents=True)
        (wd / "Temps" / "t.dat").write_text("1.5 1.0\n")
        (wd / "Fields" / "h.dat").write_text("0.0 0.3\n")
        shutil.copy(os.path.join(root, "data", "Js", "2d_nn_interfacial.dat"), wd / "Js")
        text = ("ISISING 0\nEXCHANGE 1\nDMISTREN 0.5\nISDISTRIB 0\nSIZE 16\nMEANSIZE 16\nSIZEDEV 0\n"
                "LATTSHAPE s\nWEIBULLFACT 3\nNLATTS 2\nBOLTZMANN 1\nISPERIO 1\nSAMPSWEEPS 5\nEQSWEEPS 100\n"
                "NSAMPS 200\nTEMPNAME t.dat\nFIELDNAME h.dat\nPROTOCOL 1\nINTERACTIONS 2d_nn_interfacial.dat\n")
        if name == "learned":
            gen.save(str(wd / "gen.bin"))
            text += "GENERATOR gen.bin\nWSSTEPS 8\nWSSCHED 1\n"
        (wd / "INPUT.dat").write_text(text)
        lib = L.load()
        assert lib.nmmc_run(str(wd / "INPUT.dat").encode(), str(wd).encode(), str(wd / "out").encode(), 7, 0) == 0
        runs[name] = {k: np.load(wd / "out" / (k + ".npy")) for k in ("energies", "mags")}
        if name == "learned":
            ws = np.load(wd / "out" / "warm_start.npy")
            assert ws.shape == (2,) and ws[0] in (0, 1) and ws[1] == 8
    for k in ("energies", "mags"):
        a, b = runs["plain"][k].astype(float), runs["learned"][k].astype(float)
        assert a.shape == b.shape == (2, 2, 400)
        ma, mb = a.mean(-1), b.mean(-1)
        from stats import binned_error
        ea = np.array([[binned_error(a[i, j]) for j in range(2)] for i in range(2)])
        eb = np.array([[binned_error(b[i, j]) for j in range(2)] for i in range(2)])
        assert np.all(np.abs(ma - mb) <= 4 * np.hypot(ea, eb)), (k, ma, mb, ea, eb)
    gen.close()


@pytest.mark.parametrize("L_edge,nimg", [(16, 3), (128, 2)])
def test_weight_gradient_on_tensor_cores_matches_fp64(L_edge, nimg):
    """A hidden layer's weight gradient (sum over pixels of in[p + tap][ci] * dout[p][co]) on
    tcgen05 (BF16 operands: the BF16 inputs exactly, each FP32 gradient as BF16 hi + lo, which
    represents it to 2^-18 relative) against an FP64 sum of the same BF16 inputs and FP32
    gradients: every entry within 2e-5 of the sum of its terms' magnitudes (the split's
    2^-18 ~ 3.8e-6 plus FP32 accumulation); the FMA path within 1e-5 of it. L = 16 is one
    K-block per image row, L = 128 two."""
    import ctypes as C

    from nanomagmc_gb300 import _lib as L
    from nanomagmc_gb300.warmstart import Generator
    lib = L.load()
    gen = Generator(L_edge, 0, seed=4)
    rng = np.random.default_rng(L_edge)
    x = np.ascontiguousarray(G.bf16(np.maximum(rng.normal(size=(nimg, L_edge, L_edge, 48)), 0)), np.float32)
    d = np.ascontiguousarray(rng.normal(size=(nimg, L_edge, L_edge, 48)), np.float32)
    ref = np.zeros((9, 48, 48))
    mag = np.zeros((9, 48, 48))
    for tap in range(9):
        dy, dx = tap // 3 - 1, tap % 3 - 1
        xs = np.roll(x.astype(np.float64), shift=(-dy, -dx), axis=(1, 2))   # xs[p] = x[p + tap]
        ref[tap] = np.einsum("nyxc,nyxo->co", xs, d.astype(np.float64))
        mag[tap] = np.einsum("nyxc,nyxo->co", np.abs(xs), np.abs(d.astype(np.float64)))
    for tensor, tol in ((1, 2e-5), (0, 1e-5)):
        got = np.zeros((9, 48, 48), np.float32)
        L.check(lib.nmmc_gen_probe_wgrad(gen.h, nimg, x.ctypes.data_as(C.c_void_p), d.ctypes.data_as(C.c_void_p),
                                         got.ctypes.data_as(C.c_void_p), tensor))
        assert np.all(np.abs(got - ref) <= tol * mag + 1e-30), (tensor, np.max(np.abs(got - ref) / mag))
    gen.close()
