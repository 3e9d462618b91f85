"""The generator oracle (oracle/gen_oracle.py) is pinned by central finite differences in
FP64 and by the adjoint identity of its convolution; the GPU gradients are then checked
against it (tests/test_gpu_gen.py)."""
import numpy as np

from oracle import gen_oracle as G


def random_params(rng, scale=0.15):
    n = sum(9 * ci * co + co for ci, co in G.LAYERS)
    p = rng.normal(scale=scale, size=n)
    # the pad output channel stays zero, as on the GPU
    o = 0
    for ci, co in G.LAYERS:
        w = p[o:o + 9 * ci * co].reshape(9, ci, co)
        if co == 4:
            w[..., 3] = 0
        o += 9 * ci * co
        if co == 4:
            p[o + 3] = 0
        o += co
    return p


def test_conv_adjoint():
    rng = np.random.default_rng(0)
    x = rng.normal(size=(2, 5, 5, 3))
    g = rng.normal(size=(2, 5, 5, 4))
    w = rng.normal(size=(9, 3, 4))
    assert np.isclose((G.conv(x, w) * g).sum(), (x * G.conv_t(g, w)).sum())
    # wgrad is the derivative of <conv(x, w), g> in w
    assert np.isclose((G.wgrad(x, g) * w).sum(), (G.conv(x, w) * g).sum())


def test_gradients_by_finite_differences():
    rng = np.random.default_rng(1)
    p = random_params(rng)
    inp = rng.normal(size=(1, 4, 4, 8))
    t = rng.normal(size=(1, 4, 4, 3))
    t /= np.linalg.norm(t, axis=-1, keepdims=True)
    loss, g = G.loss_and_grads(p, inp, t, round_bf16=False)
    idx = rng.choice(len(p), size=25, replace=False)
    # include some last-layer and bias entries
    idx = np.concatenate([idx, [len(p) - 5, len(p) - 2, 100]])
    h = 1e-6
    for i in idx:
        q = p.copy()
        q[i] += h
        lp, _ = G.loss_and_grads(q, inp, t, round_bf16=False)
        q[i] -= 2 * h
        lm, _ = G.loss_and_grads(q, inp, t, round_bf16=False)
        fd = (lp - lm) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 + 1e-4 * abs(g[i]), (i, fd, g[i])


def test_bf16_rounding():
    x = np.array([1.0, 1.00390625, 1.0078125, 3.14159265, -2.5e-3], np.float32)
    r = G.bf16(x)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0078125   # ties to even
    assert abs(r[3] - 3.140625) < 1e-9
