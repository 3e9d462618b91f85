"""ORACLE — test infrastructure only.

FP64 numpy restatement of the warm-start generator's loss and gradients (libnmmc
nmmc_gen_*), used to check the GPU's forward and backward kernels. It rounds to BF16 at the
same points as the GPU (weights, and the ReLU outputs stored as activations) and keeps every
sum in FP64, so the comparison isolates the GPU's FP32 accumulation.

Network: 8 periodic 3x3 convolutions; channels 8 -> 48 -> ... -> 48 -> 4 (the 4th output is
a zero pad); ReLU between layers; spin = v / |v| over the first 3 outputs; loss = mean over
sites of |spin - x|^2. Parameters in layer order W[9][cin][cout] (tap = 3*(dy+1)+(dx+1)), b[cout].
"""
import numpy as np

LAYERS = [(8, 48)] + [(48, 48)] * 6 + [(48, 4)]


def bf16(a):
    """Round FP32 values to BF16 (nearest even), returned as float64."""
    a = np.asarray(a, np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(params):
    out, o = [], 0
    for cin, cout in LAYERS:
        n = 9 * cin * cout
        w = np.asarray(params[o:o + n], np.float64).reshape(9, cin, cout)
        o += n
        b = np.asarray(params[o:o + cout], np.float64)
        o += cout
        out.append((w, b))
    assert o == len(params)
    return out


def conv(x, w):
    """x [n, L, L, cin], w [9, cin, cout]: out[p] = sum_tap x[p + off(tap)] @ w[tap]."""
    out = 0.0
    for tap in range(9):
        dy, dx = tap // 3 - 1, tap % 3 - 1
        xs = np.roll(x, shift=(-dy, -dx), axis=(1, 2))      # xs[p] = x[p + (dy, dx)]
        out = out + xs @ w[tap]
    return out


def conv_t(g, w):
    """Adjoint of conv: dx[q] = sum_tap g[q - off(tap)] @ w[tap].T."""
    out = 0.0
    for tap in range(9):
        dy, dx = tap // 3 - 1, tap % 3 - 1
        gs = np.roll(g, shift=(dy, dx), axis=(1, 2))
        out = out + gs @ w[tap].T
    return out


def wgrad(x, g):
    """dW[tap] = sum_p x[p + off(tap)]^T g[p]."""
    cin, cout = x.shape[-1], g.shape[-1]
    dw = np.zeros((9, cin, cout))
    for tap in range(9):
        dy, dx = tap // 3 - 1, tap % 3 - 1
        xs = np.roll(x, shift=(-dy, -dx), axis=(1, 2))
        dw[tap] = xs.reshape(-1, cin).T @ g.reshape(-1, cout)
    return dw


def loss_and_grads(params, inp, target, round_bf16=True):
    """inp [n, L, L, 8] (already BF16 values), target [n, L, L, 3]. Returns (loss, grads).
    round_bf16=False keeps every value in FP64 (finite-difference checks of this code)."""
    rnd = bf16 if round_bf16 else (lambda a: np.asarray(a, np.float64))
    layers = unpack(params)
    acts = [np.asarray(inp, np.float64)]
    for i, (w, b) in enumerate(layers):
        z = conv(acts[-1], rnd(w)) + b
        if i < len(layers) - 1:
            acts.append(rnd(np.maximum(z, 0.0)))
        else:
            v = z
    s3 = v[..., :3]
    norm = np.sqrt((s3 ** 2).sum(-1, keepdims=True) + 1e-12)
    s = s3 / norm
    npix = s.shape[0] * s.shape[1] * s.shape[2]
    d = s - target
    loss = (d ** 2).sum() / npix
    g = 2.0 * d / npix
    gv3 = (g - s * (s * g).sum(-1, keepdims=True)) / norm
    gv = np.zeros_like(v)
    gv[..., :3] = gv3
    grads = [None] * len(layers)
    cur = gv
    for i in range(len(layers) - 1, -1, -1):
        w, b = layers[i]
        grads[i] = (wgrad(acts[i], cur), cur.sum(axis=(0, 1, 2)))
        if i > 0:
            cur = conv_t(cur, rnd(w)) * (acts[i] > 0)
    flat = np.concatenate([np.concatenate([gw.ravel(), gb]) for gw, gb in grads])
    return loss, flat
