"""Learned warm starts for 2-D Heisenberg + DMI lattices, on top of libnmmc's C ABI.

The plain Metropolis sampler produces equilibrium snapshots over a (T, B, D) grid; a
conditional convolutional generator (nmmc_gen_*, trained on the GPU by the library's own
BF16/FP32 kernels) learns to turn a random start into an equilibrium-like configuration; the
Metropolis chain then does all sampling. A warm start is accepted only if the chain's
observables from it agree with long plain chains within 3 sigma; otherwise the chains are
restarted from random spins (`gated_warm_start`).

This module has no reference counterpart; it sits beside the plain method (the reference's
random start, Old/lib/field_type.cpp:197-204), not in place of it.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib as L
from .sampler import Sampler, interactions_file, make_options, read_interactions


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


class Generator:
    """nmmc_gen: an 8-layer, 48-channel periodic conv generator for L x L lattices."""

    def __init__(self, L_edge: int, capacity: int = 0, seed: int = 1):
        self.lib = L.load()
        h = C.c_void_p()
        L.check(self.lib.nmmc_gen_create(L_edge, capacity, seed, C.byref(h)))
        self.h = h
        self.L = L_edge
        self.nparams = self.lib.nmmc_gen_param_count(self.h)

    def close(self):
        if getattr(self, "h", None):
            self.lib.nmmc_gen_destroy(self.h)
            self.h = None

    def probe_conv(self, layer, x, tensor=True):
        """One layer's conv + bias of x [n][L][L][cin] (FP32 out [n][L][L][cout], no activation):
        layer 0 is 8 -> 48 channels, 1..6 48 -> 48, 7 48 -> 4."""
        x = np.ascontiguousarray(x, np.float32)
        cout = 4 if layer == 7 else 48
        out = np.zeros(x.shape[:-1] + (cout,), np.float32)
        L.check(self.lib.nmmc_gen_probe_conv(self.h, layer, x.shape[0], _p(x), _p(out), int(bool(tensor))))
        return out

    def tensor_cores(self, mode):
        """Hidden convolutions: 1 / True tensor cores (default; TMA-staged windows at L = 128),
        2 warp-specialised forward with cp.async staging, 3 cp.async staging at every L,
        4 warp-specialised forward with TMA staging (L = 128), 0 / False FP32 FMA pipes."""
        L.check(self.lib.nmmc_gen_set_option(self.h, L.GEN_OPT_TENSOR_CORES, int(mode)))

    def tile_rows(self, rows):
        """Output rows per tile of the TMA-staged forward convolutions at L = 128 (1 or 2)."""
        L.check(self.lib.nmmc_gen_set_option(self.h, L.GEN_OPT_TILE_ROWS, int(rows)))

    def schedule(self, kind):
        """Noise levels of the warm-start passes: 0 linear, 1 quadratic, 2 cosine."""
        L.check(self.lib.nmmc_gen_set_option(self.h, L.GEN_OPT_SCHEDULE, int(kind)))

    def weight_image(self, on):
        """TMA-staged forward convolutions: weights by one bulk copy of their operand image."""
        L.check(self.lib.nmmc_gen_set_option(self.h, L.GEN_OPT_WEIGHT_IMAGE, int(bool(on))))

    def __del__(self):
        self.close()

    @property
    def size(self):
        return self.lib.nmmc_gen_dataset_size(self.h)

    def params(self):
        p = np.zeros(self.nparams, np.float32)
        L.check(self.lib.nmmc_gen_get_params(self.h, _p(p), self.nparams))
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, np.float32)
        L.check(self.lib.nmmc_gen_set_params(self.h, _p(p), self.nparams))

    def grads(self):
        g = np.zeros(self.nparams, np.float32)
        L.check(self.lib.nmmc_gen_get_grads(self.h, _p(g), self.nparams))
        return g

    def last_input(self, nb):
        x = np.zeros((nb, self.L, self.L, 8), np.float32)
        L.check(self.lib.nmmc_gen_get_input(self.h, nb, _p(x)))
        return x

    def add_snapshots(self, sampler: Sampler, chains, cond):
        ch = np.ascontiguousarray(chains, np.int32)
        cd = np.ascontiguousarray(cond, np.float64).reshape(len(ch), 3)
        L.check(self.lib.nmmc_gen_add_snapshots(self.h, sampler.h, _p(ch), len(ch), _p(cd)))

    def train_step(self, idx, sig, lr):
        idx = np.ascontiguousarray(idx, np.int32)
        sig = np.ascontiguousarray(sig, np.float32)
        loss = C.c_double()
        L.check(self.lib.nmmc_gen_train_step(self.h, _p(idx), _p(sig), len(idx), float(lr), C.byref(loss)))
        return loss.value

    def warm_start(self, sampler: Sampler, chains, cond, steps=256, reuse_noise=2):
        """`steps` denoising passes; reuse_noise: 0 fresh noise between passes, 1 DDIM-style,
        2 (default) the DDPM-style posterior step, which keeps the skyrmion statistics."""
        ch = np.ascontiguousarray(chains, np.int32)
        cd = np.ascontiguousarray(cond, np.float64).reshape(len(ch), 3)
        L.check(self.lib.nmmc_gen_warm_start(self.h, sampler.h, _p(ch), len(ch), _p(cd), int(steps),
                                             int(reuse_noise)))

    def save(self, path):
        L.check(self.lib.nmmc_gen_save(self.h, path.encode()))

    def load(self, path):
        L.check(self.lib.nmmc_gen_load(self.h, path.encode()))


def heisenberg_sampler(L_edge, D, T, B, seed=1, periodic=True):
    """2-D Heisenberg lattice with interfacial DMI of strength D (Js/2d_nn_interfacial.dat)."""
    opt = make_options("s", edge=L_edge, periodic=periodic, J=1.0, D=D)
    inter = read_interactions(interactions_file("2d_nn_interfacial.dat"), 2, 1.0, D)
    return Sampler(opt, inter, T=np.asarray(T, float), H=np.asarray(B, float), seed=seed)


def make_dataset(gen: Generator, points, replicas=4, eq_sweeps=4000, snap_every=50, snaps=8, seed=11):
    """Equilibrium snapshots from the plain sampler: for every (T, B, D) point, `replicas`
    chains equilibrated for eq_sweeps, then `snaps` snapshots snap_every sweeps apart."""
    points = np.asarray(points, float).reshape(-1, 3)
    for D in np.unique(points[:, 2]):
        sel = points[points[:, 2] == D]
        T = np.repeat(sel[:, 0], replicas)
        B = np.repeat(sel[:, 1], replicas)
        s = heisenberg_sampler(gen.L, D, T, B, seed=seed + int(1000 * D))
        s.sweep(eq_sweeps)
        cond = np.stack([T, B, np.full_like(T, D)], 1)
        chains = np.arange(len(T))
        for _ in range(snaps):
            s.sweep(snap_every)
            gen.add_snapshots(s, chains, cond)
        s.close()
    return gen.size


def train(gen: Generator, steps, batch=16, lr=2e-3, seed=0, lr_end=2e-4):
    """Adam on the denoising loss; noise levels favour s near 1 (the warm-start input)."""
    rng = np.random.default_rng(seed)
    hist = []
    for k in range(steps):
        idx = rng.integers(0, gen.size, size=batch)
        sig = np.clip(np.sqrt(rng.uniform(0.0, 1.0, size=batch)), 0.02, 1.0)
        a = k / max(1, steps - 1)
        hist.append(gen.train_step(idx, sig, lr * (lr_end / lr) ** a))
    return np.array(hist)


@dataclass
class Relaxation:
    """Chain-averaged E/N, |M|/N and Q, measured after t[i] sweeps (t None: i * every)."""
    E: np.ndarray
    M: np.ndarray
    Q: np.ndarray
    t: np.ndarray = None


def relaxation(sampler: Sampler, chains, tmax, every=1, fine=0):
    """The chains' mean observables while they relax: after every sweep up to `fine` sweeps
    (so that starts which equilibrate in a few sweeps are resolved), then every `every` sweeps
    up to tmax."""
    E, M, Q, T = [], [], [], []
    N = sampler.box_sites
    fine = min(fine, tmax)
    times = list(range(0, fine + 1)) + list(range(fine + every, tmax + 1, every))
    done = 0
    for t in times:
        if t > done:
            sampler.sweep(t - done, chains)
            done = t
        obs = sampler.measure(chains, with_q=False)
        E.append(obs[:, L.OBS_E].mean() / N)
        M.append(obs[:, L.OBS_ABSM].mean() / N)
        Q.append(obs[:, L.OBS_QTOT].mean())
        T.append(t)
    return Relaxation(np.array(E), np.array(M), np.array(Q), np.array(T))


def _chain_stats(v):
    """v[sample, chain]: the grand mean and its standard error from the independent per-chain
    time averages (the chains share nothing, so autocorrelation within a chain is absorbed)."""
    m = v.mean(0)
    return float(m.mean()), float(m.std(ddof=1) / np.sqrt(len(m))) if len(m) > 1 else float("inf")


def reference_samples(sampler: Sampler, chains, eq_sweeps, nsamp, gap=5):
    """Long plain chains: eq_sweeps sweeps, then nsamp samples gap sweeps apart of E/N, |M|/N
    and Q, as an array [nsamp, chains, 3]."""
    sampler.sweep(eq_sweeps, chains)
    N = sampler.box_sites
    obs = sampler.sample(gap, nsamp, chains)          # [nsamp, n, OBS]
    return np.stack([obs[..., L.OBS_E] / N, obs[..., L.OBS_ABSM] / N, obs[..., L.OBS_QTOT]], -1)


def reference_stats(v):
    """For E/N, |M|/N and Q of samples v [nsamp, chains, 3]: the mean, the standard deviation of
    one chain's instantaneous value and the standard error of the mean (from the per-chain
    averages)."""
    return {k: (float(v[..., i].mean()), float(v[..., i].std(ddof=1)), _chain_stats(v[..., i])[1])
            for i, k in enumerate("EMQ")}


def reference(sampler: Sampler, chains, eq_sweeps, nsamp, gap=5):
    """Long plain chains: for E/N, |M|/N and Q the mean, the standard deviation of one chain's
    instantaneous value and the standard error of the mean (from the per-chain averages)."""
    return reference_stats(reference_samples(sampler, chains, eq_sweeps, nsamp, gap))


def sweeps_to_equilibrium(rel: Relaxation, ref, nchains, every=1, window=5, tol="spread"):
    """First sweep t after which, for `window` consecutive measurements, the nchains-averaged
    E, |M| and Q all lie within 1 sigma of the long-chain means; None if never.

    tol "spread": sigma is the spread of one chain's value in equilibrium (the long chains'
    single-chain standard deviation), so the test asks that the batch has relaxed to within
    the equilibrium fluctuation of a chain. tol "mean": sigma is that spread / sqrt(nchains),
    the standard error of the batch mean itself. A batch already in equilibrium meets the
    "spread" test at once; it meets the "mean" test, for three observables over `window`
    consecutive measurements, only by chance (each mean sits within its own 1 sigma 68 % of the
    time, and slow observables stay outside for hundreds of sweeps), so "mean" times the
    fluctuations of the slowest observable rather than the relaxation."""
    ok = np.ones(len(rel.E), bool)
    for k, series in (("E", rel.E), ("M", rel.M), ("Q", rel.Q)):
        mean, sd = ref[k][:2]
        ok &= np.abs(series - mean) <= (sd if tol == "spread" else sd / np.sqrt(nchains))
    for i in range(len(ok) - window + 1):
        if ok[i:i + window].all():
            return int(rel.t[i]) if rel.t is not None else i * every
    return None


def checked_reference(L_edge, T, B, D, nchains=16, eq_sweeps=16000, nsamp=400, gap=5, seed=77, every=10):
    """The long plain chains that define equilibrium at one (T, B, D) point, with two checks.

    The reference: nchains chains from the reference's random start, eq_sweeps sweeps, then
    nsamp samples gap sweeps apart (reference_stats). Convergence: the same run from the
    ordered start (every spin along the field axis) must agree with it on E, |M| and Q within 3
    standard errors of the difference; where it does not, the plain chains have not reached one
    equilibrium within eq_sweeps (a metastable state, typically skyrmions that the random start
    traps at low temperature and the ordered start never nucleates), and sweeps to equilibrium
    measured against them mean nothing. Control: the equilibrium test applied to the reference
    chains' own samples (every `every` sweeps), i.e. to a start already in equilibrium, under
    both tolerances of sweeps_to_equilibrium.
    Returns (reference stats, info dict)."""
    chains = np.arange(nchains)
    rs = heisenberg_sampler(L_edge, D, [T] * nchains, [B] * nchains, seed=seed)
    vr = reference_samples(rs, chains, eq_sweeps, nsamp, gap)
    rs.close()
    os_ = heisenberg_sampler(L_edge, D, [T] * nchains, [B] * nchains, seed=seed + 1000)
    up = np.zeros((os_.box_sites, 3))
    up[:, 2] = 1.0
    for c in chains:
        os_.set_spins(int(c), up)
    vo = reference_samples(os_, chains, eq_sweeps, nsamp, gap)
    os_.close()
    ref, refo = reference_stats(vr), reference_stats(vo)
    converged = all(abs(ref[k][0] - refo[k][0]) <= 3 * np.hypot(ref[k][2], refo[k][2]) for k in "EMQ")
    step = max(1, every // gap)
    m = vr[::step].mean(1)
    ctrl = Relaxation(m[:, 0], m[:, 1], m[:, 2])
    info = {"converged": bool(converged),
            "ordered_start": {k: refo[k][0] for k in "EMQ"},
            "control_t_eq": {tol: sweeps_to_equilibrium(ctrl, ref, nchains, every=step * gap, tol=tol)
                             for tol in ("spread", "mean")}}
    return ref, info


def gated_warm_start(gen: Generator, sampler: Sampler, chains, cond, ref, steps=256, check_sweeps=200,
                     nsamp=100, gap=2):
    """Warm-start the chains, then judge them with the plain chain: after check_sweeps sweeps,
    E, |M| and Q averaged over nsamp samples must agree with the long-chain reference within
    3 standard errors of the difference (each side's error from its independent per-chain
    averages). If not, the chains are restarted from random spins (the reference's start).
    Returns True when the learned start was kept."""
    chains = np.asarray(chains)
    gen.warm_start(sampler, chains, cond, steps)
    sampler.sweep(check_sweeps, chains)
    obs = sampler.sample(gap, nsamp, chains)
    N = sampler.box_sites
    vals = {"E": obs[..., L.OBS_E] / N, "M": obs[..., L.OBS_ABSM] / N, "Q": obs[..., L.OBS_QTOT]}
    keep = True
    for k, v in vals.items():
        mean, _, se_ref = ref[k]
        m, se = _chain_stats(v)
        if abs(m - mean) > 3 * np.hypot(se, se_ref) + 1e-12:
            keep = False
    if not keep:
        rng = np.random.default_rng(0)
        for c in chains:
            v = rng.normal(size=(N, 3))
            v /= np.linalg.norm(v, axis=1, keepdims=True)
            sampler.set_spins(int(c), v)
    return keep


def evaluate_point(gen: Generator, T, B, D, nchains=16, tmax=4000, every=10, ref_sweeps=16000, steps=256, fine=100):
    """Sweeps to equilibrium from random and from learned starts at one (T, B, D) point, and
    the equilibrated samples per second each start gives a fresh batch of chains."""
    import time
    L_edge = gen.L
    ref, info = checked_reference(L_edge, T, B, D, nchains, ref_sweeps, 400, every=every)
    out = {"T": T, "B": B, "D": D, "ref": ref, "reference_check": info}
    for arm in ("random", "learned"):
        s = heisenberg_sampler(L_edge, D, [T] * nchains, [B] * nchains, seed=78 if arm == "random" else 79)
        s.synchronize()
        t0 = time.perf_counter()
        if arm == "learned":
            gen.warm_start(s, np.arange(nchains), np.tile([T, B, D], (nchains, 1)), steps=steps)
        t_gen = time.perf_counter() - t0
        rel = relaxation(s, np.arange(nchains), tmax, every=every, fine=fine)
        teq = sweeps_to_equilibrium(rel, ref, nchains, every=every)
        # equilibrated samples per second for this batch: nchains samples, SAMPSWEEPS=20 apart,
        # after teq sweeps (plus the generator time for learned starts), counted over 100 samples
        s.synchronize()
        t1 = time.perf_counter()
        s.sweep(200)
        s.synchronize()
        sweep_s = (time.perf_counter() - t1) / 200
        out[arm] = {"t_eq": teq, "gen_s": t_gen,
                    "t": [int(rel.t[i]) for i in (0, 1, 5, 10, 50, 100, -1)],
                    "E": list(np.round(rel.E[[0, 1, 5, 10, 50, 100, -1]], 4)),
                    "M": list(np.round(rel.M[[0, 1, 5, 10, 50, 100, -1]], 4)),
                    "Q": list(np.round(rel.Q[[0, 1, 5, 10, 50, 100, -1]], 3))}
        if teq is not None:
            wall = t_gen + (teq + 100 * 20) * sweep_s
            out[arm]["equilibrated_samples_per_s"] = nchains * 100 / wall
        s.close()
    if out["random"]["t_eq"] is not None and out["learned"]["t_eq"] is not None:
        out["sweeps_ratio"] = max(out["random"]["t_eq"], 1) / max(out["learned"]["t_eq"], 1)
    return out


def speed(L_edge=128, batch=16, steps=20, passes=16):
    """Generator timings with the hidden convolutions on the FP32 FMA pipes and on the tensor
    cores (warp-specialised forward kernel, cp.async-staged windows, and the default: TMA-staged
    windows at L = 128): training step (forward, backward, no update) and warm-start pass, in ms
    (wall time of synchronised calls, after warm-up)."""
    import time
    gen = Generator(L_edge, capacity=batch, seed=5)
    T, B = np.linspace(0.3, 1.2, batch), np.linspace(0.0, 0.5, batch)
    s = heisenberg_sampler(L_edge, 0.5, T, B, seed=3)
    s.sweep(20)
    cond = np.stack([T, B, np.full(batch, 0.5)], 1)
    gen.add_snapshots(s, np.arange(batch), cond)
    idx, sig = np.arange(batch, dtype=np.int32), np.full(batch, 0.5, np.float32)
    out = {"L": L_edge, "batch": batch}
    for tensor in (0, 2, 3, 4, 1):   # FMA, cp.async WS, cp.async, TMA WS, default
        gen.tensor_cores(tensor)
        for _ in range(3):
            gen.train_step(idx, sig, lr=0.0)
        t0 = time.perf_counter()
        for _ in range(steps):
            loss = gen.train_step(idx, sig, lr=0.0)
        train_ms = (time.perf_counter() - t0) / steps * 1e3
        gen.warm_start(s, np.arange(batch), cond, steps=2)
        t0 = time.perf_counter()
        gen.warm_start(s, np.arange(batch), cond, steps=passes)
        pass_ms = (time.perf_counter() - t0) / passes * 1e3
        name = {0: "fma", 1: "tcgen05", 2: "tcgen05_ws_cp_async", 3: "tcgen05_cp_async", 4: "tcgen05_ws_tma"}[tensor]
        out[name] = {"train_step_ms": train_ms, "warm_pass_ms": pass_ms, "loss": loss}
    s.close()
    gen.close()
    return out


def train_launches(L_edge=128, batch=16, steps=4):
    """A profiling workload: `steps` training steps (forward, backward, no update) of the
    default tensor-core generator on a batch of `batch` snapshots of L x L lattices."""
    gen = Generator(L_edge, capacity=batch, seed=5)
    T, B = np.linspace(0.3, 1.2, batch), np.linspace(0.0, 0.5, batch)
    s = heisenberg_sampler(L_edge, 0.5, T, B, seed=3)
    s.sweep(20)
    gen.add_snapshots(s, np.arange(batch), np.stack([T, B, np.full(batch, 0.5)], 1))
    s.close()
    idx, sig = np.arange(batch, dtype=np.int32), np.full(batch, 0.5, np.float32)
    loss = [gen.train_step(idx, sig, lr=0.0) for _ in range(steps)]
    gen.close()
    return {"L": L_edge, "batch": batch, "steps": steps, "loss": loss[-1]}


def warm_launches(L_edge=128, nchains=16, passes=8, sweeps=100, seed=5):
    """A profiling workload of the learned start: one warm start of `passes` denoising passes
    for `nchains` chains of L x L (untrained generator: the same kernels and shapes as a trained
    one), then `sweeps` plain sweeps of those chains."""
    gen = Generator(L_edge, capacity=0, seed=seed)
    s = heisenberg_sampler(L_edge, 0.5, [0.6] * nchains, [0.25] * nchains, seed=3)
    chains = np.arange(nchains)
    gen.warm_start(s, chains, np.tile([0.6, 0.25, 0.5], (nchains, 1)), steps=passes)
    s.sweep(sweeps)
    s.synchronize()
    s.close()
    gen.close()
    return {"L": L_edge, "chains": nchains, "passes": passes, "sweeps": sweeps}


def main(argv=None):
    """Learned-start experiment (2-D Heisenberg L = 128): dataset over a (T, B, D) grid from
    the plain sampler, GPU training, and per-point comparison of learned and random starts.
    Prints one JSON object per line.
    --speed: generator timings only (FMA and tensor-core convolutions).
    --train-launches: four training steps of the default generator (a profiling workload).
    --warm-launches: one 8-pass warm start of 16 chains and 100 sweeps (a profiling workload)."""
    import argparse
    import json
    import time
    if argv is None:
        import sys
        argv = sys.argv[1:]
    if "--speed" in argv:
        print(json.dumps(speed()))
        return
    if "--train-launches" in argv:
        print(json.dumps(train_launches()))
        return
    if "--warm-launches" in argv:
        print(json.dumps(warm_launches()))
        return
    ap = argparse.ArgumentParser()
    ap.add_argument("--L", type=int, default=128)
    ap.add_argument("--replicas", type=int, default=4)
    ap.add_argument("--snaps", type=int, default=56)
    ap.add_argument("--train-steps", type=int, default=6000)
    ap.add_argument("--batch", type=int, default=16)
    ap.add_argument("--tmax", type=int, default=4000)
    ap.add_argument("--save", default="")
    ap.add_argument("--ws-steps", type=int, default=256, help="denoising passes of a warm start")
    ap.add_argument("--seed", type=int, default=1, help="generator initialisation and noise seed")
    a = ap.parse_args(argv)
    Ts = [0.3, 0.45, 0.6, 0.9, 1.2, 1.5]
    Bs = [0.0, 0.25, 0.5, 0.75, 1.0]
    Ds = [0.2, 0.5, 0.8]
    pts = [(T, B, D) for D in Ds for T in Ts for B in Bs]
    cap = len(pts) * a.replicas * a.snaps
    gen = Generator(a.L, capacity=cap, seed=a.seed)
    t0 = time.perf_counter()
    n = make_dataset(gen, pts, replicas=a.replicas, eq_sweeps=4000, snap_every=50, snaps=a.snaps)
    t1 = time.perf_counter()
    hist = train(gen, a.train_steps, batch=a.batch, lr=2e-3)
    t2 = time.perf_counter()
    if a.save:
        gen.save(a.save)
    print(json.dumps({"L": a.L, "seed": a.seed, "snapshots": n, "dataset_s": t1 - t0, "train_s": t2 - t1,
                      "train_steps": a.train_steps, "batch": a.batch,
                      "loss_first": float(hist[:20].mean()), "loss_last": float(hist[-20:].mean())}), flush=True)
    for (T, B, D) in [(0.6, 0.25, 0.5), (0.45, 0.25, 0.5), (0.9, 0.25, 0.8), (0.6, 0.0, 0.2), (0.3, 0.25, 0.5)]:
        print(json.dumps(evaluate_point(gen, T, B, D, tmax=a.tmax, steps=a.ws_steps)), flush=True)


if __name__ == "__main__":
    main()
