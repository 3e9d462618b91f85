"""Benchmark: spin updates/s of the checkerboard Metropolis sweep on one GB300.

Workload (default, "c4"): 3-D cubic Heisenberg lattice, L = 128 periodic (2,097,152 FP32
unit-vector spins per chain), J = 1, bulk DMI D = 0.3 (Js/3d_nn_bloch.dat), B_z = 0.2,
40 chains at temperatures evenly spaced 0.2..2.0. Spins live in HBM in split-colour SoA
planes (960 MiB for the 40 chains, larger than the 129 MB L2, so every timed sweep streams
from HBM and no L2 flush is needed).

A step is one sample of the reference's inner loop (Old/lib/main.cpp:182-233): SAMPSWEEPS
(default 10) checkerboard sweeps of all 40 chains, then E, M, subM, sub4M and Q of every chain.
  value : device-timed updates/s (CUDA events on the library's stream around K steps;
          observables stay on the device in the FP64 accumulators).
  e2e   : the same metric through the C ABI with host buffers: every step sets (T, B) of
          the 40 chains from host memory, sweeps, and reads the observables back
          (nmmc_set_points + nmmc_sweep_measure).
  roofline: the half-sweep kernel, 36 algorithmic bytes per update (each site read as a
          target, written once, read once as a neighbour of the other colour), against the
          measured HBM copy bandwidth.
  cpu_baseline: the oracle (a C++ restatement of the reference's random-site update loop)
          on one host core, on one chain of the same lattice.

--impl reference times that CPU restatement on all host cores instead (one process per
core, one chain each, as the reference runs one MPI rank per core).
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import multiprocessing as mp
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

BYTES_PER_UPDATE = 36          # Heisenberg FP32 (see module docstring)
METRIC = "spin updates/s"
UNIT = "updates/s"


def make_config(name):
    """Workloads: c1-c4 are the reference's configurations (2-D Ising L=32, 2-D Heisenberg L=64,
    512 Weibull grains, 3-D Heisenberg L=128); c4 is the benchmark workload. c4j2 (a J1 + J2
    table) and x3 (3-D Weibull spheres) cover the general-table and masked HBM paths. The others
    are reported separately (run with --config)."""
    import numpy as np
    if name == "c4":
        return dict(name=name, workload="3-D cubic Heisenberg L=128 periodic, bulk DMI D=0.3, B_z=0.2, "
                                        "40 temperatures 0.2-2.0 (FP32 spins, checkerboard)",
                    shape="c", edge=128, periodic=True, ising=False, jfile="3d_nn_bloch.dat", D=0.3,
                    T=list(np.linspace(0.2, 2.0, 40)), B=[0.2] * 40, sizes=None, samp=10,
                    bytes_per_update=36)
    if name == "c4j2":
        return dict(name=name, workload="3-D cubic Heisenberg L=128 periodic, J1 = 1 with bulk DMI D=0.3 plus "
                                        "12 face-diagonal J2 = 0.1 (Js/3d_j1j2_bloch.dat; multi-colour gather "
                                        "sweep), B_z=0.2, 40 temperatures 0.2-2.0",
                    shape="c", edge=128, periodic=True, ising=False, jfile="3d_j1j2_bloch.dat", D=0.3,
                    T=list(np.linspace(0.2, 2.0, 40)), B=[0.2] * 40, sizes=None, samp=10,
                    bytes_per_update=None, hbm=True)
    if name == "x3":
        return dict(name=name, workload="96 3-D Weibull-masked spheres (radius 30, WEIBULLFACT=3, box edge 90), "
                                        "Heisenberg J=1, bulk DMI D=0.3, B_z=0.2, 96 temperatures 0.2-2.0 "
                                        "(HBM path over per-chain lists of filled sites)",
                    shape="x", edge=90, periodic=False, ising=False, jfile="3d_nn_bloch.dat", D=0.3,
                    T=list(np.linspace(0.2, 2.0, 96)), B=[0.2] * 96, sizes=None, amean=30.0, samp=10,
                    bytes_per_update=36, hbm=True)
    if name == "c3":
        T, B = np.meshgrid(np.linspace(0.05, 1.5, 32), np.linspace(0.0, 1.0, 16))
        return dict(name=name, workload="512 circular Weibull-masked grains (radius a log-normal, mean 20, "
                                        "sd 5, WEIBULLFACT=3, edge 90), Heisenberg J=1, interfacial DMI "
                                        "D=0.5, one point of a 32 T (0.05-1.5) x 16 B_z (0-1) grid each",
                    shape="w", edge=90, periodic=False, ising=False, jfile="2d_nn_interfacial.dat", D=0.5,
                    T=list(T.ravel()), B=list(B.ravel()), sizes="lognormal", amean=20.0, asd=5.0,
                    samp=10, bytes_per_update=37)
    if name == "c2":
        T, B = np.meshgrid(np.linspace(0.05, 1.5, 20), np.linspace(0.0, 1.0, 21))
        return dict(name=name, workload="2-D Heisenberg L=64 periodic, interfacial DMI D=0.5, "
                                        "21 B_z (0-1) x 20 T (0.05-1.5) points, one chain each",
                    shape="s", edge=64, periodic=True, ising=False, jfile="2d_nn_interfacial.dat", D=0.5,
                    T=list(T.ravel()), B=list(B.ravel()), sizes=None, samp=20, bytes_per_update=36)
    if name == "c1":
        return dict(name=name, workload="2-D Ising L=32 periodic, J=1, H=0, 13 temperatures 2.0-2.6",
                    shape="s", edge=32, periodic=True, ising=True, jfile="2d_nn.dat", D=0.0,
                    T=list(np.linspace(2.0, 2.6, 13)), B=[0.0] * 13, sizes=None, samp=10,
                    bytes_per_update=3)
    if name == "c5":
        return dict(name=name, workload="learned warm start: 2-D Heisenberg L=128 periodic, interfacial DMI; "
                                        "generator (8 periodic 3x3 conv layers, 48 channels, BF16) trained on "
                                        "20,160 snapshots of the plain sampler over 6 T (0.3-1.5) x 5 B_z (0-1) x "
                                        "3 D (0.2-0.8); 16 chains per evaluation point, learned against random "
                                        "starts",
                    shape="s", edge=128, periodic=True, ising=False, jfile="2d_nn_interfacial.dat", D=0.5,
                    T=[0.6, 0.45, 0.9, 0.6, 0.3], B=[0.25, 0.25, 0.25, 0.0, 0.25], Dp=[0.5, 0.5, 0.8, 0.2, 0.5],
                    sizes=None, samp=20, bytes_per_update=36)
    raise ValueError(name)


# ------------------------------------------------------------------------------------------
# clocks during the timed region
# ------------------------------------------------------------------------------------------
class Clocks:
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in self.lines:
            p = [x.strip() for x in l.split(",")]
            if len(p) < 8:
                continue
            try:
                sm.append(float(p[0]))
                mx = float(p[1])
            except ValueError:
                continue
            for n, v in zip(names, p[4:8]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": mx, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


# DRAM bytes per site update of the benchmark's half-sweep kernel, from one ncu capture
# (dram__bytes_read.sum + dram__bytes_write.sum of a launch of 8 of the 40 chains of 128^3,
# divided by its 8,388,608 updates): 24.0 B read (own spins and the other colour once each)
# + 6.7 B written (only quads with an accepted move are stored). Traffic grows in proportion
# to the chains a launch covers, so a launch's traffic is this figure times its updates.
HALF_SWEEP_DRAM_BYTES_PER_UPDATE = 30.7


def profiled_traffic(updates_per_launch):
    """DRAM bytes of one half-sweep launch of the benchmark workload (see above)."""
    return HALF_SWEEP_DRAM_BYTES_PER_UPDATE * updates_per_launch


# ------------------------------------------------------------------------------------------
# CPU legs (the oracle restatement of the reference's update loop)
# ------------------------------------------------------------------------------------------
def _oracle_chain(cfg, T, B, size):
    from nanomagmc_gb300.sampler import interactions_file
    from oracle import oracle as O
    dim = 3 if cfg["shape"] in "cCxX" else 2
    off, J, Dv = O.read_interactions(interactions_file(cfg["jfile"]), dim, 1.0, cfg["D"])
    lat = O.Lattice.create(dim, cfg["edge"], cfg["ising"], cfg["periodic"], cfg["shape"], off, J, Dv,
                           size=size, wbeta=3.0, seed=1, chain=0, useJ=True,
                           useD=cfg["D"] != 0 and not cfg["ising"])
    lat.set_beta(1.0 / T)
    if cfg["ising"]:
        lat.set_H(B, 0.0, 0.0)
    else:
        lat.set_H(0.0, 0.0, B)
    rng = O.Rng(1, 2, 3)
    lat.all_rand(rng)
    return lat, rng


def _cpu_worker(args):
    cfg, T, B, size, steps, warmup, barrier, q, chunk = args
    lat, rng = _oracle_chain(cfg, T, B, size)
    for _ in range(warmup):
        lat.bench_equil(rng, chunk)
    if barrier is not None:
        barrier.wait()
    t0 = time.perf_counter()
    n = 0
    for _ in range(steps):
        n += lat.bench_equil(rng, chunk)
    dt = time.perf_counter() - t0
    q.put((n, dt))


def cpu_baseline(cfg, seconds=10.0):
    """One core, one chain of the workload's lattice; about `seconds` of update loop."""
    T, B = cfg["T"][len(cfg["T"]) // 2], cfg["B"][len(cfg["B"]) // 2]
    size = cfg.get("amean", cfg["edge"])
    lat, rng = _oracle_chain(cfg, T, B, size)
    lat.bench_equil(rng, 200000)
    n, t0 = 0, time.perf_counter()
    while time.perf_counter() - t0 < seconds:
        n += lat.bench_equil(rng, 1000000)
    dt = time.perf_counter() - t0
    return {"value": n / dt, "unit": UNIT, "cores": 1, "kind": "port",
            "sample": "%d random-site attempts (state::equil order, FP64) on one chain of the workload's "
                      "lattice (%d sites) at T=%.2f, %.1f s on one host core" % (n, lat.n, T, dt)}


def run_reference(args, cfg):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    cores = os.cpu_count() or 1
    procs = min(cores, len(cfg["T"]))
    chunk = 20000      # attempts per process per step
    ctx = mp.get_context("spawn")
    barrier = ctx.Barrier(procs)
    q = ctx.Queue()
    ps = []
    for i in range(procs):
        k = i * len(cfg["T"]) // procs
        p = ctx.Process(target=_cpu_worker, args=((cfg, cfg["T"][k], cfg["B"][k], cfg.get("amean", cfg["edge"]),
                                                   args.steps, args.warmup, barrier, q, chunk),))
        p.start()
        ps.append(p)
    res = [q.get() for _ in ps]
    for p in ps:
        p.join()
    n = sum(r[0] for r in res)
    wall = max(r[1] for r in res)
    value = n / wall
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": wall * 1e3 / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic",
        "config": {"workload": cfg["workload"], "name": cfg["name"], "chains_per_gpu": len(cfg["T"]),
                   "step": "a bounded sample of the workload: %d random-site attempts per process and step "
                           "(the reference's state::equil update, FP64), on %d of its chains" % (chunk, procs),
                   "parallelism": "%d host processes, one chain each (the reference's one MPI rank per core)"
                                  % procs},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": procs, "kind": "port",
                         "sample": "%d processes x %d steps x %d random-site attempts, one chain of the "
                                   "workload's lattice per process (the reference cannot be built: "
                                   "GSL, HDF5, MPI and xtensor are absent; this is the oracle "
                                   "restatement of its update loop)" % (procs, args.steps, chunk)},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


# ------------------------------------------------------------------------------------------
# replicas over ranks: every rank runs the same workload (weak scaling); the job's time is the
# slowest rank's and its rate counts every rank's updates
# ------------------------------------------------------------------------------------------
def rank_device(visible, local):
    """The one GPU of local rank `local`: its entry of CUDA_VISIBLE_DEVICES when that lists
    several devices, else the local rank. libnmmc links the CUDA runtime statically, so the
    device is fixed through the environment before the library's first CUDA call."""
    ids = [v.strip() for v in (visible or "").split(",") if v.strip()]
    if len(ids) > 1:
        return ids[local % len(ids)]
    return ids[0] if ids else str(local)


def max_over_ranks(x, dist):
    if dist is None:
        return x
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def aggregate_rate(units_per_rank, world, seconds):
    return units_per_rank * world / seconds


# ------------------------------------------------------------------------------------------
# GPU leg
# ------------------------------------------------------------------------------------------
def run_gpu(args, cfg):
    import numpy as np

    from nanomagmc_gb300 import _lib as L
    from nanomagmc_gb300.sampler import Sampler, interactions_file, make_options, read_interactions

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    dist = None
    if world > 1:
        import torch
        import torch.distributed as dist
        local = int(os.environ.get("LOCAL_RANK", "0"))
        os.environ["CUDA_VISIBLE_DEVICES"] = rank_device(os.environ.get("CUDA_VISIBLE_DEVICES"), local)
        dist.init_process_group("gloo")
    lib = L.load()

    dim = 3 if cfg["shape"] in "cCxX" else 2
    opt = make_options(cfg["shape"], edge=cfg["edge"], size=cfg.get("amean"), ising=cfg["ising"],
                       periodic=cfg["periodic"], J=1.0, D=cfg["D"], weibull=3.0, asd=cfg.get("asd", 0.0))
    inter = read_interactions(interactions_file(cfg["jfile"]), dim, 1.0, cfg["D"])
    T = np.array(cfg["T"])
    nch = len(T)
    sizes = None
    if cfg["sizes"] == "lognormal":
        am, sd = cfg["amean"], cfg["asd"]
        lm, ls = np.log(am * am / np.sqrt(sd * sd + am * am)), np.sqrt(np.log(1 + sd * sd / (am * am)))
        sizes = [lib.nmmc_lognormal_size(7, k, lm, ls) for k in range(nch)]
    s = Sampler(opt, inter, T=T, H=np.array(cfg["B"]), sizes=sizes, seed=1000 + rank)
    if args.path:
        s.option(L.OPT_SWEEP_PATH, args.path)
    if args.half_kernel:
        s.option(L.OPT_HALF_KERNEL, args.half_kernel)
    if args.ring_zseg:
        s.option(L.OPT_RING_ZSEG, args.ring_zseg)
    if args.l2_prefetch >= 0:
        s.option(L.OPT_L2_PREFETCH, args.l2_prefetch)
    if args.measure_sites:
        s.option(L.OPT_MEASURE_SITES, args.measure_sites)
    if args.masked_compact >= 0:
        s.option(L.OPT_MASKED_COMPACT, args.masked_compact)
    if args.charge_pass >= 0:
        s.option(L.OPT_CHARGE_PASS, args.charge_pass)
    sites = np.array([s.site_counts(c)[0] for c in range(nch)])
    N = int(sites.max())
    updates_per_sweep = int(sites.sum())
    updates_per_step = updates_per_sweep * cfg["samp"]

    def barrier():
        s.synchronize()
        if dist is not None:
            dist.barrier()

    S = cfg["samp"]

    def step_device():
        # SAMPSWEEPS sweeps then the observables, accumulated on the device (one launch on the
        # shared-memory resident path of a 2-D lattice)
        L.check(lib.nmmc_sweep_measure(s.h, None, nch, S, None, None, 1))

    # ---- device-timed region: K steps, inputs resident in HBM ----
    for _ in range(args.warmup):
        step_device()
    s.option(L.OPT_TIMING, 1)
    s.timing()   # reset
    barrier()
    with Clocks(int(os.environ.get("LOCAL_RANK", "0"))) as clk:
        L.check(lib.nmmc_timer_mark(s.h, 0))
        for _ in range(args.steps):
            step_device()
        L.check(lib.nmmc_timer_mark(s.h, 1))
        ms = C.c_double()
        L.check(lib.nmmc_timer_elapsed(s.h, 0, 1, C.byref(ms)))
        barrier()
    region_ms = ms.value
    k_ms, k_launches, k_updates = s.timing()
    s.option(L.OPT_TIMING, 0)
    acc = s.accumulators()
    if not (np.all(np.isfinite(acc)) and np.all(acc[:, 0] == args.warmup + args.steps)):
        raise RuntimeError("accumulators after the timed region are wrong: %r" % acc[:4])
    region_ms = max_over_ranks(region_ms, dist)
    value = aggregate_rate(updates_per_step * args.steps, world, region_ms / 1e3)

    # ---- observables of the final state: production FP32 per-site terms vs the FP64 mode
    # (the reference's formulas per site in FP64); largest difference over the chains,
    # relative to the observable's scale (E: |E|, magnetisations: N, Q: absolute) ----
    o32, q32 = s.measure()
    s.option(L.OPT_MEASURE_FP64, 1)
    o64, q64 = s.measure()
    s.option(L.OPT_MEASURE_FP64, 0)
    fp64_check = {
        "E_rel": float(np.max(np.abs(o32[:, L.OBS_E] - o64[:, L.OBS_E]) / np.abs(o64[:, L.OBS_E]))),
        "M_rel_to_N": float(np.max(np.abs(o32[:, 1:13] - o64[:, 1:13])) / N),
        "Q_abs": float(np.max(np.abs(q32.sum(1) - q64.sum(1)))),
        "chains": nch,
    }

    # ---- e2e through the C ABI with host buffers (page-locked, from nmmc_host_alloc) ----
    pinned = []

    def host_array(shape, dtype, fill):
        nbytes = int(np.prod(shape)) * np.dtype(dtype).itemsize
        ptr = C.c_void_p()
        L.check(lib.nmmc_host_alloc(nbytes, C.byref(ptr)))
        pinned.append(ptr)
        a = np.frombuffer((C.c_char * nbytes).from_address(ptr.value), dtype=dtype).reshape(shape)
        a[...] = fill
        return a, ptr

    chains, pc = host_array((nch,), np.int32, np.arange(nch))
    Th, pT = host_array((nch,), np.float64, T)
    Hh, pH = host_array((nch,), np.float64, cfg["B"])
    obs, pO = host_array((nch, L.OBS_N), np.float64, 0.0)

    def step_e2e():
        L.check(lib.nmmc_set_points(s.h, pc, pT, pH, nch))
        L.check(lib.nmmc_sweep_measure(s.h, pc, nch, S, pO, None, 0))

    e2e_steps = max(3, args.steps // 4)
    for _ in range(3):
        step_e2e()
    barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        step_e2e()
    barrier()
    e2e_s = time.perf_counter() - t0
    e2e_s = max_over_ranks(e2e_s, dist)
    e2e = aggregate_rate(updates_per_step * e2e_steps, world, e2e_s)
    assert np.all(np.isfinite(obs))
    del chains, Th, Hh, obs
    for ptr in pinned:
        L.check(lib.nmmc_host_free(ptr))

    hbm = cfg["name"] == "c4" or cfg.get("hbm", False)
    colours = s.option(L.OPT_COLOURS)
    general = colours > 2
    predraw = (not hbm) and s.option(L.OPT_RESIDENT_PREDRAW) == 2
    # masked Heisenberg lattices on the HBM path: compact form, gathered and written back per call
    compact = hbm and cfg["shape"] in "wx" and not cfg["ising"] and s.option(L.OPT_MASKED_COMPACT) == 0
    shape = {"resident_bins": s.option(L.OPT_RESIDENT_BINS), "resident_threads": s.option(L.OPT_RESIDENT_THREADS),
             "resident_drawn_ahead": predraw} \
        if not hbm else ({"colour_classes": colours} if general else {})
    # general tables: each of the q class launches reads the lattice once (targets and their
    # gathered neighbours) and writes its own class: 12 B x (q + 1) per update
    bpu = cfg["bytes_per_update"] if cfg["bytes_per_update"] else 12 * (colours + 1)
    # ---- roofline of the sweep kernel ----
    launch_ms = k_ms / max(1, k_launches)
    upd_per_launch = k_updates / max(1, k_launches)
    achieved = bpu * upd_per_launch / (launch_ms / 1e3) / 1e9
    peak, peak_kind = measured_peak()
    traffic = profiled_traffic(upd_per_launch) if cfg["name"] == "c4" else None
    s.close()
    if not hbm:
        kernel, note = ("k_resident (sweeps and observables in one launch; time includes both)",
                        "shared-memory resident: HBM is not the bound; algorithmic bytes for comparison")
    elif general:
        kernel, note = ("k_colour_sweep<3,periodic,Heisenberg> (%d colour classes)" % colours,
                        "multi-colour gather sweep of a general interaction table; per launch, updates of "
                        "one class x 12 B x (classes + 1)")
    elif cfg["shape"] == "x":
        kernel, note = (("k_heis_compact<3,axial DMI> (filled sites in compact planes)" if compact else
                         "k_heis_half<3,open,masked,axial DMI> over filled-site lists"),
                        "algorithmic bytes of the half-sweep launches (filled sites only); time per call "
                        "includes the gather into and write-back from the compact planes" if compact else
                        "algorithmic bytes of the half-sweep launches (filled sites only)")
    else:
        kernel, note = "k_heis_half_q4<3,periodic,axial DMI>", "algorithmic bytes of the half-sweep launches"

    if rank != 0:
        return 0
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": region_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": cfg["workload"], "name": cfg["name"], "chains_per_gpu": nch,
                   "sites_per_chain": N if cfg["sizes"] is None else "%d..%d" % (sites.min(), sites.max()),
                   "step": "one sample of the reference's inner loop: SAMPSWEEPS=%d checkerboard sweeps "
                           "of every chain, then E, M, subM, sub4M and Q of every chain" % cfg["samp"],
                   "l2": ("inputs (%.0f MiB of %sspins) larger than L2 (129 MB); no flush"
                          % (int(sites.sum()) * 12 / 2 ** 20, "filled sites' " if cfg["shape"] == "x" else ""))
                         if hbm else "shared-memory resident lattices; L2/HBM not binding",
                   "parallelism": "replicas" if world > 1 else "single GPU", **shape},
        # H2D per step, from page-locked memory: the chain list (4 B) + (beta, H) FP32 (16 B)
        # and H FP64 (24 B) per chain; D2H into page-locked memory: NMMC_OBS_N doubles per chain
        "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": int(nch * (4 + 16 + 24)),
                "d2h_bytes_per_step": int(nch * L.OBS_N * 8),
                "step": "nmmc_set_points (T,B from host) + nmmc_sweep_measure(SAMPSWEEPS) "
                        "(observables to host)"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic, "kernel": kernel, "bytes_per_update": bpu,
                     "peak_source": peak_kind + " (MEASURED_PEAKS.json hbm_gbs)", "note": note},
        # per step: HBM path one launch per colour class and sweep + counter advance + measure
        # (+ the general energy term) + finalize; resident path one launch (sweeps and
        # observables; the chain marks are kept), preceded by k_predraw in the drawn-ahead variant;
        # the compact form adds its gather and write-back
        "gpu_launches": int(args.steps * ((colours * cfg["samp"] + 3 + int(general) + 2 * int(compact)) if hbm
                                          else 1 + int(predraw))),
        "clocks": clk.summary(),
        "fp64_check": fp64_check,
    }
    if not args.no_cpu:
        line["cpu_baseline"] = cpu_baseline(cfg, args.cpu_seconds)
    print(json.dumps(line))
    return 0


# ------------------------------------------------------------------------------------------
# c5: learned warm start against the plain random start (equilibrated samples/s)
# ------------------------------------------------------------------------------------------
def run_c5(args, cfg):
    """At each evaluation point, 16 chains of 128^2 start either from random spins (the
    reference's start) or from the generator's warm start; both then run the plain Metropolis
    chain. Sweeps to equilibrium: the first sweep after which the 16-chain means of E/N, |M|/N
    and Q stay within 1 sigma of long plain chains for 5 consecutive measurements (after every
    sweep for the first 100 sweeps, then every 10), sigma the
    spread of one chain's value in equilibrium (warmstart.sweeps_to_equilibrium; the figure with
    sigma / sqrt(16) is reported beside it, with the same test applied to the equilibrated long
    chains themselves as a control); a start that does not get there within 4000 sweeps is
    charged 4000 (a lower bound, flagged). The long chains are checked: run again from the
    ordered start they must agree within 3 sigma (warmstart.checked_reference); a point where
    they do not has no equilibrium to measure against and is left out of the ratios and the
    line's value (reported). The 3 sigma gate (the chains' E, |M|, Q over 100 samples after
    equilibration against the long chains) is reported per point. Equilibrated samples/s of an
    arm: the 16 chains brought to equilibrium, divided by the wall time of the warm start
    (generator passes, learned arm only) and of the sweeps to equilibrium (sweep time measured
    on the same batch); the figure with a sampling phase of NSAMPS = 100 samples SAMPSWEEPS = 20
    apart is reported beside it. The generator is trained once; its dataset and training time
    are reported beside the line. Each pass count of --ws-steps (comma separated) is evaluated
    with the same generator; the first is the line's value."""
    import numpy as np

    from nanomagmc_gb300 import _lib as L
    from nanomagmc_gb300 import warmstart as W

    L.load()
    nch, every, fine, tmax, nsamp = 16, 10, 100, 4000, 100
    # pass counts; a "q" suffix runs the passes on the quadratic noise schedule
    passes = [v.strip() for v in str(args.ws_steps).split(",")]
    Ts = [0.3, 0.45, 0.6, 0.9, 1.2, 1.5]
    Bs = [0.0, 0.25, 0.5, 0.75, 1.0]
    Ds = [0.2, 0.5, 0.8]
    grid = [(T, B, D) for D in Ds for T in Ts for B in Bs]
    gen = W.Generator(cfg["edge"], capacity=len(grid) * 4 * 56, seed=1)
    t0 = time.perf_counter()
    nsnap = W.make_dataset(gen, grid, replicas=4, eq_sweeps=4000, snap_every=50, snaps=56)
    t1 = time.perf_counter()
    hist = W.train(gen, args.train_steps, batch=16, lr=2e-3)
    t2 = time.perf_counter()

    def arm_run(T, B, D, ref, arm):
        ws = int(str(arm).rstrip("q"))
        gen.schedule(1 if str(arm).endswith("q") else 0)
        s = W.heisenberg_sampler(cfg["edge"], D, [T] * nch, [B] * nch, seed=78 if ws == 0 else 79)
        chains = np.arange(nch)
        cond = np.tile([T, B, D], (nch, 1))
        if ws:   # warm-up of the generator kernels (a warm start redraws every spin)
            for _ in range(args.warmup):
                gen.warm_start(s, chains, cond, steps=2)
        s.synchronize()
        tg = time.perf_counter()
        if ws:
            gen.warm_start(s, chains, cond, steps=ws)
        s.synchronize()
        t_gen = time.perf_counter() - tg
        rel = W.relaxation(s, chains, tmax, every=every, fine=fine)
        teq = W.sweeps_to_equilibrium(rel, ref, nch, every=every)
        teq_mean = W.sweeps_to_equilibrium(rel, ref, nch, every=every, tol="mean")
        s.synchronize()
        ts = time.perf_counter()
        s.sweep(200)
        s.synchronize()
        sweep_s = (time.perf_counter() - ts) / 200
        obs = s.sample(2, nsamp, chains)
        N = s.box_sites
        vals = {"E": obs[..., L.OBS_E] / N, "M": obs[..., L.OBS_ABSM] / N, "Q": obs[..., L.OBS_QTOT]}
        gate = all(abs(W._chain_stats(v)[0] - ref[k][0]) <= 3 * np.hypot(W._chain_stats(v)[1], ref[k][2])
                   for k, v in vals.items())
        s.close()
        t_eq = teq if teq is not None else tmax
        wall_eq = t_gen + t_eq * sweep_s
        wall_samp = wall_eq + nsamp * cfg["samp"] * sweep_s
        return {"sweeps_to_eq": teq, "reached": teq is not None, "sweeps_to_eq_sigma_of_mean": teq_mean,
                "gen_ms": t_gen * 1e3, "sweep_us": sweep_s * 1e6,
                "gate_3sigma": bool(gate), "wall_to_eq_ms": wall_eq * 1e3,
                "equilibrated_samples_per_s": nch / wall_eq,
                "samples_per_s_with_nsamps": nch * nsamp / wall_samp}

    points = []
    with Clocks(int(os.environ.get("LOCAL_RANK", "0"))) as clk:
        for T, B, D in zip(cfg["T"], cfg["B"], cfg["Dp"]):
            ref, rinfo = W.checked_reference(cfg["edge"], T, B, D, nch, 16000, 400, every=every)
            pt = {"T": T, "B": B, "D": D, "reference_check": rinfo, "random": arm_run(T, B, D, ref, 0)}
            for ws in passes:
                pt["learned_%s" % ws] = arm_run(T, B, D, ref, ws)
            points.append(pt)

    valid = [p for p in points if p["reference_check"]["converged"]]

    def rate(key, field, pts=valid):
        if not pts:
            return None
        wall = sum(nch / p[key][field] for p in pts) if field == "equilibrated_samples_per_s" else \
            sum(nch * nsamp / p[key][field] for p in pts)
        return (nch if field == "equilibrated_samples_per_s" else nch * nsamp) * len(pts) / wall

    def ratio(p, key):
        if not p["reference_check"]["converged"]:
            return None
        return round(max(p["random"]["sweeps_to_eq"] or tmax, 1) / max(p[key]["sweeps_to_eq"] or tmax, 1), 2)

    summary = {}
    for key in ["learned_%s" % ws for ws in passes]:
        rat = [ratio(p, key) for p in points]
        summary[key] = {
            "equilibrated_samples_per_s": rate(key, "equilibrated_samples_per_s"),
            "equilibrated_samples_per_s_all_points": rate(key, "equilibrated_samples_per_s", points),
            "samples_per_s_with_nsamps": rate(key, "samples_per_s_with_nsamps"),
            "sweeps_ratio_per_point": rat,
            "points_ratio_ge_3": sum(1 for r in rat if r is not None and r >= 3.0),
            "gate_passed": sum(p[key]["gate_3sigma"] for p in points)}
    plain = rate("random", "equilibrated_samples_per_s")
    main_key = "learned_%s" % passes[0]
    value = summary[main_key]["equilibrated_samples_per_s"]
    line = {
        "metric": "equilibrated samples/s (learned start vs plain random start)", "value": value,
        "unit": "samples/s", "n_gpus": 1, "steps": len(points), "warmup": args.warmup,
        "ms_per_step": sum(p[main_key]["wall_to_eq_ms"] for p in points) / len(points),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32 chain, bf16 generator",
        "data": "synthetic",
        "config": {"workload": cfg["workload"], "name": "c5", "chains_per_point": nch, "ws_passes": passes,
                   "train_steps": args.train_steps, "tmax_sweeps": tmax,
                   "step": "one evaluation point: warm start (learned arm) and sweeps to equilibrium of 16 chains"},
        "plain_value": plain, "learned_over_plain": (value / plain) if value and plain else None,
        "points_with_converged_reference": len(valid),
        "plain_samples_per_s_with_nsamps": rate("random", "samples_per_s_with_nsamps"),
        "by_passes": summary, "points": points,
        "generator": {"snapshots": nsnap, "dataset_s": t1 - t0, "train_s": t2 - t1,
                      "loss_first": float(hist[:20].mean()), "loss_last": float(hist[-20:].mean())},
        "e2e": {"value": value, "unit": "samples/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": int(nch * L.OBS_N * 8 * (fine + 1 + (tmax - fine) // every)),
                "step": "host-timed (synchronised) warm start + sweeps to equilibrium; relaxation measurements "
                        "not charged"},
        "clocks": clk.summary(),
    }
    gen.close()
    print(json.dumps(line))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--config", default="c4", choices=["c4", "c3", "c2", "c1", "c4j2", "x3", "c5"],
                    help="workload (c4 is the benchmark workload)")
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--path", type=int, default=0, help="sweep path: 0 auto, 1 HBM, 2 resident")
    ap.add_argument("--half-kernel", type=int, default=0,
                    help="HBM half-sweep variant: 0 four sites/thread (3 CTAs/SM), 1 one site/thread, "
                         "2 four sites/thread (2 CTAs/SM), 3-7 ring-pipelined (3-5 one barrier per plane, "
                         "6-7 producer and consumer warps)")
    ap.add_argument("--l2-prefetch", type=int, default=-1,
                    help="four-site half-sweeps: L2 prefetch distance in quarter waves (-1: library default)")
    ap.add_argument("--ring-zseg", type=int, default=0, help="z-planes per CTA of the ring-pipelined half-sweeps")
    ap.add_argument("--measure-sites", type=int, default=0, choices=[0, 2, 4],
                    help="HBM-path measurement kernel: sites per thread item (0: library default)")
    ap.add_argument("--masked-compact", type=int, default=-1, choices=[-1, 0, 1],
                    help="masked Heisenberg HBM sweeps: 0 compact form, 1 box layout (default: library choice)")
    ap.add_argument("--charge-pass", type=int, default=-1, choices=[-1, 0, 1],
                    help="charge pass after the fused half-sweeps: 0 sliding rows, 1 measurement-kernel items "
                         "(default: library choice)")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--ws-steps", default="8,16,32,64,128,64q,128q",
                    help="c5: denoising passes of a learned warm start (comma-separated list: each evaluated, the "
                         "first is the line's value; a q suffix: quadratic noise schedule)")
    ap.add_argument("--train-steps", type=int, default=6000, help="c5: generator training steps")
    ap.add_argument("--chains", type=int, default=0,
                    help="use only the first N chains of the configuration (profiling captures)")
    args = ap.parse_args()
    if args.warmup < 3:
        ap.error("at least 3 warm-up steps")
    cfg = make_config(args.config)
    if args.chains and args.chains != len(cfg["T"]):
        cfg["T"] = cfg["T"][: args.chains]
        cfg["B"] = cfg["B"][: args.chains]
        cfg["workload"] += " [reduced to %d chains]" % args.chains
    if cfg["name"] == "c5":
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "the reference has no learned warm start; its "
                              "plain random start is this workload's plain arm"}))
            return 0
        return run_c5(args, cfg)
    if args.impl == "reference":
        return run_reference(args, cfg)
    return run_gpu(args, cfg)


if __name__ == "__main__":
    sys.exit(main())
