"""Benchmark: fused RK4 site-updates/s at 1024^2 on GB300 (one JSON line on rank 0).

Workload (the precision-check physics at 1024^2): periodic 1024x1024 grid,
lx = ly = 400 um, dt = 5e-4 ps, single reservoir, zero potential, continuous
Gaussian pump (P0 = 0.02, sigma drawn per member in [8, 20] um), truncated-Wigner
noise on (Philox seed 42 + member), complex64.  ``--members`` same-shape fields
are stepped together (default 32: 512 MB of state, four times the 129 MB L2, so
every step streams from HBM).  A "step" is one RK4 time step of every member.

* ``value``  -- device-resident throughput: K steps between CUDA events on the
  library stream, inputs already in HBM.
* ``e2e``    -- the same metric through the public solver API
  (``RK4CudaSolver.advance`` on pinned host state): each call copies psi and n_R
  host->device, runs 64 steps in CUDA graphs and copies them back.
* ``roofline`` -- 28 algorithmic bytes per site-update (psi r/w 16 B, n_R r/w 8 B,
  pump 4 B) / average kernel time, against the measured HBM copy bandwidth.
* ``cpu_baseline`` -- the FP64 NumPy oracle (a restatement of the reference's
  rk4-fdm) on a bounded sample, on this host's cores.

``--impl reference`` times the reference algorithm's CPU implementation (the
oracle port, one worker process per member up to the host's core count) on the
same workload and metric.  Multi-GPU runs (torchrun) step independent replicas:
the path has no exchange step.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

NX = NY = 1024
LX = LY = 400.0
DT = 5e-4
P0 = 0.02
BYTES_PER_SITE = 28  # FP32: psi 8 B read + 8 B write, n_R 4 + 4, pump envelope 4
METRIC = "RK4 site-updates/s at 1024^2"


def dist_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def rank_members(rank, world, members):
    """Weak scaling: every rank steps its own `members` replicas, global indices
    rank * members .. rank * members + members - 1 (no data-path exchange between ranks)."""
    if not 0 <= rank < world:
        raise ValueError("rank out of range")
    return list(range(rank * members, (rank + 1) * members))


def max_over_ranks(value, world, device="cpu"):
    """The slowest rank's time (MAX all-reduce); the value itself for one rank."""
    if world <= 1:
        return float(value)
    import torch
    import torch.distributed as dist

    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def partition_by_sites(sites, world):
    """Split uneven members over ranks, largest first onto the least-loaded rank."""
    loads = [0] * world
    parts = [[] for _ in range(world)]
    for m in sorted(range(len(sites)), key=lambda i: -sites[i]):
        r = min(range(world), key=lambda i: loads[i])
        parts[r].append(m)
        loads[r] += sites[m]
    return [sorted(p) for p in parts]


def workload(members, precision="single", first=0):
    """Host arrays of the benchmark workload (members first .. first + members - 1):
    psi0, n0, per-member envelopes and seeds."""
    from polarism_gb300.host import make_initial_psi

    dx, dy = LX / NX, LY / NY
    x = (np.arange(NX) - (NX - 1) * 0.5) * dx
    y = (np.arange(NY) - (NY - 1) * 0.5) * dy
    rng = np.random.default_rng(1234)
    sigmas = rng.uniform(8.0, 20.0, size=first + members)[first:]
    cdt = np.complex64 if precision == "single" else np.complex128
    rdt = np.float32 if precision == "single" else np.float64
    env = np.stack([np.exp(-0.5 * (x[None, :] ** 2 + y[:, None] ** 2) / s ** 2) for s in sigmas])
    seeds = [42 + first + m for m in range(members)]
    psi = np.stack([make_initial_psi((NY, NX), 1e-3, sd, cdt, rdt) for sd in seeds])
    return dict(dx=dx, dy=dy, psi=psi[:, None], n=np.zeros((members, 1, NY, NX), rdt),
                env=env[:, None].astype(rdt), seeds=seeds, sigmas=sigmas)


PHYSICS = dict(hbar=0.6582119514, m_eff=0.284, g_C=0.001, g_R=0.002, g_I=0.0, R=0.02,
               gamma_C=0.083, gamma_R=0.005)


# ----------------------------------------------------------------------------- clocks
class ClockSampler:
    """Sample nvidia-smi clocks and throttle reasons during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.gpu_index = gpu_index
        self.proc = None
        self.lines = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu_index}", f"--query-gpu={self.QUERY}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, ValueError):
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()
        # nvidia-smi's start-up can hold the GPU for a while (seconds have been seen on a
        # GB300 machine): wait for its first sample so that this happens before the timed region.
        deadline = time.perf_counter() + 10.0
        while not self.lines and self.proc.poll() is None and time.perf_counter() < deadline:
            time.sleep(0.02)
        time.sleep(0.1)

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=5)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for name, flag in zip(names, parts[5:9]):
                if flag.lower() == "active":
                    reasons.add(name)
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)),
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peak():
    path = ROOT / "MEASURED_PEAKS.json"
    if path.exists():
        data = json.loads(path.read_text())
        return float(data["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profiled_traffic(members):
    """DRAM bytes per launch of the RK4 kernel from the committed ncu summary (profiled at
    1024^2), if any."""
    path = ROOT / "profiles" / "rk4_stream_traffic.json"
    if not path.exists() or NX != 1024:
        return None
    data = json.loads(path.read_text())
    per_site = data.get("dram_bytes_per_site")
    if per_site is None:
        return None
    return float(per_site) * members * NX * NY


def profiled_sweep_traffic(tiling, sites):
    """DRAM bytes per launch of the sweep kernel from the committed ncu summary, when the
    tile shape in use is the profiled one (the strips' pipeline fill depends on it)."""
    path = ROOT / "profiles" / "rk4_sweep_traffic.json"
    if not path.exists():
        return None
    data = json.loads(path.read_text())
    if [int(tiling["lanes"]), int(tiling["strip_rows"])] != list(data.get("tiling", [])):
        return None
    return float(data["dram_bytes_per_site"]) * sites


# ----------------------------------------------------------------------------- CPU legs
_CPU_WORK = {}


def _cpu_member_steps(args):
    """Worker: FP64 oracle RK4 steps on one member (used by the CPU legs).  Returns the time of
    the steps alone; the inputs (member 0's field and envelope; the member's own noise seed) are
    built once per worker process, so the timed region holds the stepping only."""
    member, steps, precision, n = args
    global NX, NY, LX, LY
    if NX != n:
        NX = NY = n
        LX = LY = 400.0 * n / 1024
        _CPU_WORK.clear()
    sys.path.insert(0, str(ROOT))
    from oracle import gpe

    if "w" not in _CPU_WORK:
        _CPU_WORK["w"] = workload(1, "double")
    w = _CPU_WORK["w"]
    p = dict(PHYSICS)
    env = w["env"][0, 0].astype(np.float64) * P0
    psi, fields = w["psi"].astype(np.complex128), (w["n"].astype(np.float64),)
    noise = gpe.Noise([42 + member], [p["gamma_C"]], [p["R"]], [1.0], DT, w["dx"] * w["dy"])
    t0 = time.perf_counter()
    gpe.rk4_advance(psi, fields, lambda t: env, 0.0, p, w["dx"], w["dy"], DT, 0, steps,
                    noise=noise)
    return time.perf_counter() - t0


def cpu_baseline(sample_steps=12):
    """Oracle port, one core, a bounded sample (sample_steps RK4 steps of one 1024^2 member)."""
    _cpu_member_steps((0, 1, "double", NX))  # warm-up
    elapsed = _cpu_member_steps((0, sample_steps, "double", NX))
    return {"value": sample_steps * NX * NY / elapsed, "unit": "site-updates/s", "cores": 1,
            "kind": "port",
            "sample": f"{sample_steps} RK4 steps of one {NX}^2 member, FP64 NumPy oracle "
                      "(restatement of the reference rk4-fdm + Wigner), 1 thread"}


def rk4_workload_config(args, members, world):
    """The RK4 workload's config keys, the same on both arms."""
    return {"workload": f"rk4-cuda fused step, {NX}^2 periodic, lx=ly={LX:g}, dt=5e-4, "
                        "single reservoir, Wigner noise on, complex64" +
                        (f", {args.potential} potential" if args.potential != "none" else "") +
                        (f", kinetic relaxation eta={args.eta:g}" if args.eta else ""),
            "members": members, "global_members": members * world, "grid": [NY, NX],
            "parallelism": f"replicas{world}"}


REFERENCE_ARM_BUDGET_S = 240.0  # longest the reference arm's timed steps may take


def run_reference(args):
    """--impl reference: the reference algorithm's CPU implementation on all host cores.

    A step is one RK4 step of every member (the GPU arm's step), the members spread over one
    worker process per core.  W warm-up steps and K timed steps run as asked; only when K
    steps would take longer than REFERENCE_ARM_BUDGET_S (estimated from the warm-up) does the
    arm time fewer, and the line's ``steps`` and ``same_steps`` say so."""
    import multiprocessing as mp

    rank, world, _ = dist_info()
    if rank != 0:
        return
    cores = os.cpu_count() or 1
    workers = max(1, min(args.members, cores))
    ctx = mp.get_context("spawn")
    tasks = [(m, 1, "double", NX) for m in range(args.members)]
    chunk = max(1, math.ceil(args.members / workers))
    with ctx.Pool(workers) as pool:
        # Every worker builds its inputs on its first task, outside any timed step.
        pool.map(_cpu_member_steps, [(m, 1, "double", NX) for m in range(workers)], chunksize=1)
        warm = max(1, args.warmup)
        t0 = time.perf_counter()
        for k in range(warm):
            pool.map(_cpu_member_steps, tasks, chunksize=chunk)
            if time.perf_counter() - t0 > REFERENCE_ARM_BUDGET_S / 4:
                warm = k + 1
                break
        per_step = (time.perf_counter() - t0) / warm
        steps = max(1, min(args.steps, int(REFERENCE_ARM_BUDGET_S // max(per_step, 1e-9))))
        t0 = time.perf_counter()
        for _ in range(steps):
            pool.map(_cpu_member_steps, tasks, chunksize=chunk)
        elapsed = time.perf_counter() - t0
    value = steps * args.members * NX * NY / elapsed
    line = {
        "metric": METRIC, "value": value, "unit": "site-updates/s", "n_gpus": world,
        "steps": steps, "warmup": warm, "same_steps": steps == args.steps and warm == args.warmup,
        "ms_per_step": 1e3 * elapsed / steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "impl": "reference",
        "config": dict(rk4_workload_config(args, args.members, world),
                       kernel="reference CPU path (FP64 NumPy port of rk4-fdm + Wigner)"),
        "cpu_baseline": {"value": value, "unit": "site-updates/s", "cores": workers, "kind": "port",
                         "sample": f"{steps} RK4 steps of {args.members} members at {NX}^2 after "
                                   f"{warm} warm-up steps, FP64 NumPy oracle port, {workers} "
                                   "worker processes"},
        "e2e": {"value": value, "unit": "site-updates/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ----------------------------------------------------------------------------- GPU leg
def run_ours(args):
    import torch

    rank, world, local = dist_info()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    from polarism_gb300 import build as _build

    _build.build()
    from polarism_gb300.engine import MemberPhysics, RK4Engine

    members = args.members
    w = workload(members, first=rank_members(rank, world, members)[0])
    from polarism_gb300 import _lib

    pot_kind = {"none": _lib.PG_POT_NONE, "real": _lib.PG_POT_REAL,
                "complex": _lib.PG_POT_COMPLEX}[args.potential]
    physics = dict(PHYSICS, kinetic_relaxation_eta=args.eta)
    eng = RK4Engine(NX, NY, members, w["dx"], w["dy"], DT, MemberPhysics(**physics), "single",
                    pump_per_member=True, potential=pot_kind)
    if args.rk4_kernel != "auto":
        eng.set_kernel({"wide": 2, "tiled": 1, "wide4": 3}[args.rk4_kernel])
    kernel_name = ("tiled" if eng.kernel() == 1 else
                   "full-width, four sites a thread" if eng.kernel() == 3 else
                   "full-width" if NX <= 1024 else
                   f"full-width, clusters of {NX // 1024} CTAs (1024-site bands)" if NX <= 8192 else
                   "full-width, 1024-site bands with recomputed halo")
    eng.set_pump(w["env"])
    if args.potential != "none":
        # A harmonic trap (real part) and an absorbing rim (imaginary part), shared by members.
        x = (np.arange(NX) - (NX - 1) * 0.5) * w["dx"]
        y = (np.arange(NY) - (NY - 1) * 0.5) * w["dy"]
        r2 = x[None, :] ** 2 + y[:, None] ** 2
        trap = 1e-4 * r2
        if args.potential == "complex":
            rim = -0.5 * np.clip(np.sqrt(r2) / (0.5 * LX) - 0.9, 0.0, None)
            eng.set_potential((trap + 1j * rim).astype(np.complex64))
        else:
            eng.set_potential(trap.astype(np.float32))
    eng.set_noise(w["seeds"], PHYSICS["gamma_C"], PHYSICS["R"], 1.0, DT / (4 * w["dx"] * w["dy"]))
    eng.set_state(w["psi"], w["n"])
    stream = torch.cuda.ExternalStream(eng.stream)
    total = args.warmup + args.steps
    scales = np.full((total, 3, members), P0)

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            import torch.distributed as dist

            dist.barrier()
        torch.cuda.synchronize()

    eng.advance(0, args.warmup, scales[:args.warmup])
    # The timed call's CUDA graphs are built here (capture and instantiation are one-time
    # set-up costs of a long run, not per-step work); the timed region replays them.
    eng.prepare(args.steps)
    barrier()
    sampler = ClockSampler(local)
    sampler.start()
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier()
    start.record(stream)
    eng.advance(args.warmup, args.steps, scales[args.warmup:])
    stop.record(stream)
    barrier()
    clocks = sampler.stop()
    launches = eng.last_launch_count
    elapsed_ms = max_over_ranks(start.elapsed_time(stop), world, "cuda")
    sites = members * NX * NY
    value = world * sites * args.steps / (elapsed_ms / 1e3)
    kernel_s = elapsed_ms / 1e3 / args.steps
    bytes_per_site = BYTES_PER_SITE + {"none": 0, "real": 4, "complex": 8}[args.potential]
    achieved = bytes_per_site * sites / kernel_s / 1e9
    peak, peak_kind = measured_peak()
    traffic = profiled_traffic(members) if args.potential == "none" and args.eta == 0.0 else None

    # End to end through the public solver API on pinned host state.
    e2e = run_e2e(args, w, members, torch)
    if args.potential != "none" or args.eta:
        e2e["step"] += " (without the potential / relaxation: the host mirror's configs have none)"
    eng.close()
    if rank != 0:
        return
    line = {
        "metric": METRIC, "value": value, "unit": "site-updates/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": elapsed_ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": dict(rk4_workload_config(args, members, world), kernel=kernel_name,
                       l2="inputs larger than L2 (%.0f MB state vs 129 MB L2)" % (sites * 16 / 1e6),
                       graphs="CUDA graphs of the timed call built before the timed region "
                              "(pg_rk4_prepare); the timed region replays them"),
        "gpu_launches": launches,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic, "peak_source": peak_kind,
                     "algorithmic_bytes_per_site": bytes_per_site},
        "e2e": e2e,
        "clocks": clocks,
    }
    if world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(args.cpu_sample_steps)
    print(json.dumps(line), flush=True)


def run_e2e(args, w, members, torch):
    """Steps/s through RK4CudaSolver.advance with pinned host state (64-step calls)."""
    from polarism_gb300.host import Config, build_simulation
    from polarism_gb300.solvers import RK4CudaSolver

    cfg = Config()
    cfg.grid.nx, cfg.grid.ny, cfg.grid.lx, cfg.grid.ly = NX, NY, LX, LY
    cfg.solver.dt, cfg.solver.precision = DT, "single"
    cfg.noise.stochastic, cfg.noise.seed = "wigner", 42
    cfg.laser.P0 = P0
    member_cfgs = []
    import copy

    for m in range(members):
        c = copy.deepcopy(cfg)
        c.noise.seed = int(w["seeds"][m])
        c.laser.sigma_space = float(w["sigmas"][m])
        member_cfgs.append(c)
    grid, model, state = build_simulation(cfg, member_cfgs if members > 1 else None)
    pinned_psi = torch.empty(state.field.shape, dtype=torch.complex64, pin_memory=True).numpy()
    pinned_psi[...] = state.field
    state.field = pinned_psi
    pinned_n = torch.empty(model.reservoir.nR.shape, dtype=torch.float32, pin_memory=True).numpy()
    pinned_n[...] = model.reservoir.nR
    model.reservoir.nR = pinned_n
    solver = RK4CudaSolver(cfg, grid, model)
    solver.inplace_host = True  # results land in the same pinned arrays every call
    chunk = 64
    solver.advance(model, state, chunk)  # warm-up: uploads pump/noise, captures graphs

    calls = max(2, args.e2e_calls)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(calls):
        solver.advance(model, state, chunk)
    elapsed = time.perf_counter() - t0
    sites = members * NX * NY
    per_call = sites * (8 + 4)  # psi (complex64) and n_R (float32), each way, every call
    return {"value": sites * chunk * calls / elapsed, "unit": "site-updates/s",
            "h2d_bytes_per_step": per_call / chunk, "d2h_bytes_per_step": per_call / chunk,
            "h2d_bytes_per_call": per_call, "d2h_bytes_per_call": per_call,
            "step": f"{calls} RK4CudaSolver.advance calls of {chunk} RK4 steps each on pinned "
                    "host state (bytes per step = bytes per call / steps per call)",
            "calls": calls, "steps_per_call": chunk}


# ----------------------------------------------------------------------------- split-step leg
SPLIT_BYTES = {"kouter": 44, "cpu": 76}  # FP32 algorithmic bytes per site-update


def run_split_bench(args):
    """Split-step Fourier throughput at 1024^2 (the precision-check configuration stepped by
    split-step-fft-cuda, or split-step-fft with --split-ordering cpu): members x 1024^2 FP32,
    Wigner noise on, site-updates/s against the HBM roofline at 44 B/site (K-outer: one column
    pass and one row pass per step, each reading and writing psi, plus the reservoir and the
    pump in the column pass) or 76 B/site (CPU ordering: two of each pass)."""
    import torch

    rank, world, local = dist_info()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    from polarism_gb300 import build as _build

    _build.build()
    from polarism_gb300.engine import MemberPhysics, RK4Engine

    ordering = args.split_ordering
    members = args.members
    w = workload(members, first=rank_members(rank, world, members)[0])
    eng = RK4Engine(NX, NY, members, w["dx"], w["dy"], DT, MemberPhysics(**PHYSICS), "single",
                    pump_per_member=True)
    eng.set_pump(w["env"])
    eng.set_noise(w["seeds"], PHYSICS["gamma_C"], PHYSICS["R"], 1.0, DT / (4 * w["dx"] * w["dy"]))
    eng.set_state(w["psi"], w["n"])
    stream = torch.cuda.ExternalStream(eng.stream)
    code = 1 if ordering == "kouter" else 0
    half = np.full((args.warmup + args.steps, 2, members), P0)

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            import torch.distributed as dist

            dist.barrier()
        torch.cuda.synchronize()

    eng.split_advance(code, 0, args.warmup, half[:args.warmup])
    eng.split_prepare(code, args.steps)  # the timed call's graphs, built before timing
    barrier()
    sampler = ClockSampler(local)
    sampler.start()
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier()
    start.record(stream)
    eng.split_advance(code, args.warmup, args.steps, half[args.warmup:])
    stop.record(stream)
    barrier()
    clocks = sampler.stop()
    launches = eng.last_launch_count
    elapsed_ms = max_over_ranks(start.elapsed_time(stop), world, "cuda")
    sites = members * NX * NY
    value = world * sites * args.steps / (elapsed_ms / 1e3)
    bytes_per_site = SPLIT_BYTES[ordering]
    achieved = bytes_per_site * sites / (elapsed_ms / 1e3 / args.steps) / 1e9
    peak, peak_kind = measured_peak()

    # End to end: host state in (pinned), 64 steps, host state out, every call.
    psi_host = torch.empty(w["psi"].shape, dtype=torch.complex64, pin_memory=True).numpy()
    n_host = torch.empty(w["n"].shape, dtype=torch.float32, pin_memory=True).numpy()
    psi_host[...] = w["psi"]
    n_host[...] = w["n"]
    chunk = 64
    calls = max(2, args.e2e_calls)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for c in range(calls):
        eng.set_state(psi_host, n_host)
        eng.set_state_kind(False)
        eng.split_advance(code, c * chunk, chunk, np.full((chunk, 2, members), P0))
        eng.get_state(psi_host, n_host)  # K-outer leaves the spectrum, read back as it is
    e2e_s = time.perf_counter() - t0
    eng.close()
    if rank != 0:
        return
    line = {
        "metric": f"split-step site-updates/s at {NX}^2 ({ordering} ordering)", "value": value,
        "unit": "site-updates/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": elapsed_ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": ("split-step-fft-cuda (K/2 [R/2 N R/2] K/2)" if code == 1 else
                                "split-step-fft (R/2 K/2 N K/2 R/2)") +
                               f", {NX}^2 periodic, lx=ly={LX:g}, dt=5e-4, single reservoir, "
                               "Wigner noise on, complex64",
                   "members": members, "global_members": members * world, "grid": [NY, NX],
                   "parallelism": f"replicas{world}",
                   "l2": "inputs larger than L2 (%.0f MB state vs 129 MB L2)" % (sites * 16 / 1e6)},
        "gpu_launches": launches,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": None, "peak_source": peak_kind,
                     "algorithmic_bytes_per_site": bytes_per_site},
        "e2e": {"value": sites * chunk * calls / e2e_s, "unit": "site-updates/s",
                "h2d_bytes_per_step": sites * 12 / chunk, "d2h_bytes_per_step": sites * 12 / chunk,
                "h2d_bytes_per_call": sites * 12, "d2h_bytes_per_call": sites * 12,
                "step": f"{calls} calls of set_state + {chunk} split steps + get_state from pinned "
                        "host arrays (bytes per step = bytes per call / steps per call)",
                "calls": calls, "steps_per_call": chunk},
        "clocks": clocks,
    }
    if world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = split_cpu_baseline(ordering)
    print(json.dumps(line), flush=True)


def split_cpu_baseline(ordering, sample_steps=4):
    """Oracle port, one core: sample_steps split steps of one 1024^2 member (FP64 NumPy)."""
    from oracle import gpe

    w = workload(1, "double")
    p = dict(PHYSICS)
    env = w["env"][0, 0].astype(np.float64) * P0
    kx = 2 * np.pi * np.fft.fftfreq(NX, d=w["dx"])
    ky = 2 * np.pi * np.fft.fftfreq(NY, d=w["dy"])
    k2 = kx[None, :] ** 2 + ky[:, None] ** 2
    psi, fields = w["psi"].astype(np.complex128), (w["n"].astype(np.float64),)
    noise = gpe.Noise([42], [p["gamma_C"]], [p["R"]], [1.0], DT, w["dx"] * w["dy"])
    gpe.split_advance(ordering, psi.copy(), fields, lambda t: env, 0.0, p, k2, w["dx"], w["dy"],
                      DT, 0, 1, noise=noise)
    t0 = time.perf_counter()
    gpe.split_advance(ordering, psi, fields, lambda t: env, 0.0, p, k2, w["dx"], w["dy"], DT, 0,
                      sample_steps, noise=noise)
    elapsed = time.perf_counter() - t0
    return {"value": sample_steps * NX * NY / elapsed, "unit": "site-updates/s", "cores": 1,
            "kind": "port",
            "sample": f"{sample_steps} split steps ({ordering} ordering) of one 1024^2 member, "
                      "FP64 NumPy oracle, 1 thread"}


# ----------------------------------------------------------------------------- sweep leg
SWEEP_SIZES = (128, 256, 512)
SWEEP_DX = 100.0 / 128  # lx scaled with nx so every member has the same cell


def sweep_members(members):
    """Uneven-size sweep workload: sizes cycle 128^2 / 256^2 / 512^2 (a third each, the same
    dx), P0 uniform in [0.5, 3] x threshold, sigma uniform in [8, 20] um, seeds 0..members-1
    (parameters drawn from numpy default_rng(1234)); single reservoir, no Wigner noise (the
    steady-state criterion needs a deterministic run)."""
    from polarism_gb300 import host

    rng = np.random.default_rng(1234)
    p_th = PHYSICS["gamma_R"] * PHYSICS["gamma_C"] / PHYSICS["R"]
    p0 = rng.uniform(0.5, 3.0, size=members) * p_th
    sigma = rng.uniform(8.0, 20.0, size=members)
    cfgs = []
    for m in range(members):
        c = host.Config()
        n = SWEEP_SIZES[m % 3]
        c.grid.nx = c.grid.ny = n
        c.grid.lx = c.grid.ly = n * SWEEP_DX
        c.solver.dt, c.solver.precision, c.solver.total_time = 1e-3, "single", 1000.0
        c.noise.seed, c.noise.stochastic = m, "none"
        c.laser.P0, c.laser.sigma_space = float(p0[m]), float(sigma[m])
        c.stop.steady_state, c.stop.rtol, c.stop.check_every = True, 1e-6, 10.0
        cfgs.append(c)
    return cfgs


def run_sweep_bench(args):
    """Device throughput of the one-launch uneven sweep (site-updates/s over all members)."""
    import torch

    rank, world, local = dist_info()
    torch.cuda.set_device(local)
    from polarism_gb300 import build as _build

    _build.build()
    from polarism_gb300.engine import MemberPhysics
    from polarism_gb300.sweep import SweepEngine, _member_inputs, autotune_tiling, run_sweep

    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    cfgs_all = sweep_members(args.members)
    sites_all = [c.grid.nx * c.grid.ny for c in cfgs_all]
    # Several GPUs: members are independent, so each rank takes a site-balanced share.
    mine = partition_by_sites(sites_all, world)[rank] if world > 1 else list(range(len(cfgs_all)))
    cfgs = [cfgs_all[m] for m in mine]
    inputs = [_member_inputs(c) for c in cfgs]
    grids = [(g.nx, g.ny, g.dx, g.dy) for g, *_ in inputs]
    eng = SweepEngine(grids, [MemberPhysics(**PHYSICS)] * len(cfgs), 1e-3)
    eng.set_pump([laser._spatial_envelope for _, laser, *_ in inputs])
    psi0 = [p for _, _, p, _, _ in inputs]
    n0 = [np.zeros((g.ny, g.nx), np.float32) for g, *_ in inputs]
    eng.set_state(psi0, n0)
    if args.sweep_tiling:
        eng.set_tiling(*args.sweep_tiling)
        tune = {"timings": None}
    else:
        tune = autotune_tiling(eng, noise=False, use_cache=False, steps=32)
    p0 = np.asarray([c.laser.P0 for c in cfgs])
    total = args.warmup + args.steps
    scales = np.broadcast_to(p0, (total, 3, len(cfgs))).copy()
    eng.advance(0, args.warmup, scales[:args.warmup])
    eng.synchronize()
    sampler = ClockSampler(local)
    sampler.start()
    eng.advance(args.warmup, args.steps, scales[args.warmup:])
    elapsed_ms = max_over_ranks(eng.last_time_ms(), world, "cuda")
    clocks = sampler.stop()
    launches = eng.last_launch_count
    sites = eng.sites
    value = sum(sites_all) * args.steps / (elapsed_ms / 1e3)
    achieved = BYTES_PER_SITE * sites / (elapsed_ms / 1e3 / args.steps) / 1e9
    peak, peak_kind = measured_peak()

    # End to end through SweepEngine with host arrays: upload, 64 steps, download.
    chunk = 64
    psi_h, n_h = eng.get_packed_state()
    t0 = time.perf_counter()
    calls = 4
    for c in range(calls):
        eng.set_state([eng.unpack(psi_h, m) for m in range(eng.members)],
                      [eng.unpack(n_h, m) for m in range(eng.members)])
        eng.advance(total + c * chunk, chunk, np.broadcast_to(p0, (chunk, 3, len(cfgs))).copy())
        psi_h, n_h = eng.get_packed_state()
    e2e_s = time.perf_counter() - t0
    line = {
        "metric": "sweep RK4 site-updates/s (uneven sizes, one persistent launch per step)",
        "value": value, "unit": "site-updates/s", "n_gpus": world, "steps": args.steps,
        "scaling_note": "members split over ranks by sites (strong scaling of one sweep)" if world > 1 else None,
        "warmup": args.warmup, "ms_per_step": elapsed_ms / args.steps, "higher_is_better": True,
        "scaling": "strong" if world > 1 else "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": f"uneven sweep: {len(cfgs_all)} members, 128^2/256^2/512^2 a third each, "
                               "dx fixed, P0 in [0.5,3] x threshold, sigma in [8,20] um, seeds "
                               "0..N-1, single reservoir, dt=1e-3, complex64",
                   "members": len(cfgs), "sites": sites, "tiling": eng.tiling,
                   "autotune_ms_per_step": tune["timings"],
                   "l2": "inputs larger than L2 (%.0f MB state vs 129 MB L2)" % (sites * 16 / 1e6)},
        "gpu_launches": launches,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak,
                     "traffic": profiled_sweep_traffic(eng.tiling, sites),
                     "peak_source": peak_kind,
                     "algorithmic_bytes_per_site": BYTES_PER_SITE},
        "e2e": {"value": sites * chunk * calls / e2e_s, "unit": "site-updates/s",
                "h2d_bytes_per_step": sites * 12, "d2h_bytes_per_step": sites * 12,
                "step": f"SweepEngine set_state + {chunk} steps + get_state from host arrays"},
        "clocks": clocks,
    }
    eng.close()
    if args.steady_time > 0:
        for c in cfgs:
            c.solver.total_time = args.steady_time
        res = run_sweep(cfgs, autotune=True, freeze_stopped=args.freeze_stopped)
        line["steady_state"] = {
            "wall_s": res.wall_time, "t_end_ps": res.t, "steps": res.steps,
            "stopped": int(np.isfinite(res.stop_times).sum()), "members": len(cfgs),
            "stop_time_ps_median": float(np.nanmedian(res.stop_times)) if np.isfinite(res.stop_times).any() else None,
            "freeze_stopped": bool(args.freeze_stopped), "rtol": 1e-6, "check_every_ps": 10.0,
            "host_waits_before_first_decision": res.loop_syncs,
            "stop_times_ps": [None if not np.isfinite(v) else float(v) for v in res.stop_times]}
    if rank == 0:
        print(json.dumps(line), flush=True)


# ----------------------------------------------------------------------------- IFRK leg
# Classical RK4 in Butcher form (the tableau pg_ifrk_advance runs as "rk4").
IFRK4_A = ((), (0.5,), (0.0, 0.5), (0.0, 0.0, 1.0))
IFRK4_B = (1 / 6, 1 / 3, 1 / 3, 1 / 6)


def ifrk_bytes_per_site(A, b, complex_bytes=8, real_bytes=4):
    """Bytes per site and step that the Lawson IFRK pass structure of ``csrc/api_ifrk.cu``
    reads and writes in DRAM (scalar field, single reservoir, one laser, no potential).  W is
    the y-transformed field the passes hand on; stage i's row pass reads W, stores the stage's
    transformed row (psi0_hat at stage 0, f_hat_{i-1} after), reads psi0_hat (i > 0) and every
    earlier f_hat_j with a_ij != 0 except the one it has just formed, writes W; its column pass
    reads W, n_0, the pump envelope and dn_j for a_ij != 0, writes dn_i and W.  The final row
    pass combines psi0_hat and the f_hat_j with b_j != 0; the final column pass reads dn_j,
    writes n_1, psi_1 and W.  The Lawson tables (nx + ny values per factor) stay in cache."""
    c, r = complex_bytes, real_bytes
    s = len(b)
    total = 0
    for i in range(s):
        row = 3 * c + (c if i > 0 else 0) + c * sum(1 for j in range(i - 1) if A[i][j] != 0.0)
        col = 2 * c + r + r + r * sum(1 for j in range(i) if A[i][j] != 0.0) + r
        total += row + col
    final_row = 4 * c + c * sum(1 for j in range(s - 1) if b[j] != 0.0)
    final_col = 3 * c + r + r * sum(1 for j in range(s) if b[j] != 0.0) + r
    return total + final_row + final_col


def run_ifrk_bench(args):
    """Fixed-step Lawson IFRK4 (ifrk4-fft-cuda) throughput at 1024^2: members x 1024^2 FP32,
    single reservoir, Wigner noise on, site-updates/s against the HBM roofline at the pass
    structure's bytes per site (ifrk_bytes_per_site)."""
    import torch

    rank, world, local = dist_info()
    torch.cuda.set_device(local)
    from polarism_gb300 import build as _build

    _build.build()
    from polarism_gb300.engine import TABLEAU_NODES, MemberPhysics, RK4Engine

    members = args.members
    w = workload(members, first=rank_members(rank, world, members)[0])
    eng = RK4Engine(NX, NY, members, w["dx"], w["dy"], DT, MemberPhysics(**PHYSICS), "single",
                    pump_per_member=True)
    eng.set_pump(w["env"])
    eng.set_noise(w["seeds"], PHYSICS["gamma_C"], PHYSICS["R"], 1.0, DT / (4 * w["dx"] * w["dy"]))
    eng.set_state(w["psi"], w["n"])
    stream = torch.cuda.ExternalStream(eng.stream)
    stages = len(TABLEAU_NODES["rk4"])
    scales = np.full((args.warmup + args.steps, stages, members), P0)
    eng.ifrk_advance("rk4", 0, args.warmup, scales[:args.warmup])
    torch.cuda.synchronize()
    sampler = ClockSampler(local)
    sampler.start()
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    start.record(stream)
    eng.ifrk_advance("rk4", args.warmup, args.steps, scales[args.warmup:])
    stop.record(stream)
    torch.cuda.synchronize()
    clocks = sampler.stop()
    launches = eng.last_launch_count
    elapsed_ms = start.elapsed_time(stop)
    eng.close()
    sites = members * NX * NY
    value = sites * args.steps / (elapsed_ms / 1e3)
    bytes_per_site = ifrk_bytes_per_site(IFRK4_A, IFRK4_B)
    achieved = bytes_per_site * sites / (elapsed_ms / 1e3 / args.steps) / 1e9
    peak, peak_kind = measured_peak()
    line = {
        "metric": f"IFRK4 site-updates/s at {NX}^2 (fixed step)", "value": value,
        "unit": "site-updates/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": elapsed_ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"ifrk4-fft-cuda (Lawson RK4, fixed dt=5e-4), {NX}^2 periodic, "
                               f"lx=ly={LX:g}, single reservoir, Wigner noise on, complex64",
                   "members": members, "grid": [NY, NX],
                   "l2": "inputs larger than L2 (%.0f MB state vs 129 MB L2)" % (sites * 16 / 1e6)},
        "gpu_launches": launches,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": None, "peak_source": peak_kind,
                     "algorithmic_bytes_per_site": bytes_per_site},
        "clocks": clocks,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


# ----------------------------------------------------------------------------- spinor leg
SPINOR_N = 512
SPINOR_L = 128.0          # um: dx = 0.25 um, the ring (r = 30, w = 4) well inside the box
SPINOR_TE_TM = 0.05       # meV um^2 (the config leaves beta open; this value is ours)


def spinor_setup(precision="single"):
    """Config 3: circular-basis spinor with TE-TM (beta = 0.05 meV um^2), Zeeman 0.05 meV,
    alpha_2 = -0.1 g_C, double reservoir per component, ring pump (r = 30 um, w = 4 um),
    linear polarisation, P0 = 1.5 x threshold (the double-reservoir threshold with n_A = gamma_C/R
    at psi = 0 and half the pump per component), 512^2 periodic, lx = ly = 128 um."""
    from polarism_gb300 import host

    cfg = host.Config()
    cfg.grid.nx = cfg.grid.ny = SPINOR_N
    cfg.grid.lx = cfg.grid.ly = SPINOR_L
    cfg.solver.precision, cfg.solver.dt, cfg.solver.tableau = precision, 0.1, "dp5"
    cfg.solver.adaptive, cfg.solver.rtol, cfg.solver.atol = True, 1e-6, 1e-8
    cfg.reservoir.reservoir_type = "double"
    ph = cfg.physics
    ph.spin, ph.zeeman, ph.te_tm, ph.alpha_2 = "spinor", 0.05, SPINOR_TE_TM, -0.1 * ph.g_C
    n_a = ph.gamma_C / ph.R
    per_component = ((ph.gamma_I + ph.R_IA) * (ph.gamma_A + ph.R_AI) / ph.R_IA - ph.R_AI) * n_a
    p_th = 2.0 * per_component
    cfg.laser.laser_type, cfg.laser.P0 = "profile", 1.5 * p_th
    cfg.laser.profile = {"type": "ring", "radius": 30.0, "width": 4.0}
    cfg.laser.circular_polarization = 0.0
    cfg.noise.seed = 0
    return cfg, p_th


def run_spinor_bench(args):
    """Adaptive DP5 spinor run to --spinor-time ps with FP64 observable accumulation every ps
    after the first fifth of the run; device-resident (engine API)."""
    import torch

    rank, world, local = dist_info()
    torch.cuda.set_device(local)
    from polarism_gb300 import build as _build

    _build.build()
    from polarism_gb300 import host
    from polarism_gb300.engine import TABLEAU_NODES, Engine, MemberPhysics
    from polarism_gb300.step_control import StepController

    cfg, p_th = spinor_setup()
    grid, model, state = host.build_simulation(cfg)
    phys = MemberPhysics.from_object(cfg.physics)
    phys.pump_weight_plus = phys.pump_weight_minus = 0.5
    eng = Engine(grid.nx, grid.ny, 1, grid.dx, grid.dy, cfg.solver.dt, phys, "single",
                 reservoir="double", components=2, reservoir_components=2)
    eng.set_pump(model.pump.lasers[0]._spatial_envelope.astype(np.float32))
    eng.set_state(state.field.astype(np.complex64),
                  np.stack([f.astype(np.float32) for f in model.reservoir.get_state()]))
    ctl = StepController(cfg.solver.dt)
    nodes = TABLEAU_NODES["dp5"]
    scales = np.full((len(nodes), 1), cfg.laser.P0)
    total = float(args.spinor_time)
    sample_from = 0.2 * total
    sites = 2 * grid.nx * grid.ny
    t, next_sample, samples = 0.0, sample_from, 0
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    sampler = ClockSampler(local)
    sampler.start()
    while t < total - 1e-12:
        target = min(total, math.floor(t + 1.0 + 1e-9))
        while t < target - 1e-12:
            h, clamped, proposal = ctl.propose(t, target)
            err, acc = eng.ifrk_trial(h, scales, cfg.solver.rtol, cfg.solver.atol)
            if acc:
                t = target if clamped else t + h
            ctl.update(h, clamped, proposal, acc, err)
        if t >= next_sample - 1e-9:
            eng.accumulate(density=True, momentum=True)
            samples += 1
            next_sample += 1.0
    eng.synchronize()
    wall = time.perf_counter() - t0
    clocks = sampler.stop()
    norms = eng.norms()
    line = {
        "metric": "spinor DP5 accepted site-updates/s (config 3)",
        "value": ctl.accepted * sites / wall, "unit": "site-updates/s", "n_gpus": world,
        "higher_is_better": True, "dtype": "f32 state, f64 error norm and observables",
        "data": "synthetic",
        "config": {"workload": "spinor 512^2, lx=ly=128 um, TE-TM beta=0.05 meV um^2, Zeeman 0.05 meV, "
                               "alpha_2=-0.1 g_C, double reservoir per component, ring r=30 w=4, "
                               "linear polarisation, P0=1.5 P_th, IFRK dp5 rtol 1e-6",
                   "p_th": p_th, "P0": cfg.laser.P0, "t_end_ps": t},
        "wall_s": wall, "ps_per_s": t / wall, "trials_accepted": ctl.accepted,
        "trials_rejected": ctl.rejected, "observable_samples": samples,
        "final_norm": float(norms[0]), "clocks": clocks,
    }
    line["observables"] = spinor_observables(eng, grid, samples, args.observables_out)
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = spinor_cpu_baseline(cfg, grid, model, state)
    eng.close()
    if rank == 0:
        print(json.dumps(line), flush=True)


def spinor_observables(eng, grid, samples, out_path=None):
    """The run's FP64 accumulators finalised into Polarism's observables (momentum
    distribution n(k), g1(r), <n>, g2) per circular component, summarised; with ``out_path``
    the full arrays are written there (npz)."""
    from polarism_gb300 import observables as ob

    if samples == 0:
        return None
    sum_rho, s_rho = eng.accumulator_sums("rho")
    sum_rho2, _ = eng.accumulator_sums("rho2")
    sum_k, s_k = eng.accumulator_sums("k")
    cell, cells = grid.dx * grid.dy, grid.nx * grid.ny
    n_k = ob.momentum_distribution(sum_k, s_k, cell, cells)[0]   # (2, ny, nx), centred
    g1 = ob.g1(n_k)
    mean, sq = ob.density_moments(sum_rho, sum_rho2, s_rho)
    g2 = ob.g2(mean, sq)[0]
    mean = mean[0]
    kx = np.fft.fftshift(2 * np.pi * np.fft.fftfreq(grid.nx, grid.dx))
    ky = np.fft.fftshift(2 * np.pi * np.fft.fftfreq(grid.ny, grid.dy))
    x = (np.arange(grid.nx) - grid.nx // 2) * grid.dx
    y = (np.arange(grid.ny) - grid.ny // 2) * grid.dy
    r = np.hypot(x[None, :], y[:, None])
    out = {"samples": int(samples), "components": []}
    for c, name in enumerate(("psi_plus", "psi_minus")):
        peak = np.unravel_index(int(np.argmax(n_k[c])), n_k[c].shape)
        core = mean[c] > 0.1 * mean[c].max()
        g1_r = {f"{d:g}um": float(np.mean(np.abs(g1[c][(r >= d - 0.5 * grid.dx) & (r < d + 0.5 * grid.dx)])))
                for d in (2.0, 5.0, 10.0, 20.0, 40.0)}
        out["components"].append({
            "component": name,
            "particles": float(mean[c].sum() * cell),
            "n_k_peak": float(n_k[c][peak]), "k_peak_per_um": [float(kx[peak[1]]), float(ky[peak[0]])],
            "n_k_total": float(n_k[c].sum()),
            "g1_abs_ring_mean": g1_r,
            "g2_condensate_mean": float(np.mean(g2[c][core])) if core.any() else None,
            "g2_at_density_max": float(g2[c].reshape(-1)[int(np.argmax(mean[c]))]),
        })
    if out_path:
        np.savez_compressed(out_path, n_k=n_k, g1=g1, mean_density=mean, g2=g2, kx=kx, ky=ky,
                            samples=samples)
        out["arrays"] = str(out_path)
    return out


def spinor_cpu_baseline(cfg, grid, model, state, trials=2):
    """FP64 NumPy oracle (the reference's generic Lawson path restated) on one core: a bounded
    sample of adaptive DP5 trials of the same 512^2 spinor."""
    from oracle import gpe

    p = {k: getattr(cfg.physics, k) for k in ("hbar", "m_eff", "g_C", "g_R", "g_I", "R", "gamma_C",
                                              "gamma_R", "gamma_I", "gamma_A", "R_IA", "R_AI",
                                              "alpha_2", "zeeman", "te_tm")}
    spin = {"kx": grid.KX, "ky": grid.KY, "weights": model.pump_weights.reshape(-1, 2)}
    pump = model.pump.lasers[0]._spatial_envelope * cfg.laser.P0
    st = gpe.IFRKState(psi=state.field.astype(np.complex128),
                       fields=tuple(f.astype(np.float64) for f in model.reservoir.get_state()))
    t0 = time.perf_counter()
    for _ in range(trials):
        gpe.ifrk_step(st, cfg.solver.dt, gpe.DP5_TABLEAU, lambda t: pump, 0.0, p, grid.k_squared,
                      grid.dx, grid.dy, kind="double", adaptive=True, rtol=1e-6, atol=1e-8,
                      spinor=spin)
    elapsed = time.perf_counter() - t0
    sites = 2 * grid.nx * grid.ny
    return {"value": trials * sites / elapsed, "unit": "site-updates/s", "cores": 1, "kind": "port",
            "sample": f"{trials} DP5 trials of the 512^2 spinor, FP64 NumPy oracle, 1 thread"}


# ----------------------------------------------------------------------------- warm-start leg
def run_fno_bench(args):
    """Config 5: solver-made steady states of random pumps at --fno-n^2, FNO training with the
    BF16 tensor-core kernels, then held-out members started plain and warm (time to the
    steady-state criterion, steady density within 1e-3)."""
    import torch

    rank, world, local = dist_info()
    torch.cuda.set_device(local)
    from polarism_gb300 import build as _build

    _build.build()
    from polarism_gb300 import warmstart as ws

    n = args.fno_n
    kinds = tuple(args.fno_kinds.split(","))
    train_cfgs = ws.pump_members(args.fno_train, seed=11, n=n, total_time=args.fno_time, dt=args.fno_dt,
                                 kinds=kinds, precision=args.fno_precision)
    test_cfgs = ws.pump_members(args.fno_test, seed=12, n=n, total_time=args.fno_time, dt=args.fno_dt,
                                kinds=kinds, precision=args.fno_precision)
    t0 = time.perf_counter()
    data = ws.run_uniform(train_cfgs)
    gen_s = time.perf_counter() - t0
    # Lasing members that became stationary (decayed members have nothing to learn); with
    # --fno-targets final every member's final state is a target (short profiling runs).
    lasing = data.final_norms > 1e-6
    keep = np.ones_like(lasing) if args.fno_targets == "final" else np.isfinite(data.stop_times) & lasing
    print(f"training runs: {len(train_cfgs)} members, {int(lasing.sum())} lasing, {int(keep.sum())} "
          f"reached the criterion, {gen_s:.1f} s", file=sys.stderr, flush=True)
    if not keep.any():
        raise SystemExit("no training targets: no member reached a lasing steady state")
    a = ws.features([c for c, k in zip(train_cfgs, keep) if k])
    y = ws.targets([p for p, k in zip(data.psi, keep) if k], [r for r, k in zip(data.reservoir, keep) if k])
    model = ws.WarmStart(n, width=args.fno_width, modes=args.fno_modes)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    losses = model.fit(a, y, epochs=args.fno_epochs, batch=min(args.fno_batch, len(a)), lr=args.fno_lr)
    torch.cuda.synchronize()
    train_s = time.perf_counter() - t1
    print(f"training: {len(a)} states, {args.fno_epochs} epochs, {time.perf_counter() - t1:.1f} s, loss "
          f"{losses[0]:.3e} -> {np.mean(losses[-10:]):.3e}", file=sys.stderr, flush=True)
    plain = ws.run_uniform(test_cfgs)
    ev = ws.evaluate(model, test_cfgs, plain)
    valid = np.isfinite(ev.plain_time) & (plain.final_norms > 1e-6)
    test_kinds = [c.laser.profile["type"] for c in test_cfgs]
    train_kinds = [c.laser.profile["type"] for c in train_cfgs]
    by_kind = {k: {"train": train_kinds.count(k), "train_steady": int(sum(1 for c, q in zip(train_kinds, keep) if c == k and q)),
                   "test": test_kinds.count(k), "test_plain_steady": int(sum(1 for c, q in zip(test_kinds, valid) if c == k and q)),
                   "accepted": int(sum(1 for c, q, v in zip(test_kinds, ev.accepted, valid) if c == k and q and v))}
               for k in kinds}
    line = {
        "metric": "sweep time-to-steady-state, plain start / warm start (config 5)",
        "value": ev.speedup_time, "unit": "x (simulated time)", "n_gpus": world,
        "higher_is_better": True,
        "dtype": f"{'f64' if args.fno_precision == 'double' else 'f32'} solver, bf16 network with f32 accumulate",
        "data": "synthetic (solver-generated steady states)",
        "config": {"workload": f"{n}^2, lx=ly=128 um, dt={args.fno_dt} ps, pumps gaussian/ring/square lattice, "
                               "P0 in [1,3] P_th, rtol 1e-6 per 10 ps, FNO width "
                               f"{args.fno_width} modes {args.fno_modes} 4 layers",
                   "train_members": len(train_cfgs), "train_steady": int(keep.sum()),
                   "test_members": len(test_cfgs), "test_plain_steady": int(valid.sum()),
                   "epochs": args.fno_epochs, "batch": args.fno_batch,
                   "solver_precision": args.fno_precision, "reservoir_closure": True,
                   "amplitude_balance": True,
                   "by_kind": by_kind},
        "speedup_wall": ev.speedup_wall, "plain_wall_s": ev.plain_wall, "warm_wall_s": ev.warm_wall,
        "accepted": int(ev.accepted[valid].sum()),
        "plain_time_ps_mean": float(np.mean(ev.plain_time[valid])) if valid.any() else None,
        "warm_cost_ps_mean": float(np.mean(ev.cost_time[valid])) if valid.any() else None,
        "density_error_median": float(np.median(ev.density_error[valid])) if valid.any() else None,
        "plain_time_ps": [float(v) for v in ev.plain_time[valid]],
        "warm_time_ps": [float(v) for v in ev.warm_time[valid]],
        "train_loss_first_last": [losses[0], float(np.mean(losses[-10:]))],
        "data_generation_s": gen_s, "training_s": train_s,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=4000)
    ap.add_argument("--warmup", type=int, default=50)
    ap.add_argument("--members", type=int, default=32)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--e2e-calls", type=int, default=8)
    ap.add_argument("--cpu-sample-steps", type=int, default=12)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--grid", type=int, default=1024,
                    help="rk4 / split workloads: grid size n (n^2 sites, lx = ly = 400 n / 1024, the same "
                         "cell); members default to keep 32 x 1024^2 sites")
    ap.add_argument("--potential", choices=["none", "real", "complex"], default="none",
                    help="rk4 workload: add a trap (and an absorbing rim) potential")
    ap.add_argument("--eta", type=float, default=0.0,
                    help="rk4 workload: kinetic relaxation eta (the general kernel variant)")
    ap.add_argument("--rk4-kernel", choices=["auto", "wide", "tiled", "wide4"], default="auto",
                    help="rk4 workload: the full-width TMA kernel (wide), the same with four "
                         "sites a thread (wide4), the tiled kernel, or the engine's choice")
    ap.add_argument("--split-ordering", choices=["kouter", "cpu"], default="kouter",
                    help="split workload: K-outer (split-step-fft-cuda) or CPU ordering")
    ap.add_argument("--workload", choices=["rk4", "split", "sweep", "spinor", "fno", "ifrk"],
                    default="rk4",
                    help="rk4: the 1024^2 fused-step benchmark; sweep: the uneven-size sweep; "
                         "spinor: the adaptive two-component IFRK run")
    ap.add_argument("--spinor-time", type=float, default=500.0)
    ap.add_argument("--observables-out", default=None,
                    help="spinor workload: write n(k), g1, <n> and g2 to this npz file")
    ap.add_argument("--fno-n", type=int, default=256)
    ap.add_argument("--fno-train", type=int, default=2000)
    ap.add_argument("--fno-test", type=int, default=200)
    ap.add_argument("--fno-time", type=float, default=4000.0)
    ap.add_argument("--fno-dt", type=float, default=0.01)
    ap.add_argument("--fno-epochs", type=int, default=20)
    ap.add_argument("--fno-batch", type=int, default=16)
    ap.add_argument("--fno-lr", type=float, default=1e-3)
    ap.add_argument("--fno-width", type=int, default=32)
    ap.add_argument("--fno-modes", type=int, default=16)
    ap.add_argument("--fno-targets", choices=["steady", "final"], default="steady")
    ap.add_argument("--fno-precision", choices=["single", "double"], default="double",
                    help="precision of the runs that make and judge steady states")
    ap.add_argument("--fno-kinds", default="gaussian,ring,lattice")
    ap.add_argument("--steady-time", type=float, default=0.0,
                    help="sweep workload: also run to steady state (up to this many ps)")
    ap.add_argument("--freeze-stopped", action="store_true")
    ap.add_argument("--sweep-tiling", type=int, nargs=2, metavar=("LANES", "ROWS"),
                    help="sweep workload: use this tile shape instead of the autotuner's")
    args = ap.parse_args()
    if args.warmup < 3:
        raise SystemExit("--warmup must be >= 3")
    if args.grid != 1024:
        global NX, NY, LX, LY, METRIC
        NX = NY = int(args.grid)
        LX = LY = 400.0 * NX / 1024
        METRIC = f"RK4 site-updates/s at {NX}^2"
        if "--members" not in sys.argv:
            args.members = max(1, 32 * 1024 * 1024 // (NX * NY))
    if args.workload == "split":
        run_split_bench(args)
        return
    if args.workload == "spinor":
        run_spinor_bench(args)
        return
    if args.workload == "fno":
        run_fno_bench(args)
        return
    if args.workload == "ifrk":
        run_ifrk_bench(args)
        return
    if args.workload == "sweep":
        if args.members == 32 and "--members" not in sys.argv:
            args.members = 256
        run_sweep_bench(args)
        return
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
