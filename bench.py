"""Benchmark of the FP64 2D DG shallow-water stage on GB300.

Workload (one "step" = one full SSP-RK3 step: the positivity-bounded dt,
three fused stages of RHS + combination + damping + wet/dry correction):
the synthetic coastal box of ≈ 1.0 M quads at N = 3 (16 M nodes), a seeded
Gaussian random bed of 2–300 m with 30 islands, a 4-constituent tide at the
open western side, Manning n = 0.02, Coriolis at 63° N.

Metric: DOF-updates/s = 3 · K · (N+1)² · steps / s (one DOF advanced by one
full step). ``value`` is device time (CUDA events on the library's stream)
with the state resident in HBM; ``e2e`` is the same metric through the C
ABI with host buffers: every step one ``dgswe_step_host`` call on a pinned
host state (upload, dt, step, download, the copies overlapped with the
compute in element chunks).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Under torchrun (N > 1) every rank runs its own replica of the workload on
its GPU (the path has no exchange between independent runs: replicas only,
weak scaling); rank 0 prints the line. ``--impl reference`` times the
reference's CPU path — the oracle port (oracle/, a C++ restatement of the
reference CPU path; the Rust reference cannot be built here) — on the host
cores."""

from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

import numpy as np  # noqa: E402

METRIC = "FP64 DG SWE DOF-updates/s"
UNIT = "DOF-updates/s"
BYTES_PER_NODE_STAGE = {2: 81.8, 3: 77.5}  # algorithmic bytes (state, bed, mesh), N=2 / N=3
# stage_kernel<4>'s DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) per
# node-stage in one ncu capture of the 200k-quad coastal box, for scaling by nodes
STAGE_TRAFFIC_PER_NODE_STAGE = {3: 187.3}
# FP64 floating-point operations the step's kernels execute per node (an FMA
# as 2): ncu's dadd + dmul + 2·dfma instruction counts of one capture of the
# 200k-quad coastal box at N = 3 — the stage and face kernels per stage (three
# a step) and the dt kernel once a step
FP64_FLOPS_PER_NODE = {3: {"stage": 157.4, "face": 77.1, "dt": 11.4}}


def fp64_gemm_tflops(device: int, n: int = 6144, reps: int = 5) -> float | None:
    """cuBLAS FP64 GEMM throughput on this GPU (torch.mm of n × n doubles,
    CUDA events, after one warm-up): the FP64 roof the kernels are held to."""
    try:
        import torch

        a = torch.randn(n, n, dtype=torch.float64, device=f"cuda:{device}")
        b = torch.randn(n, n, dtype=torch.float64, device=f"cuda:{device}")
        torch.mm(a, b)
        torch.cuda.synchronize(device)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            torch.mm(a, b)
        e1.record()
        torch.cuda.synchronize(device)
        seconds = e0.elapsed_time(e1) * 1e-3
        del a, b
        torch.cuda.empty_cache()
        return 2.0 * n ** 3 * reps / seconds / 1e12
    except Exception:  # noqa: BLE001 - a missing roof leaves the figure without a fraction
        return None


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class Dist:
    """Barrier and max over ranks (torch.distributed), a no-op alone."""

    def __init__(self, world: int, backend: str):
        self.world = world
        self.dist = None
        if world > 1:
            import torch.distributed as dist

            dist.init_process_group(backend=backend)
            self.dist = dist

    def barrier(self):
        if self.dist:
            self.dist.barrier()

    def max(self, x: float) -> float:
        if not self.dist:
            return x
        import torch

        dev = "cuda" if self.dist.get_backend() == "nccl" else "cpu"
        t = torch.tensor([x], dtype=torch.float64, device=dev)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def sum(self, x: float) -> float:
        if not self.dist:
            return x
        import torch

        dev = "cuda" if self.dist.get_backend() == "nccl" else "cpu"
        t = torch.tensor([x], dtype=torch.float64, device=dev)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.SUM)
        return float(t.item())

    def close(self):
        if self.dist:
            self.dist.destroy_process_group()


class ClockSampler:
    """nvidia-smi clocks and throttle reasons of one GPU every 200 ms."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200", "-i", str(self.gpu)], stdout=self.file, stderr=subprocess.DEVNULL)
        except (FileNotFoundError, OSError):
            self.proc = None

    def stop(self) -> dict | None:
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.file.flush()
        rows = []
        for line in Path(self.file.name).read_text().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                rows.append((float(parts[1]), float(parts[2]), parts[5:9]))
            except ValueError:
                continue
        os.unlink(self.file.name)
        if not rows:
            return None
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for _, _, flags in rows for i, f in enumerate(flags)
                          if f.lower() == "active"})
        return {"sm_mhz": statistics.median(r[0] for r in rows), "sm_max_mhz": max(r[1] for r in rows),
                "reasons": reasons, "samples": len(rows)}


def build_workload(n_elements: int, order: int):
    from dgcom_gb300 import cases

    return cases.coastal_box(n_elements=n_elements, order=order)


def cpu_model() -> str:
    """The host CPU's model name (lscpu, else /proc/cpuinfo), or the machine."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        for line in Path("/proc/cpuinfo").read_text().splitlines():
            if line.lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except OSError:
        pass
    import platform

    return platform.machine()


def oracle_steps(case, steps: int, threads: int, warmup: int = 0, contract: bool = False,
                 state=None, t_start: float = 0.0) -> dict:
    """The oracle (C++ restatement of the reference CPU path, OpenMP) timed
    on the host cores over ``steps`` SSP-RK3 steps of ``case`` after
    ``warmup`` untimed ones; ``contract``: the FMA-contracted build."""
    sys.path.insert(0, str(ROOT / "tests"))
    from oracle_lib import oracle

    ref = oracle(case.form, threads=threads, contract=contract)
    try:
        ref.upload(*(state if state is not None else case.state))
        t = t_start
        for _ in range(warmup):
            dt = ref.compute_dt_ssp(case.cfl)
            ref.step(t, dt)
            t += dt
        t0 = time.perf_counter()
        for _ in range(steps):
            dt = ref.compute_dt_ssp(case.cfl)
            ref.step(t, dt)
            t += dt
        seconds = time.perf_counter() - t0
    finally:
        ref.close()
    nodes = case.form.n_values
    return {"value": 3.0 * nodes * steps / seconds, "seconds": seconds, "steps": steps}


def cpu_baseline_figures(case, threads: int, budget_s: float = 10.0) -> dict:
    """Both oracle builds on the whole workload from its start: the build
    that rounds every multiply and add (the reference's arithmetic, and its
    target-cpu=native tuning) as the baseline, the FMA-contracted build
    beside it; each over as many steps (1 to 10) as fit ``budget_s``."""
    probe = oracle_steps(case, 1, threads)
    steps = int(max(1, min(10, budget_s / max(probe["seconds"], 1e-3))))
    plain = oracle_steps(case, steps, threads)
    fma = oracle_steps(case, steps, threads, contract=True)
    model = cpu_model()
    return {
        "value": plain["value"], "unit": UNIT, "cores": threads, "kind": "port",
        "sample": (f"{steps} SSP-RK3 steps of the whole {case.form.mesh.n_elements}-element mesh "
                   f"from rest, {plain['seconds']:.1f} s on {threads} host threads of {model}; "
                   "oracle build -O3 -ffp-contract=off with the host CPU's tuning"),
        "cpu_model": model,
        "contraction_on": {"value": fma["value"], "unit": UNIT, "seconds": fma["seconds"],
                           "steps": steps, "build": "-O3 -ffp-contract=fast with the host "
                                                    "CPU's tuning (FMA-contracted)"},
    }


def run_reference(args, rank: int, world: int):
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    # each bench step is one oracle SSP-RK3 step of the whole workload the
    # GPU arm times (≈ 0.15 s a step on 16 host threads)
    case = build_workload(args.elements, args.order)
    full = case.form
    run = oracle_steps(case, args.steps, threads, warmup=args.warmup)
    fma = oracle_steps(case, args.steps, threads, warmup=args.warmup, contract=True)
    seconds = run["seconds"]
    nodes = full.n_values
    value = 3.0 * nodes * args.steps / seconds
    model = cpu_model()
    sample = (f"{args.steps} SSP-RK3 steps (after {args.warmup}) of the whole coastal box, "
              f"{full.mesh.n_elements} elements, N={args.order}, from rest; oracle port "
              f"(-O3 -ffp-contract=off, host CPU tuning) on {threads} host threads of {model}")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * seconds / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic",
        "config": workload_config(full, args.order, world),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": sample, "cpu_model": model,
                         "contraction_on": {"value": fma["value"], "unit": UNIT,
                                            "seconds": fma["seconds"], "steps": args.steps,
                                            "build": "-O3 -ffp-contract=fast with the host "
                                                     "CPU's tuning (FMA-contracted)"}},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def workload_config(form, order: int, world: int, weather: bool = False) -> dict:
    return {"workload": f"coastal box {form.mesh.n_elements} quads N={order} "
                        "SSP-RK3 (wet/dry, Manning, Coriolis, 4-constituent tide"
                        + (", synthetic storm: wind, pressure, raised open boundary)"
                           if weather else ")"),
            "elements": form.mesh.n_elements, "order": order,
            "nodes": form.n_values, "parallelism": f"replicas x{world}",
            "start": "from rest at t = 0 under the 1-hour tide ramp",
            "l2": "inputs larger than L2 (state and tables ≫ 129 MB)"}


def run_ours(args, rank: int, world: int, local: int):
    import ctypes as C

    from dgcom_gb300 import abi
    from dgcom_gb300.device import SWEPhysics2D

    dist = Dist(world, "nccl")
    case = build_workload(args.elements, args.order)
    form = case.form
    if args.weather:
        # a synthetic storm over the box: the wind-stress and pressure source
        # and the open boundary raised by its inverse-barometer level
        import dataclasses

        from dgcom_gb300 import cases
        from dgcom_gb300.mesh import TAG_OPEN

        weather = cases.synthetic_atmosphere(form, t0=0.0, t1=3600.0, dt_snap=3600.0)
        open_bc = dataclasses.replace(form.boundaries[TAG_OPEN], raise_factor=1.0)
        form = dataclasses.replace(form, atmosphere=weather,
                                   boundaries={**form.boundaries, TAG_OPEN: open_bc})
    nodes = form.n_values
    dev = SWEPhysics2D(form, local)
    dev.upload(*case.state)
    lib = dev.lib
    # the kernels' launch shapes, timed on this mesh and state (dgswe_autotune)
    tuning = dev.autotune(5)

    def profile(steps: int, t_start: float) -> abi.Profile:
        cfg = abi.RunConfig()
        cfg.scheme = abi.SSP_RK3
        cfg.cfl = case.cfl
        cfg.t_start = t_start
        cfg.t_end = 1e300
        out = abi.Profile()
        st = lib.profile_steps(dev.handle, C.byref(cfg), steps, C.byref(out))
        if st != abi.OK:
            raise RuntimeError(lib.error_text(dev.handle, st))
        return out

    warm = profile(args.warmup, 0.0)
    sampler = ClockSampler(local)
    dist.barrier()
    sampler.start()
    timed = profile(args.steps, warm.t_final)
    clocks = sampler.stop()
    dist.barrier()
    seconds = dist.max(timed.total_ms * 1e-3)
    total_nodes = dist.sum(float(nodes))
    value = 3.0 * total_nodes * args.steps / seconds

    # the same box flowing, after the ramp: the step time on a state whose
    # wet nodes all move (η = 0.5 cos(2πx/Lx) m, (u, v) = (0.3, −0.1) m/s)
    # from t = 2 h, so the friction, wave-speed and subcell branches of a
    # running tide are the ones taken
    flowing = None
    if not args.no_flowing:
        from dgcom_gb300 import cases

        dev.upload(*cases.with_flow(case))
        profile(args.warmup, 7200.0)
        flow = profile(args.steps, 7200.0)
        flowing = {"ms_per_step": flow.total_ms / args.steps,
                   "value": 3.0 * nodes * args.steps / (flow.total_ms * 1e-3), "unit": UNIT,
                   "kernel_ms": {"stage": flow.stage_ms / args.steps,
                                 "face": flow.face_ms / args.steps,
                                 "dt": flow.dt_ms / args.steps},
                   "state": "eta = 0.5 cos(2 pi x/Lx) m, (u, v) = (0.3, -0.1) m/s at the wet "
                            "nodes, from t = 2 h (after the ramp)"}

    # e2e: through the C ABI with pinned host buffers, every step one call of
    # dgswe_step_host: upload the state, the positivity-bounded dt, one step,
    # the new state back into the host buffers (overlapped with the last stage)
    e2e_steps = max(1, args.steps)
    try:
        import torch

        pinned = [torch.empty(nodes, dtype=torch.float64, pin_memory=True).numpy() for _ in range(3)]
    except Exception:  # noqa: BLE001 - pinned memory is an optimisation of the copy
        pinned = [np.empty(nodes) for _ in range(3)]
    dev.upload(*case.state)
    profile(args.warmup, 0.0)
    h, hu, hv = dev.download()
    for dst, src in zip(pinned, (h, hu, hv)):
        dst[:] = src
    # warm-up calls (the first builds the upload chunks' ready lists and the
    # copy stream), then the timed ones, each from the state the last left
    t = warm.t_final
    for _ in range(max(1, min(args.warmup, 3))):
        t += dev.step_host(t, case.cfl, *pinned)
    dist.barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        t += dev.step_host(t, case.cfl, *pinned)
    e2e_seconds = dist.max(time.perf_counter() - t0)
    e2e_value = 3.0 * total_nodes * e2e_steps / e2e_seconds

    peak, peak_kind = peaks()
    stage_avg_ms = timed.stage_ms / max(1, timed.stage_launches)
    bytes_per_launch = BYTES_PER_NODE_STAGE.get(args.order, 77.5) * nodes
    achieved = bytes_per_launch / (stage_avg_ms * 1e-3) / 1e9
    baseline = None
    if rank == 0 and not args.no_cpu_baseline:
        baseline = cpu_baseline_figures(case, os.cpu_count() or 1)
    dev.close()
    fp64 = None
    if args.order in FP64_FLOPS_PER_NODE:
        f = FP64_FLOPS_PER_NODE[args.order]
        per_node_step = 3.0 * (f["stage"] + f["face"]) + f["dt"]
        achieved_tf = per_node_step * nodes * args.steps / (timed.total_ms * 1e-3) / 1e12
        gemm = fp64_gemm_tflops(local)
        sm_ghz = (clocks or {}).get("sm_mhz", 2070.0) / 1e3
        fp64 = {"achieved": achieved_tf, "unit": "TFLOP/s", "flops_per_node_step": per_node_step,
                "peak_dgemm": gemm, "frac_of_dgemm": achieved_tf / gemm if gemm else None,
                "peak_pipe": 152 * 2 * 2 * sm_ghz / 1e3,
                "note": "FP64 operations the step's kernels execute (ncu instruction counts at "
                        "200k quads, an FMA as 2) over the step's device time; peak_dgemm is "
                        "cuBLAS FP64 GEMM measured in this run, peak_pipe 2 FP64 FMA per SM "
                        "per clock at the sampled SM clock"}
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * seconds / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic",
            "config": workload_config(form, args.order, world, args.weather),
            "launch": {"face_threads": tuning["face_threads"],
                       "stage_threads": tuning["stage_threads"],
                       "face_ms": tuning["face_ms"], "stage_ms": tuning["stage_ms"]},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak,
                         "traffic": (STAGE_TRAFFIC_PER_NODE_STAGE[args.order] * nodes
                                     if args.order in STAGE_TRAFFIC_PER_NODE_STAGE else None),
                         "peak_kind": peak_kind, "kernel": f"stage_kernel<{args.order + 1}>",
                         "note": "bound by the FP64 pipe (86.9 % of it in ncu), not HBM; traffic "
                                 "from an ncu capture at 200k quads scaled by nodes"},
            "fp64": fp64,
            "kernel_ms": {"stage": timed.stage_ms / args.steps, "face": timed.face_ms / args.steps,
                          "dt": timed.dt_ms / args.steps, "control": timed.control_ms / args.steps},
            # the state each way, and the step's 496-byte control record each
            # way (plus the 8-byte clip count read before it)
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": 3 * 8 * nodes + 496,
                    "d2h_bytes_per_step": 3 * 8 * nodes + 504,
                    "call": "dgswe_step_host (pinned host state, one call per step)"},
            "gpu_launches": int(timed.face_launches + timed.stage_launches + timed.dt_launches
                                + timed.control_launches),
            "clocks": clocks,
            "cpu_baseline": baseline,
            "flowing": flowing,
        }
        print(json.dumps(line), flush=True)
    dist.close()


def plain_run_seconds(form, state, steps: int, warmup: int, cfl: float, device: int,
                      t_start: float = 0.0) -> float:
    """Host wall time of one plain-method run (dgswe_run, the CaseDevice
    path) of ``steps`` SSP-RK3 steps of one member from ``t_start``, after
    ``warmup`` steps."""
    import ctypes as C

    from dgcom_gb300 import abi
    from dgcom_gb300.device import SWEPhysics2D

    dev = SWEPhysics2D(form, device)
    dev.upload(*state)
    lib = dev.lib
    report = abi.Report()
    no_callback = abi.CALLBACK()

    def run(n: int, t0: float) -> float:
        cfg = abi.RunConfig()
        cfg.scheme = abi.SSP_RK3
        cfg.cfl = cfl
        cfg.t_start = t0
        cfg.t_end = 1e300
        cfg.max_steps = n
        st = lib.run(dev.handle, C.byref(cfg), no_callback, None, C.byref(report))
        if st not in (abi.OK, abi.ERR_MAX_STEPS):
            raise RuntimeError(lib.error_text(dev.handle, st))
        return report.final_time

    t = run(warmup, t_start) if warmup else t_start
    t0 = time.perf_counter()
    run(steps, t)
    seconds = time.perf_counter() - t0
    dev.close()
    return seconds


def sequential_breakdown(per_member: list, steps: int, batched_seconds: float) -> dict:
    """The sequential arm member by member: a least-squares fit of each
    run's seconds per step to overhead + nodes / throughput, the share the
    overhead takes, and the batching bound — the sequential time over the
    time the members' work takes at the largest throughput any run reached
    (a batched run that wasted nothing would take that long)."""
    nodes = np.array([m[2] for m in per_member], dtype=np.float64)
    per_step = np.array([m[3] for m in per_member]) / steps
    a = np.stack([np.ones_like(nodes), nodes], axis=1)
    (overhead, per_node), *_ = np.linalg.lstsq(a, per_step, rcond=None)
    total = float(per_step.sum())
    best = float((3.0 * nodes / per_step).max())          # DOF-updates/s of the fastest run
    ideal = float(3.0 * nodes.sum() / best)                 # s per step of all members at it
    sizes = np.quantile(nodes, [0.0, 0.5, 1.0]).tolist()
    return {"members": len(per_member), "overhead_ms_per_run_step": 1e3 * float(overhead),
            "ns_per_node_step": 1e9 * float(per_node),
            "overhead_share": float(overhead) * len(per_member) / total,
            "fastest_run_dof_per_s": best,
            "sequential_ms_per_step": 1e3 * total,
            "batched_ms_per_step": 1e3 * batched_seconds / steps,
            "ideal_ms_per_step": 1e3 * ideal,
            "bound_speedup": total / ideal,
            "member_nodes_min_median_max": sizes,
            "runs": [{"elements": m[0], "order": m[1], "ms_per_step": 1e3 * m[3] / steps}
                     for m in per_member]}


def member_share(members: list, rank: int, world: int) -> list:
    """The ensemble members rank ``rank`` of ``world`` advances: every
    world-th member from its rank, so each member runs on exactly one rank
    and the ranks' element counts stay close (members are independent: no
    exchange between ranks)."""
    if not 0 <= rank < world:
        raise ValueError(f"rank {rank} of {world}")
    return members[rank::world]


def run_ensemble(args, rank: int, world: int, local: int):
    """The batched ensemble against the same members run one after another
    with the plain method, on the same GPU: members are independent, so
    ranks split them (weak scaling, no collective on the data path)."""
    from dgcom_gb300 import cases
    from dgcom_gb300.ensemble import Ensemble

    dist = Dist(world, "nccl")
    t_gen = time.perf_counter()
    members = cases.ensemble_members(args.members, k_range=(args.k_min, args.k_max))
    mine = member_share(members, rank, world)
    t_gen = time.perf_counter() - t_gen
    nodes = sum(c.form.n_values for c in mine)
    cfl = mine[0].cfl
    # from rest at t = 0 (in the tide's ramp), or flowing after the ramp:
    # η = 0.5 cos(2πx/Lx) m and (u, v) = (0.3, −0.1) m/s at the wet nodes
    starts = [cases.with_flow(c) if args.ens_flowing else c.state for c in mine]
    t_first = 7200.0 if args.ens_flowing else 0.0
    t_setup = time.perf_counter()
    ens = Ensemble([c.form for c in mine], local)
    for i, q in enumerate(starts):
        ens.upload(i, *q)
    t_setup = time.perf_counter() - t_setup
    if args.warmup:
        ens.run(args.warmup, cfl, t_start=t_first)
    sampler = ClockSampler(local)
    dist.barrier()
    sampler.start()
    t0 = time.perf_counter()
    reports, prof = ens.run(args.steps, cfl, t_start=t_first if not args.warmup else float("nan"))
    wall = time.perf_counter() - t0
    clocks = sampler.stop()
    dist.barrier()
    seconds = dist.max(wall)
    total_nodes = dist.sum(float(nodes))
    value = 3.0 * total_nodes * args.steps / seconds
    ens.close()
    # the same members, one plain-method run after another, each timed: its
    # seconds per step against its nodes give the per-run overhead and the
    # throughput a member reaches alone
    seq = 0.0
    per_member = []
    for c, q in zip(mine, starts):
        sec = plain_run_seconds(c.form, q, args.steps, args.warmup, cfl, local, t_first)
        seq += sec
        per_member.append((c.form.mesh.n_elements, c.form.order, c.form.n_values, sec))
    seq_seconds = dist.max(seq)
    seq_value = 3.0 * total_nodes * args.steps / seq_seconds
    orders = sorted({c.form.order for c in members})
    elements = sum(c.form.mesh.n_elements for c in members)
    if rank == 0:
        line = {
            "metric": METRIC + " (batched ensemble)", "value": value, "unit": UNIT,
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * seconds / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": f"ensemble of {len(members)} coastal-box members, "
                                   f"{args.k_min}-{args.k_max} quads log-uniform, N in {orders}, "
                                   "Manning n and M2 amplitude per member, SSP-RK3 "
                                   + ("flowing after the ramp" if args.ens_flowing else "from rest"),
                       "members": len(members), "elements": elements,
                       "nodes": int(total_nodes), "parallelism": f"members split over {world}",
                       "l2": "inputs larger than L2"},
            "sequential": {"value": seq_value, "unit": UNIT, "seconds": seq_seconds,
                           "what": "the same members, one dgswe_run each, back to back"},
            "speedup_vs_sequential": value / seq_value,
            "device_ms_per_step": prof.total_ms / args.steps,
            "gpu_launches": int(prof.face_launches + prof.stage_launches + prof.dt_launches
                                + prof.control_launches),
            "setup_s": {"generate": t_gen, "create_and_upload": t_setup},
            "sequential_breakdown": sequential_breakdown(per_member, args.steps, seconds),
            "start": ("flowing after the ramp, from t = 2 h" if args.ens_flowing
                      else "from rest at t = 0 in the tide's ramp"),
            "clocks": clocks,
            "members_failed": sum(0 if r.success else 1 for r in reports),
        }
        print(json.dumps(line), flush=True)
    dist.close()


def run_adjoint(args, rank: int, world: int, local: int):
    """The discrete adjoint on the refined tidal channel: the gradient of a
    50-station misfit (observations from a forward run with a perturbed
    friction field) w.r.t. Manning's n per element, the bed, and the M2
    amplitude and phase; its time against the forward's with checkpoints
    every 45 steps (the replay keeping each step's full reverse data, or
    only the step-start states) and with every state stored; central differences on random directions, by replaying the
    forward's steps. One GPU: replicas are independent runs."""
    import dataclasses

    from dgcom_gb300 import cases
    from dgcom_gb300.adjoint import Adjoint
    from dgcom_gb300.physics import TidalBoundary

    dist = Dist(world, "nccl")
    case, stations, n_obs = cases.adjoint_channel(nx=args.adj_nx, ny=args.adj_ny, order=args.order)
    form = case.form
    nn = (args.order + 1) ** 2
    steps = args.steps
    state = case.state
    nodes = form.n_values
    obs_form = dataclasses.replace(form, manning_n=np.repeat(n_obs, nn))
    t0 = args.adj_t_start
    with Adjoint(obs_form, steps, stations, cfl=case.cfl, t_start=t0) as a:
        _, eta_obs, _ = a.forward(state)
    state_bytes = 3.0 * 8.0 * nodes
    results = {}
    g = None
    dts = None
    # checkpoints every 45 steps: with the segment's full reverse data (10
    # states a step), or with its step-start states only; every state stored
    every = 45
    full_budget = (math.ceil(steps / every) + 10 * every + 1) * state_bytes
    start_budget = (math.ceil(steps / every) + every + 1) * state_bytes
    for label, budget, ck in [("every 45, full segments", full_budget, every),
                              ("every 45, step-start segments", start_budget, every),
                              ("all stored", 0.0, 0)]:
        with Adjoint(form, steps, stations, cfl=case.cfl, t_start=t0, memory_budget=budget,
                     device=local, checkpoint_every=ck) as a:
            a.forward(state, eta_obs=eta_obs)  # warm-up
            J, _, dts = a.forward(state, eta_obs=eta_obs)
            g = a.reverse()
            st = a.stats()
        results[label] = {"J": J, "forward_ms": st.forward_ms, "reverse_ms": st.reverse_ms,
                          "reverse_over_forward": st.reverse_ms / st.forward_ms,
                          "gradient_over_forward": (st.forward_ms + st.reverse_ms) / st.forward_ms,
                          "stride": int(st.stride), "full_segments": bool(st.full_segments),
                          "stored_gb": st.stored_bytes / 1e9,
                          "recomputed_steps": int(st.recomputed_steps)}
    # central differences of the forward (the steps replayed) on random directions
    rng = np.random.default_rng(7)
    n0 = np.asarray(form.manning_n)
    b0 = form.bathymetry.reshape(-1)
    x, y = form.positions()
    x = x.reshape(-1)
    y = y.reshape(-1)
    OPEN = 1
    c0 = form.boundaries[OPEN].constituents[0]

    def J_of(f):
        with Adjoint(f, steps, stations, cfl=case.cfl, t_start=t0, device=local) as a:
            return a.forward(state, dts=dts, eta_obs=eta_obs)[0]

    with Adjoint(form, steps, stations, cfl=case.cfl, t_start=t0, device=local) as a:
        st_elem, st_w = a.station_weights()

    def J_oracle(f):
        """J of the oracle's forward (the CPU restatement of the reference
        forward) over the same time steps, on the host cores."""
        sys.path.insert(0, str(ROOT / "tests"))
        from oracle_lib import oracle

        ref = oracle(f, threads=os.cpu_count() or 1)
        try:
            ref.upload(*state)
            b = f.bathymetry.reshape(-1)
            t, J = t0, 0.0
            for n, dt in enumerate(dts):
                ref.step(t, dt)
                t += dt
                h = ref.download()[0]
                for s_, (k, w) in enumerate(zip(st_elem, st_w)):
                    sl = slice(k * nn, (k + 1) * nn)
                    J += (float(np.dot(w, h[sl] + b[sl])) - float(eta_obs[n, s_])) ** 2
        finally:
            ref.close()
        return J

    def with_tide(amplitude, phase):
        cons = list(form.boundaries[OPEN].constituents)
        c = type(cons[0])()
        for name, _ in type(c)._fields_:
            setattr(c, name, getattr(cons[0], name))
        c.amplitude = amplitude
        c.phase = phase
        cons[0] = c
        bc = form.boundaries[OPEN]
        new = dict(form.boundaries)
        new[OPEN] = TidalBoundary(cons, mean_elevation=bc.mean_elevation,
                                  ramp_duration=bc.ramp_duration, incoming_wave=bc.incoming_wave)
        return dataclasses.replace(form, boundaries=new)

    checks = []
    oracle_base = {}
    for i in range(args.fd_directions):
        kind = ("manning", "bed", "tide")[i % 3]
        if kind == "manning":
            d_el = rng.standard_normal(form.mesh.n_elements)
            d = np.repeat(d_el, nn)
            adj = float(np.dot(g.manning_per_element(nn), d_el))
            eps = 1e-4 * 0.02  # at 1e-6 the difference is within J's rounding
            make = lambda e, d=d: dataclasses.replace(form, manning_n=n0 + e * d)
        elif kind == "bed":
            kx, ky = rng.uniform(1.0, 8.0), rng.uniform(0.5, 3.0)
            ph = rng.uniform(0.0, 2 * np.pi)
            d = np.sin(kx * 2 * np.pi * x / 50_000.0 + ph) * np.cos(ky * np.pi * y / 5_000.0)
            adj = float(np.dot(g.bed, d))
            eps = 1e-6 * float(np.abs(b0).max())
            make = lambda e, d=d: dataclasses.replace(
                form, bathymetry=(b0 + e * d).reshape(form.bathymetry.shape))
        else:  # a direction in the (amplitude, phase) plane
            th = rng.uniform(0.0, 2 * np.pi)
            da, dp = np.cos(th) * c0.amplitude, np.sin(th)
            adj = float(g.tide[OPEN, 0, 0] * da + g.tide[OPEN, 0, 1] * dp)
            eps = 1e-6
            make = lambda e, da=da, dp=dp: with_tide(c0.amplitude + e * da, c0.phase + e * dp)
        fd = (J_of(make(eps)) - J_of(make(-eps))) / (2.0 * eps)
        check = {"kind": kind, "adjoint": adj, "fd": fd,
                 "rel": abs(adj - fd) / max(abs(fd), abs(adj), 1e-300)}
        if args.fd_oracle_above is not None and check["rel"] > args.fd_oracle_above:
            # the oracle's forward at p ± εd, p ± εd/2 and p: its central and
            # one-sided differences (a kink crossed shows as one-sided
            # differences that disagree), and the Richardson extrapolation
            # (4·D(ε/2) − D(ε))/3, which removes the central difference's
            # ε² term where J is smooth but strongly curved
            if "j0" not in oracle_base:
                oracle_base["j0"] = J_oracle(form)
            jm, j0, jp = J_oracle(make(-eps)), oracle_base["j0"], J_oracle(make(eps))
            ofd = (jp - jm) / (2.0 * eps)
            ofd2 = (J_oracle(make(0.5 * eps)) - J_oracle(make(-0.5 * eps))) / eps
            rich = (4.0 * ofd2 - ofd) / 3.0

            def rel_to(v):
                return abs(adj - v) / max(abs(v), abs(adj), 1e-300)

            check["oracle"] = {"fd": ofd, "rel": rel_to(ofd), "fd_half_step": ofd2,
                               "rel_half_step": rel_to(ofd2), "richardson": rich,
                               "rel_richardson": rel_to(rich),
                               "forward_diff": (jp - j0) / eps, "backward_diff": (j0 - jm) / eps}
        checks.append(check)
    rels = [c["rel"] for c in checks]
    headline = results["every 45, full segments"]
    if rank == 0:
        line = {
            "metric": "adjoint time / forward time (discrete adjoint of the FP64 DG SWE run)",
            "value": headline["reverse_over_forward"], "unit": "ratio", "n_gpus": world,
            "steps": steps, "warmup": 1, "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": f"tidal channel {form.mesh.n_elements} quads N={args.order} "
                                   f"(drying flat), {steps} SSP-RK3 steps from rest at t = {t0:g} s "
                                   f"(past the 1 h tide ramp), {len(stations)} stations; "
                                   "gradient w.r.t. Manning n per element, bed per node, M2 "
                                   "amplitude and phase",
                       "elements": form.mesh.n_elements, "order": args.order, "nodes": nodes,
                       "parallelism": f"replicas x{world}"},
            "runs": results,
            "fd_check": {"directions": len(checks), "what": "central differences of the GPU "
                         "forward with the adjoint's time steps replayed: Manning n per element "
                         "(step 1e-4 relative: at 1e-6 the difference is within J's rounding), "
                         "smooth bed fields and (amplitude, phase) directions (step 1e-6)",
                         "max_rel": max(rels) if rels else None,
                         "median_rel": float(np.median(rels)) if rels else None,
                         "checks": checks},
        }
        print(json.dumps(line), flush=True)
    dist.close()


def run_adjoint_ensemble(args, rank: int, world: int, local: int):
    """The batched adjoint ensemble: ``--adj-members`` coastal boxes of
    ``--adj-k-min``..``--adj-k-max`` quads (log-uniform), each with 30
    stations, eight tide constituents and Manning's n per element, in one
    batched forward and reverse sweep within a shared checkpoint budget of
    ``--adj-budget-gb``. The observations come from a forward run under
    perturbed forcing (the same step times); the gradient is w.r.t. every
    member's Manning n per element and constituent amplitudes and phases.
    Central differences of the batched forward (steps replayed, the
    parameters moved in place) check random directions. One GPU: replicas
    are independent runs."""
    from dgcom_gb300 import cases
    from dgcom_gb300.adjoint import Adjoint
    from dgcom_gb300.mesh import TAG_OPEN

    dist = Dist(world, "nccl")
    t_gen = time.perf_counter()
    ms = cases.adjoint_ensemble_members(n_members=args.adj_members, seed=2029 + rank,
                                        k_range=(args.adj_k_min, args.adj_k_max),
                                        order=args.order, n_stations=30)
    t_gen = time.perf_counter() - t_gen
    forms = [m.case.form for m in ms]
    stations = np.vstack([m.stations for m in ms])
    member = np.repeat(np.arange(len(ms)), [m.stations.shape[0] for m in ms]).astype(np.int32)
    # a flowing state (η = 0.5 m·cos(2πx/L), u = 0.4, v = −0.15 m/s where wet):
    # from rest, the first steps' currents are too weak for friction to matter
    flows = [cases.with_flow(m.case, eta_amp=0.5, u=0.4, v=-0.15) for m in ms]
    state = tuple(np.concatenate([f[c] for f in flows]) for c in range(3))
    nn = (args.order + 1) ** 2
    quads = int(sum(f.mesh.n_elements for f in forms))
    nodes = quads * nn
    steps = args.steps
    t0 = args.adj_ens_t_start
    budget = args.adj_budget_gb * 1e9
    t_create = time.perf_counter()
    ens = Adjoint.ensemble(forms, steps, stations, member, cfl=0.5, t_start=t0,
                           memory_budget=budget, device=local)
    t_create = time.perf_counter() - t_create
    try:
        tide0 = ens.tide_parameters()
        n0 = np.concatenate([np.asarray(f.manning_n) for f in forms])
        tide_obs = tide0.copy()
        row = 0
        for m, f in zip(ms, forms):
            tide_obs[row + sorted(f.boundaries).index(TAG_OPEN)] = m.tide_obs
            row += len(f.boundaries)
        n_obs = np.concatenate([m.manning_obs for m in ms])
        # the CFL steps (also the warm-up), then the observations at the same times
        _, _, dts = ens.forward(state)
        ens.set_parameters(manning=n_obs, tide=tide_obs)
        _, eta_obs, _ = ens.forward(state, dts=dts)
        ens.set_parameters(manning=n0, tide=tide0)
        J, _, _ = ens.forward(state, dts=dts, eta_obs=eta_obs)
        Jm = ens.member_J()
        # the gradients asked of the batched adjoint: Manning and the tides, no bed
        g = ens.reverse(bed=False)
        st = ens.stats()

        def J_at(manning=None, tide=None):
            ens.set_parameters(manning=manning, tide=tide)
            return ens.forward(state, dts=dts, eta_obs=eta_obs)[0]

        # each direction at two or three steps: the difference's rounding
        # noise falls and its truncation error grows with the step, so their
        # agreement shows which dominates; the closest one is reported
        rng = np.random.default_rng(17)
        checks = []
        for i in range(args.fd_directions):
            m = int(rng.integers(len(forms)))
            if i % 2 == 0:  # Manning n per element of one member
                sl = ens.member_slice(m)
                d = np.zeros_like(n0)
                d[sl] = np.repeat(rng.standard_normal((sl.stop - sl.start) // nn), nn)
                adj = float(np.dot(g.manning, d))
                # J is piecewise smooth in n at the scale of 1e-4 of it (wet/dry
                # and limiter switches move with n), so the steps are smaller
                steps_rel = (1e-4, 1e-5, 3e-6)
                scale = float(n0[sl].max())
                J_dir = lambda e, d=d: J_at(manning=n0 + e * d)
                kind = "manning"
            else:  # the eight constituents' amplitudes and phases of one member
                r = sum(len(f.boundaries) for f in forms[:m]) + \
                    sorted(forms[m].boundaries).index(TAG_OPEN)
                d = np.zeros_like(tide0)
                d[r] = rng.standard_normal(d[r].shape)
                adj = float(np.sum(g.tide * d))
                steps_rel = (1e-4, 1e-5)
                scale = 1.0
                J_dir = lambda e, d=d: J_at(tide=tide0 + e * d)
                kind = "tide"
            fds = []
            for sr in steps_rel:
                eps = sr * scale
                fds.append((J_dir(eps) - J_dir(-eps)) / (2 * eps))
            ens.set_parameters(manning=n0, tide=tide0)
            rel = [abs(adj - fd) / max(abs(fd), abs(adj), 1e-300) for fd in fds]
            best = int(np.argmin(rel))
            checks.append({"kind": kind, "member": m, "adjoint": adj, "fd": fds[best],
                           "step": steps_rel[best], "rel": rel[best],
                           "fd_both_steps": fds, "steps": list(steps_rel)})
    finally:
        ens.close()
    rels = [c["rel"] for c in checks]
    if rank == 0:
        fwd_s = st.forward_ms / 1e3
        line = {
            "metric": "batched adjoint ensemble: adjoint time / forward time",
            "value": st.reverse_ms / st.forward_ms, "unit": "ratio", "n_gpus": world,
            "steps": steps, "warmup": 1, "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": f"{len(forms)} coastal boxes of {args.adj_k_min}-"
                                   f"{args.adj_k_max} quads (log-uniform, {quads} in all), "
                                   f"N={args.order}, {steps} SSP-RK3 steps from a flowing state "
                                   f"at t = {t0:g} s, 30 stations each, 8 constituents; gradient "
                                   "w.r.t. Manning n per element and every constituent's "
                                   "amplitude and phase, one batched sweep",
                       "members": len(forms), "elements": quads, "order": args.order,
                       "nodes": nodes, "checkpoint_budget_gb": args.adj_budget_gb,
                       "parallelism": f"replicas x{world}"},
            "forward_ms": st.forward_ms, "reverse_ms": st.reverse_ms,
            "gradient_over_forward": (st.forward_ms + st.reverse_ms) / st.forward_ms,
            "forward_dof_updates_per_s": 3.0 * nodes * steps / fwd_s,
            "gradient_wall_s": st.forward_wall_s + st.reverse_wall_s,
            "stride": int(st.stride), "stored_gb": st.stored_bytes / 1e9,
            "recomputed_steps": int(st.recomputed_steps),
            "J": J, "J_member_min": float(Jm.min()), "J_member_max": float(Jm.max()),
            "dt_range_s": [float(dts.min()), float(dts.max())],
            "setup_s": {"generate": t_gen, "create": t_create},
            "fd_check": {"directions": len(checks), "what": "central differences of the batched "
                         "GPU forward with the adjoint's time steps replayed and the parameters "
                         "moved in place: Manning n per element of one member (steps 1e-4, "
                         "1e-5 and 3e-6 relative), all eight constituents' (amplitude, phase) "
                         "of one member (steps 1e-4 and 1e-5); each check reports the closest "
                         "step",
                         "max_rel": max(rels) if rels else None,
                         "median_rel": float(np.median(rels)) if rels else None,
                         "checks": checks},
        }
        print(json.dumps(line), flush=True)
    dist.close()


def run_multirate(args, rank: int, world: int, local: int):
    """Local time stepping on the coastal box: the same model span with
    global SSP-RK3 steps and with multirate coarse steps of up to
    ``--levels`` levels (dgswe_run with DeviceRun::levels), each timed on
    the host around the run (the multirate run's level planning, on the
    host, included), after a warm-up of both. The span starts from a
    flowing state after the tide's ramp. One GPU: replicas are independent."""
    from dgcom_gb300 import cases
    from dgcom_gb300.device import DeviceRun, SWEPhysics2D

    dist = Dist(world, "nccl")
    case = cases.coastal_box(args.elements, args.order)
    form = case.form
    nodes = form.n_values
    state = cases.with_flow(case, eta_amp=0.5, u=0.4, v=-0.15)
    t0 = 3600.0
    span = args.lts_span
    dev = SWEPhysics2D(form, local)

    def run(levels, t_len):
        dev.upload(*state)
        rep = dev.run_with_callback(DeviceRun(span=(t0, t0 + t_len), cfl=case.cfl, levels=levels))
        if not rep.success:
            raise RuntimeError(rep.message)
        return rep

    run(0, 2.0)
    run(args.levels, 2.0)
    sampler = ClockSampler(local)
    dist.barrier()
    sampler.start()
    g = run(0, span)
    g_state = dev.download()
    m = run(args.levels, span)
    m_state = dev.download()
    clocks = sampler.stop()
    dist.barrier()
    dev.close()
    s = m.local_time_stepping
    b = form.bathymetry.reshape(-1)
    wet = (m_state[0] > 0.0) & (g_state[0] > 0.0)
    d_eta = np.abs((m_state[0] + b) - (g_state[0] + b))[wet]
    eta_diff = {"max": float(d_eta.max()), "p99": float(np.percentile(d_eta, 99.0)),
                "median": float(np.median(d_eta)),
                "change_median": float(np.median(np.abs(g_state[0] - state[0])[wet]))}
    g_rate = 3.0 * nodes * g.n_steps / g.wall_time
    if rank == 0:
        line = {
            "metric": "local time stepping: model time per wall second against global steps",
            "value": g.wall_time / m.wall_time, "unit": "speedup", "n_gpus": world,
            "steps": int(s.steps), "warmup": 1, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": f"coastal box {form.mesh.n_elements} quads N={args.order}, "
                                   f"{span:g} s of model time from a flowing state at "
                                   f"t = {t0:g} s, SSP-RK3, up to {args.levels} levels",
                       "elements": form.mesh.n_elements, "order": args.order, "nodes": nodes,
                       "levels": args.levels, "parallelism": f"replicas x{world}"},
            "global": {"steps": g.n_steps, "wall_s": g.wall_time, "dof_updates_per_s": g_rate,
                       "dt_min": g.dt_min, "dt_max": g.dt_max},
            "multirate": {"coarse_steps": int(s.steps), "wall_s": m.wall_time,
                          "finest_level": int(s.finest_level),
                          "element_evaluations": int(s.element_evaluations),
                          "global_evaluations_at_finest": int(s.global_evaluations),
                          "level_evaluations": s.level_evaluations,
                          "ideal_evaluations": s.ideal_evaluations,
                          "line_local_elements_per_step": s.line_local_elements / max(1, s.steps),
                          "plans": int(s.plans), "plan_s": s.plan_seconds,
                          "device_pass_s": s.device_seconds,
                          "coarse_dt_range": [m.dt_min, m.dt_max]},
            "evaluations_global_over_multirate":
                (3.0 * form.mesh.n_elements * g.n_steps) / max(1, s.element_evaluations),
            "eta_difference_m": eta_diff,
            "clocks": clocks,
        }
        print(json.dumps(line), flush=True)
    dist.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--elements", type=int, default=1_000_000)
    ap.add_argument("--order", type=int, default=3)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-flowing", action="store_true",
                    help="skip the step time on the flowing state of the same box")
    ap.add_argument("--weather", action="store_true",
                    help="coastal: add a synthetic storm (GriddedAtmosphere2D's device form)")
    ap.add_argument("--workload", default="coastal",
                    choices=["coastal", "ensemble", "adjoint", "adjoint_ensemble", "multirate"],
                    help="coastal: the 1 M-quad coastal box (the headline); ensemble: batched "
                         "members against sequential plain runs; adjoint: the discrete "
                         "adjoint's time against the forward's on the refined channel; "
                         "adjoint_ensemble: the batched adjoint of coastal-box members; "
                         "multirate: local time stepping against global steps")
    ap.add_argument("--members", type=int, default=256)
    ap.add_argument("--k-min", type=int, default=5_000)
    ap.add_argument("--k-max", type=int, default=200_000)
    ap.add_argument("--ens-flowing", action="store_true",
                    help="start the ensemble's members flowing, after the ramp")
    ap.add_argument("--adj-nx", type=int, default=1000)
    ap.add_argument("--adj-ny", type=int, default=100)
    ap.add_argument("--fd-directions", type=int, default=20)
    ap.add_argument("--fd-oracle-above", type=float, default=None,
                    help="repeat the differences of the directions above this bar with the "
                         "oracle's forward, with one-sided differences")
    ap.add_argument("--adj-t-start", type=float, default=4000.0)
    ap.add_argument("--adj-members", type=int, default=64)
    ap.add_argument("--adj-k-min", type=int, default=10_000)
    ap.add_argument("--adj-k-max", type=int, default=150_000)
    ap.add_argument("--adj-budget-gb", type=float, default=120.0)
    ap.add_argument("--adj-ens-t-start", type=float, default=3600.0)
    ap.add_argument("--levels", type=int, default=4)
    ap.add_argument("--lts-span", type=float, default=60.0)
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    rank, world, local = dist_env()
    if args.impl == "reference":
        run_reference(args, rank, world)
    elif args.workload == "ensemble":
        run_ensemble(args, rank, world, local)
    elif args.workload == "adjoint":
        run_adjoint(args, rank, world, local)
    elif args.workload == "adjoint_ensemble":
        run_adjoint_ensemble(args, rank, world, local)
    elif args.workload == "multirate":
        run_multirate(args, rank, world, local)
    else:
        run_ours(args, rank, world, local)


if __name__ == "__main__":
    main()
