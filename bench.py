"""Benchmark: 3D Cahn-Hilliard at 256^3, FP32 device state, semi-implicit Euler.

Workload (the configuration the headline metric is quoted on): periodic
256x256x256 grid, dx = 1, c0 = U(-0.1, 0.1) i.i.d. from seed 1 (SplitMix64,
synthetic), M = 1, gamma = 0.5, dt = 0.05, the plain splitting of
examples/cahnHilliard/main.go:33:
    dconc/dt = M*LAP conc^3 + m1*LAP conc + m1*gamma*LAP^2 conc,  m1 = -M.

One step = one Euler step of the whole grid (pf/euler.go:16-47).
  value : steps/s with the field resident in HBM (CUDA events on the stepping stream)
  e2e   : steps/s through the C ABI with host buffers: every step uploads the
          []complex128 field from pinned memory, steps once and downloads it
  roofline : dominant kernel's algorithmic bytes / its average duration
  cpu_baseline : the FP64 CPU oracle (a restatement of the reference's Euler
                 step, OpenMP over all host cores) on a bounded sample
  config.monitors : the mass and free-energy monitors on the stepped field
                    (time per synchronous call, algorithmic bytes, GB/s)

--impl reference times the CPU oracle alone (the reference itself is Go +
FFTW and cannot be built on these machines).
Multi-GPU: the path does not shard (one grid per step); N > 1 runs N
independent replicas, one per rank, and reports the aggregate.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

METRIC = ("CH steps/s at 256³ FP32 vs GPU FP64 (rel-L2≤1e-4); FFT % of HBM peak; sweep steps/s")
UNIT = "steps/s"
# DRAM traffic (dram__bytes_read.sum + dram__bytes_write.sum) of one launch of each step kernel, from
# one ncu capture on a GB300 of `python bench.py --steps 20 --warmup 17 --no-cpu-baseline --no-e2e
# --no-precision --no-monitors` (the kernels' summaries under profiles/).  Bytes that a launch leaves in L2 are not
# in these counts.
NCU_TRAFFIC = {"zpass_update": 211.8e6, "xpass_pointwise": 72.6e6, "ypass_forward": 72.6e6,
               "ypass_inverse": 72.6e6}
DIMS = [256, 256, 256]
GAMMA, M, DT, SEED = 0.5, 1.0, 0.05, 1
CH_EQ = "dconc/dt = M*LAP conc^3 + m1*LAP conc + m1*gamma*LAP^2 conc"
FALLBACK_HBM_GBS = 6800.0
WORKLOAD = "cahn_hilliard_3d_256cube_fp32_euler"


def peaks():
    p = os.path.join(HERE, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        try:
            d = json.load(open(p))
            return float(d["hbm_gbs"]), "measured"
        except Exception:
            pass
    return FALLBACK_HBM_GBS, "fallback"


def config(extra=None):
    c = {
        "workload": WORKLOAD,
        "grid": "x".join(str(d) for d in DIMS),
        "gamma": GAMMA,
        "M": M,
        "dt": DT,
        "splitting": "examples/cahnHilliard plain (c^3 explicit, k^2 and gamma k^4 implicit)",
        "init": "c0 = U(-0.1, 0.1), seed 1 (SplitMix64)",
        "l2": "inputs larger than L2: state 67.6 MB + work 67.6 MB = 135 MB > 129 MB",
    }
    if extra:
        c.update(extra)
    return c


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = None

    def __enter__(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-lms", "200", "-i", str(self.device)], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
            time.sleep(0.3)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.f.close()

    def summary(self):
        if not self.path or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            p = [x.strip() for x in line.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                smax.append(float(p[2]))
            except ValueError:
                continue
            for n, v in zip(names, p[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        os.unlink(self.path)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def cpu_oracle_step_rate(dims, max_seconds: float, max_steps: int, warmup: int = 0, keep_field: bool = False):
    """Steps/s of the FP64 CPU oracle's Euler step (all host threads); with keep_field, also the
    oracle's real field after the steps it took (warm-up included)."""
    from gopf_gb300.synthetic import uniform_field
    from oracle import oracle as O

    n = int(np.prod(dims))
    O.build()
    threads = O.num_threads()
    m = O.cahn_hilliard(dims, gamma=GAMMA, M=M)
    m.set_field(0, uniform_field(SEED, n, 0.0, 0.1))
    for _ in range(warmup):
        m.step_euler(DT, 1)
    t0 = time.perf_counter()
    steps = 0
    while steps < max_steps:
        m.step_euler(DT, 1)
        steps += 1
        if time.perf_counter() - t0 > max_seconds:
            break
    el = time.perf_counter() - t0
    if keep_field:
        return steps / el, steps, el, threads, m.field(0).real.copy()
    return steps / el, steps, el, threads


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def run_reference(args):
    world, rank, local = dist_setup()
    if rank != 0:
        return 0
    budget = float(os.environ.get("GOPF_REF_SECONDS", "120"))
    # the requested warm-up steps, untimed (a fraction of a second each on the host cores), capped
    # so that a large request cannot stretch the run
    warm = min(args.warmup, 10)
    rate, steps, el, threads = cpu_oracle_step_rate(DIMS, max_seconds=budget, max_steps=args.steps,
                                                    warmup=warm)
    sample = (f"{steps} Euler steps of the 256^3 grid in FP64 (complex128 fields, Z2Z FFTs, as the reference), "
              f"{el:.1f} s; steps capped by a {budget:.0f} s budget")
    out = {
        "metric": METRIC, "value": rate, "unit": UNIT, "impl": "reference", "n_gpus": args.gpus,
        "steps": steps, "warmup": warm, "ms_per_step": 1000.0 / rate, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": config({"backend": "CPU oracle (C restatement of pf/euler.go; Go reference unbuildable here)"}),
        "cpu_baseline": {"value": rate, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": rate, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out))
    return 0


def run_gpu(args):
    import torch

    global DIMS, WORKLOAD
    if args.grid != 256:
        DIMS = [args.grid] * 3
        WORKLOAD = f"cahn_hilliard_3d_{args.grid}cube_fp32_euler"

    import gopf_gb300 as G
    from gopf_gb300.synthetic import uniform_field

    world, rank, local = dist_setup()
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    n = int(np.prod(DIMS))
    c0 = uniform_field(SEED, n, 0.0, 0.1)

    stream = torch.cuda.Stream()
    m = ch3d_model(G, "fp32", c0, local, stream)
    if args.tma is not None:
        m.set_option(G._lib.OPT_TMA, args.tma)
    if args.x_rows is not None:
        m.set_option(G._lib.OPT_X_ROWS, args.x_rows)
    if args.z_lines is not None:
        m.set_option(G._lib.OPT_Z_LINES, args.z_lines)
    if args.pdl is not None:
        m.set_option(G._lib.OPT_PDL, args.pdl)
    mass0 = m.mass(0)
    m.prepare_graphs(args.steps)  # capture the graphs the timed steps replay (no stepping)
    m.step(warmup_steps(args))
    torch.cuda.synchronize()

    # ---- device-resident timed region ----
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        e0.record(stream)
        m.step(args.steps)
        e1.record(stream)
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
    ms = e0.elapsed_time(e1)
    if dist:
        t = torch.tensor([ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    clocks = clk.summary()
    per_step_ms = ms / args.steps
    value = world * args.steps / (ms / 1000.0)
    mass1 = m.mass(0)
    finite = m.reduce(0, G.RED_NONFINITE) == 0
    monitors = None if args.no_monitors else time_monitors(m, n)

    # ---- per-kernel roofline (launch by launch, events on the same stream) ----
    prof = m.profile_step(20)
    dom = max(prof, key=lambda p: p["ms"])
    hbm, peak_kind = peaks()
    achieved = dom["bytes"] / (dom["ms"] * 1e-3) / 1e9
    step_bytes = sum(p["bytes"] for p in prof)

    # ---- end to end through the C ABI with pinned host buffers ----
    e2e = None
    if not args.no_e2e:
        e2e = run_e2e(args, m, stream, c0, n, world, dist, torch, G)
    gpu_launches = m.kernel_launches(args.steps)
    m.close()
    # ---- CPU baseline (the FP64 oracle on the host cores) and the metric's precision half ----
    cpu, oracle_run = None, None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        rate, steps, el, threads, ofield = cpu_oracle_step_rate(DIMS, max_seconds=args.cpu_seconds, max_steps=50,
                                                                keep_field=True)
        cpu = {"value": rate, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"{steps} FP64 Euler steps of the 256^3 grid ({el:.1f} s) on the host cores"}
        oracle_run = (steps, ofield)
    precision = None
    if rank == 0 and not args.no_precision:
        precision = measure_precision(args, G, torch, c0, n, stream, value / world, oracle_run)
    out = emit(args, world, rank, value, per_step_ms, mass0, mass1, finite, prof, dom, hbm, peak_kind, achieved,
               step_bytes, e2e, clocks, n, cpu, precision, gpu_launches, monitors)
    if dist:
        dist.barrier()
        dist.destroy_process_group()
    return 0


def time_monitors(m, n, reps=20):
    """The device monitors on the stepped field, each call synchronous (the result is on the host when
    it returns): median wall time per call over `reps` calls, and the algorithmic bytes over that time.
    Mass (gopf_reduce): the inverse x pass of T with FP64 block sums, C bytes.  Free energy
    (gopf_free_energy): the inverse x pass to real rows, the bulk sum over the cells and the gradient
    sum over the spectrum, 2C + 2R bytes (C = the half spectrum, R = the real field, FP32)."""
    C = (DIMS[0] // 2 + 1) * DIMS[1] * DIMS[2] * 8
    R = n * 4
    out = {}
    for name, call, nbytes in (("mass", lambda: m.mass(0), C),
                               ("free_energy", lambda: m.free_energy(0, kappa=GAMMA), 2 * C + 2 * R)):
        call()
        ts = []
        for _ in range(reps):
            t0 = time.perf_counter()
            call()
            ts.append(time.perf_counter() - t0)
        t = sorted(ts)[len(ts) // 2]
        out[name] = {"us_per_call": t * 1e6, "bytes_algorithmic": nbytes, "GBps": nbytes / t / 1e9,
                     "includes": "launches, FP64 partial sums and the host synchronisation"}
    out["free_energy_value"] = m.free_energy(0, kappa=GAMMA)[2]
    return out


def warmup_steps(args) -> int:
    """Untimed warm-up steps (at least 3).  The graphs the timed steps replay are captured
    beforehand by prepare_graphs, so the warm-up needs no minimum of its own."""
    return max(args.warmup, 3)


def ch3d_model(G, prec, c0, device, stream, dims=None):
    """The benchmark's model: 3D CH, the examples/cahnHilliard splitting, Euler dt 0.05."""
    m = G.Model(dims or DIMS, prec, device=device)
    m.add_field("conc")
    m.add_scalar("gamma", GAMMA)
    m.add_scalar("M", M)
    m.add_scalar("m1", -M)
    m.add_equation(CH_EQ)
    m.init()
    m.set_stepper("euler", DT)
    if stream is not None:
        m.set_stream(stream.cuda_stream)
    m.set_option(G._lib.OPT_CHECK_FINITE, 0)
    m.upload(0, c0)
    return m


def timed_steps(m, torch, stream, k):
    """Device time (ms) of k graph-replayed steps, CUDA events on the stepping stream."""
    m.prepare_graphs(k)
    m.step(3)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    m.step(k)
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1)


def measure_precision(args, G, torch, c0, n, stream, fp32_rate, oracle_run):
    """The metric's other clauses on the same workload:
    - the FP64 device mode's steps/s (the same kernels' FP64 form) and the FP32/FP64 ratio;
    - FP64 device against the FP64 oracle after the steps the CPU baseline took (full size);
    - FP32 against FP64 device after `precision_steps` steps (1000: the metric's horizon):
      rel-L2 and each run's mass drift per cell."""
    out = {}
    if oracle_run is not None:
        k, ofield = oracle_run
        a = ch3d_model(G, "fp64", c0, 0, stream)
        a.step(k)
        d = a.download_real(0)
        out["fp64_vs_oracle"] = {"steps": k, "rel_l2": float(np.linalg.norm(d - ofield) / np.linalg.norm(ofield)),
                                 "tolerance": 1e-11}
        a.close()
    k64 = 20
    a = ch3d_model(G, "fp64", c0, 0, stream)
    ms = timed_steps(a, torch, stream, k64)
    a.close()
    fp64_rate = k64 / (ms / 1000.0)
    out["fp64_steps_per_s"] = fp64_rate
    out["fp32_over_fp64"] = fp32_rate / fp64_rate
    S = args.precision_steps
    if S > 0:
        a32 = ch3d_model(G, "fp32", c0, 0, stream)
        a64 = ch3d_model(G, "fp64", c0, 0, stream)
        a32.step(S)
        a64.step(S)
        d32, d64 = a32.download_real(0), a64.download_real(0)
        out["fp32_vs_fp64"] = {"steps": S, "rel_l2": float(np.linalg.norm(d32 - d64) / np.linalg.norm(d64)),
                               "tolerance": 1e-4,
                               "mass_drift_per_cell": {"fp32": abs(a32.mass(0) - c0.sum()) / n,
                                                       "fp64": abs(a64.mass(0) - c0.sum()) / n}}
        a32.close()
        a64.close()
    return out


def run_e2e(args, m, stream, c0, n, world, dist, torch, G):
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    host = torch.empty(2 * n, dtype=torch.float64, pin_memory=True)
    host.numpy()[0::2] = c0
    host.numpy()[1::2] = 0.0
    ptr = host.data_ptr()
    import ctypes

    L = G.load()
    dp = ctypes.cast(ptr, ctypes.POINTER(ctypes.c_double))
    k_e2e = max(3, min(args.steps, 50))
    for _ in range(2):
        m._ck(L.gopf_field_upload(m.handle, 0, dp, n))
        m.step(1)
        m._ck(L.gopf_field_download(m.handle, 0, dp, n))
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    t0 = time.perf_counter()
    e0.record(stream)
    for _ in range(k_e2e):
        m._ck(L.gopf_field_upload(m.handle, 0, dp, n))
        m.step(1)
        m._ck(L.gopf_field_download(m.handle, 0, dp, n))
    e1.record(stream)
    torch.cuda.synchronize()
    e2e_ms = max(e0.elapsed_time(e1), (time.perf_counter() - t0) * 1000.0)
    if dist:
        t = torch.tensor([e2e_ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_ms = float(t.item())
    link = host_link(torch, host, stream)
    bound = 1.0 / (16 * n / (link["h2d_gbs"] * 1e9) + 16 * n / (link["d2h_gbs"] * 1e9))
    value = world * k_e2e / (e2e_ms / 1000.0)
    # the step's own copies alone, at the link's measured rates, allow `bound` steps/s per GPU
    link.update({"bound_steps_per_s": bound * world, "frac": value / (bound * world)})
    return {"value": value, "unit": UNIT, "h2d_bytes_per_step": 16 * n,
            "d2h_bytes_per_step": 16 * n, "steps": k_e2e, "host_link": link,
            "path": "gopf_field_upload ([]complex128, pinned) + gopf_step(1) + gopf_field_download per step"}


def host_link(torch, host, stream, reps=5):
    """Copy-engine bandwidth of the host link for the e2e buffer (pinned host <-> device, one
    direction at a time), timed with CUDA events on the stepping stream."""
    dev = torch.empty(host.numel(), dtype=host.dtype, device="cuda")
    nbytes = host.numel() * host.element_size()
    out = {}
    with torch.cuda.stream(stream):
        for key, dst, src in (("h2d_gbs", dev, host), ("d2h_gbs", host, dev)):
            dst.copy_(src, non_blocking=True)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(reps):
                dst.copy_(src, non_blocking=True)
            e1.record(stream)
            torch.cuda.synchronize()
            out[key] = reps * nbytes / (e0.elapsed_time(e1) * 1e-3) / 1e9
    del dev
    return out


def emit(args, world, rank, value, per_step_ms, mass0, mass1, finite, prof, dom, hbm, peak_kind, achieved,
         step_bytes, e2e, clocks, n, cpu, precision, gpu_launches, monitors=None):
    out = None
    if rank == 0:
        out = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": warmup_steps(args), "ms_per_step": per_step_ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": config({"parallelism": "replicas" if world > 1 else "single GPU",
                              "cell_updates_per_s": value * n,
                              "step_bytes_algorithmic": step_bytes,
                              "step_fraction_of_hbm": (step_bytes * value / world / 1e9) / hbm,
                              "mass_drift_per_cell": abs(mass1 - mass0) / n, "finite": bool(finite),
                              "precision": precision,
                              "monitors": monitors,
                              "per_pass_gbs": {p["name"]: p["bytes"] / p["ms"] / 1e6 for p in prof if p["ms"] > 0},
                              "per_pass_frac_of_hbm": {p["name"]: p["bytes"] / p["ms"] / 1e6 / hbm
                                                       for p in prof if p["ms"] > 0}}),
            "e2e": e2e,
            "roofline": {"bound": "hbm", "kernel": dom["name"], "achieved": achieved, "peak": hbm,
                         "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / hbm,
                         "traffic": NCU_TRAFFIC.get(dom["name"]),
                         "per_kernel": [{"name": p["name"], "ms": p["ms"], "GBps": p["bytes"] / p["ms"] / 1e6,
                                         "bytes": p["bytes"]} for p in prof]},
            "cpu_baseline": cpu,
            "clocks": clocks,
            "gpu_launches": gpu_launches,
        }
        print(json.dumps(out))
    return out


SWEEP_SIDES = [128, 256, 384, 512, 768, 1024]


def sweep_params(n=64, seed=2):
    """64 instances: side uniform over SWEEP_SIDES, gamma ~ U(0.2, 2), M ~ U(0.5, 2) (SplitMix64, seed 2)."""
    from gopf_gb300.synthetic import splitmix64_uniform

    u = splitmix64_uniform(seed, 3 * n)
    return [(SWEEP_SIDES[min(int(u[3 * i] * 6), 5)], 0.2 + 1.8 * u[3 * i + 1], 0.5 + 1.5 * u[3 * i + 2])
            for i in range(n)]


def sweep_models(prec, params, fast=True, first=0, indices=None, device=0):
    """Contexts of the sweep instances `indices` (default: all of `params`, numbered from `first`);
    instance i starts from c0 = 0.5 + U(-0.05, 0.05) with seed 1000 + i."""
    import gopf_gb300 as G
    from gopf_gb300.synthetic import uniform_field

    if indices is None:
        indices = list(range(first, first + len(params)))
        params = dict(zip(indices, params))
    models = []
    for i in indices:
        side, gamma, Mv = params[i]
        m = G.Model([side, side], prec, device=device)
        m.set_option(G._lib.OPT_FAST_KERNELS, int(fast))
        m.set_option(G._lib.OPT_CHECK_FINITE, 0)
        m.add_field("conc")
        m.add_scalar("gamma", gamma)
        m.add_scalar("M", Mv)
        m.add_scalar("mM", -Mv)
        m.add_equation("dconc/dt = M*LAP conc^3 + mM*LAP conc + mM*gamma*LAP^2 conc")
        m.init()
        m.set_stepper("euler", 0.05)
        m.upload(0, uniform_field(1000 + i, side * side, 0.5, 0.05))
        models.append(m)
    return models


def run_sweep(args):
    """Batched parameter sweep: 64 independent 2D CH instances of uneven size, FP32, dt 0.05.
    Under torchrun the instances are sharded over the ranks (gopf_sweep_partition: greedy bin
    packing on cells, no collective on the data path); every rank steps its share as one batch and
    the whole sweep's step time is the slowest rank's.  The total work is fixed (strong scaling)."""
    import torch

    import gopf_gb300 as G
    from gopf_gb300 import sweep

    world, rank, local = dist_setup()
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    params = sweep_params()
    cells_of = [s * s for s, _, _ in params]
    owner, rank_cells = sweep.partition(cells_of, world)
    mine = [i for i, r in enumerate(owner) if r == rank]
    cells = sum(cells_of)
    sweep_bytes = float(sum(6 * (s // 2 + 1) * s * 8 for s, _, _ in params))
    models = sweep_models("fp32", params, indices=mine, device=local)
    batch = G.Batch(models)
    if args.batch_mode != "auto":
        batch.set_mode(G._lib.BATCH_MODE_PERSISTENT if args.batch_mode == "persistent" else G._lib.BATCH_MODE_CHAINS)
    tuned, tune_s = None, None
    if not args.no_tune:
        # the autotuner: kernel family, tile width and plan variant per kind of instance, timed on
        # this rank's instances before the warm-up (fields restored afterwards)
        t0 = time.perf_counter()
        batch.tune(5)
        tune_s = time.perf_counter() - t0
        tuned = {}
        for k, i in enumerate(mine):
            tuned.setdefault(str(params[i][0]), batch.choice(k))
    stream = torch.cuda.Stream()
    batch.set_stream(stream.cuda_stream)
    warm = max(args.warmup, 3)
    batch.step(max(warm, 16))  # warm-up: both graphs of the batch (1 and 16 steps) exist afterwards
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        e0.record(stream)
        batch.step(args.steps)
        e1.record(stream)
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
    ms = e0.elapsed_time(e1)
    if dist:
        t = torch.tensor([ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    batched = args.steps / (ms / 1000.0)
    seq = None
    if world == 1:
        # sequential: every instance stepped by its own launches (own CUDA graphs)
        seq_models = sweep_models("fp32", params)
        for m in seq_models:
            m.set_stream(stream.cuda_stream)
            m.step(3)
        torch.cuda.synchronize()
        kseq = max(3, min(args.steps, 200))
        e0.record(stream)
        for _ in range(kseq):
            for m in seq_models:
                m.step(1)
        e1.record(stream)
        torch.cuda.synchronize()
        seq = kseq / (e0.elapsed_time(e1) / 1000.0)
        for m in seq_models:
            m.close()
    launches = batch.launches(args.steps)
    check = None
    if args.check_steps != 0:
        # per-instance rel-L2 of the FP32 batch against sequential FP64 runs, each rank checking its
        # own instances; the results are merged on the host
        S = args.check_steps if args.check_steps > 0 else 2000
        a = sweep_models("fp32", params, indices=mine, device=local)
        G.Batch(a).step(S)

        def work(idx):
            out = {}
            for i, m in zip(idx, a):
                r = sweep_models("fp64", params, indices=[i], device=local)[0]
                r.step(S)
                ref = r.download_real(0)
                out[i] = float(np.linalg.norm(m.download_real(0) - ref) / np.linalg.norm(ref))
                r.close()
            return out

        errs = sweep.run_sharded(cells_of, work, rank, world)
        check = {"steps": S, "rel_l2_max": max(errs), "rel_l2_median": float(np.median(errs)), "tolerance": 1e-4,
                 "rel_l2": errs}
    if rank == 0:
        out = {"metric": "sweep steps/s (64 uneven 2D CH instances, one step of all instances)", "value": batched,
               "unit": "sweep-steps/s", "n_gpus": world, "steps": args.steps, "warmup": max(warm, 16),
               "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "strong",
               "vs_baseline": None, "dtype": "f32", "data": "synthetic",
               "config": {"workload": "sweep_64_ch2d_uneven_fp32", "sides": [p[0] for p in params], "cells": cells,
                          "dt": 0.05, "params_seed": 2, "init": "c0 = 0.5 + U(-0.05, 0.05), seed 1000 + i",
                          "parallelism": f"instances sharded over {world} GPU(s), no collective"
                                         if world > 1 else "single GPU",
                          "rank_cells": rank_cells,
                          "mode": "persistent" if batch.mode() == G._lib.BATCH_MODE_PERSISTENT else "chains",
                          "tuned": tuned, "tune_seconds": tune_s,
                          "families": "0 line engine, 1 compile-time Stockham, 2 runtime Stockham"},
               "sequential_value": seq, "speedup_vs_sequential": (batched / seq) if seq else None,
               # bytes one sweep step moves: per instance the x pass reads T and writes the group (2C),
               # the fused y pass reads the group and c-hat and writes c-hat and T (4C); FP32,
               # C = (X/2+1) Y 8 B
               "step_bytes_moved": sweep_bytes,
               "fraction_of_hbm": sweep_bytes * batched / (peaks()[0] * 1e9 * world),
               "cell_updates_per_s": batched * cells, "clocks": clk.summary(),
               "gpu_launches": launches, "check": check}
        print(json.dumps(out))
    if dist:
        dist.barrier()
        dist.destroy_process_group()
    return 0


def run_adjoint(args):
    """Adjoint parameter fit workload: 2D CH 512^2, 200 steps, dt 0.05, checkpoints every 20 (FP32 adjoint)."""
    import torch

    from gopf_gb300.adjoint import AdjointCH
    from gopf_gb300.synthetic import uniform_field
    from oracle import adjoint_ref as A

    dims, T, dt, every = [512, 512], 200, 0.05, 20
    c0 = uniform_field(4, 512 * 512, 0.5, 0.05)
    ref64 = AdjointCH(dims, "fp64", dt=dt, nsteps=T, every=every)
    target = ref64.forward(c0, 1.3, 0.8)  # target microstructure from the FP64 forward at gamma*=1.3, M*=0.8
    run = AdjointCH(dims, "fp32", dt=dt, nsteps=T, every=every)
    run.loss_and_grad(c0, 1.0, 1.0, target)  # warm-up
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    reps = max(1, min(args.steps, 5))
    for _ in range(reps):
        loss, dg, dm, dc0 = run.loss_and_grad(c0, 1.0, 1.0, target)
    el = (time.perf_counter() - t0) / reps
    l64, g64, m64, c64 = ref64.loss_and_grad(c0, 1.0, 1.0, target)

    def L(g, m):
        r = ref64.forward(c0, g, m) - target
        return 0.5 * float(r @ r)

    h = 1e-4
    fdg = (L(1.0 + h, 1.0) - L(1.0 - h, 1.0)) / (2 * h)
    fdm = (L(1.0, 1.0 + h) - L(1.0, 1.0 - h)) / (2 * h)
    out = {"metric": "adjoint gradient (gamma, M, c0) of CH 512^2 x 200 steps, FP32, checkpoints every 20",
           "value": 1.0 / el, "unit": "forward+adjoint/s", "n_gpus": 1, "steps": reps, "warmup": 1,
           "ms_per_step": el * 1000.0, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": "f32", "data": "synthetic",
           "config": {"workload": "adjoint_ch2d_512_200steps", "target": "FP64 forward at gamma*=1.3, M*=0.8",
                      "at": "gamma=1.0, M=1.0", "checkpoint_every": every},
           "loss": loss, "grad": {"gamma": dg, "M": dm},
           "fd_fp64": {"gamma": fdg, "M": fdm, "h": h},
           "rel_err_vs_fd": {"gamma": abs(dg - fdg) / abs(fdg), "M": abs(dm - fdm) / abs(fdm)},
           "rel_err_vs_fp64_adjoint": {"gamma": abs(dg - g64) / abs(g64), "M": abs(dm - m64) / abs(m64),
                                       "c0": float(np.linalg.norm(dc0 - c64) / np.linalg.norm(c64))},
           "fp64_adjoint_vs_fd": {"gamma": abs(g64 - fdg) / abs(fdg), "M": abs(m64 - fdm) / abs(fdm)}}
    if args.check_steps > 0:
        cT = ref64.forward(c0, 1.0, 1.0)
        rg, rm, rc0 = A.adjoint(c0, dims, 1.0, 1.0, dt, T, cT - target)
        out["fp64_adjoint_vs_numpy"] = {"gamma": abs(g64 - rg) / abs(rg), "M": abs(m64 - rm) / abs(rm),
                                        "c0": float(np.linalg.norm(c64 - rc0) / np.linalg.norm(rc0))}
    print(json.dumps(out))
    return 0


def _cubic(c11, c12, c44):
    C = np.zeros((3, 3, 3, 3))
    for i in range(3):
        C[i, i, i, i] = c11
    for i in range(3):
        for j in range(i + 1, 3):
            C[i, i, j, j] = c12
            C[j, j, i, i] = c12
            C[i, j, i, j] = c44
            C[j, i, j, i] = c44
    return C


def run_elastic(args):
    """CH + Khachaturyan elasticity, 256^3, FP32: C11=1.0, C12=0.6, C44=0.5, misfit 0.01*I coupled through H(c),
    c0 = 0.3 + U(-0.02, 0.02) (seed 3), M=1, gamma=1, dt=0.02, "- LAP LIN_ELAST" in the CH string."""
    import torch

    import gopf_gb300 as G
    from gopf_gb300.synthetic import uniform_field

    n = 256 ** 3
    c0 = uniform_field(3, n, 0.3, 0.02)
    m = G.Model([256] * 3, "fp32", device=0)
    m.set_option(G._lib.OPT_CHECK_FINITE, 0)
    if args.pdl is not None:
        m.set_option(G._lib.OPT_PDL, args.pdl)
    m.add_field("conc")
    m.add_scalar("gamma", 1.0)
    m.add_scalar("m1", -1.0)
    m.register_elastic("LIN_ELAST", "conc", _cubic(1.0, 0.6, 0.5), np.eye(3) * 0.01)
    m.add_equation("dconc/dt = LAP conc^3 + m1*LAP conc + m1*gamma*LAP^2 conc - LAP LIN_ELAST")
    m.init()
    m.set_stepper("euler", 0.02)
    stream = torch.cuda.Stream()
    m.set_stream(stream.cuda_stream)
    m.upload(0, c0)
    mass0 = m.mass(0)
    m.step(warmup_steps(args))
    m.prepare_graphs(args.steps)  # after the first (unreplayed) elastic step
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(0) as clk:
        e0.record(stream)
        m.step(args.steps)
        e1.record(stream)
        torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    prof = m.profile_step(10)
    step_bytes = sum(p["bytes"] for p in prof)
    hbm, kind = peaks()
    value = args.steps / (ms / 1000.0)
    out = {"metric": "CH + Khachaturyan elasticity steps/s at 256^3 FP32", "value": value, "unit": "steps/s",
           "n_gpus": 1, "steps": args.steps, "warmup": warmup_steps(args), "ms_per_step": ms / args.steps,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
           "config": {"workload": "ch_elastic_3d_256cube_fp32", "C11": 1.0, "C12": 0.6, "C44": 0.5, "misfit": 0.01,
                      "dt": 0.02, "init": "c0 = 0.3 + U(-0.02, 0.02), seed 3"},
           "step_bytes_algorithmic": step_bytes, "step_fraction_of_hbm": step_bytes * value / 1e9 / hbm,
           "mass_drift_per_cell": abs(m.mass(0) - mass0) / n,
           "per_kernel": [{"name": p["name"], "ms": p["ms"], "GBps": p["bytes"] / p["ms"] / 1e6 if p["ms"] > 0 else 0}
                          for p in prof], "clocks": clk.summary(), "gpu_launches": m.kernel_launches(args.steps),
           "elastic_energy_monitor": time_elastic_energy(m)}
    print(json.dumps(out))
    return 0


def time_elastic_energy(m, reps=5):
    """HomogeneousModulusEnergy of the stepped field's indicator (the elastic monitor): median wall time
    of a synchronous call over `reps` calls (the first call, which allocates its work buffers, untimed)."""
    C, mis = _cubic(1.0, 0.6, 0.5), np.eye(3) * 0.01
    e = m.elastic_energy(C, mis, indicator=True)
    ts = []
    for _ in range(reps):
        t0 = time.perf_counter()
        m.elastic_energy(C, mis, indicator=True)
        ts.append(time.perf_counter() - t0)
    return {"value": e, "ms_per_call": sorted(ts)[len(ts) // 2] * 1e3,
            "passes": "x-hat (3 forward passes), the six strain spectra in one kernel, 6 x 3 inverse passes, "
                      "the energy density with FP64 sums"}


def run_c1(args):
    """2D Cahn-Hilliard 128^2 (gamma = 1, M = 1, dt = 0.1, c0 = 0.5 + U(-0.05, 0.05) seed 0), 1000 steps:
    FP64 and FP32 device steps/s (graph replays; the grid is L2-resident, so this is launch- and
    latency-bound, not an HBM roofline case), rel-L2 of both against the committed FP64 oracle
    fixture tests/golden/ch2d_128.npz, and the FP64 CPU oracle's steps/s on the host cores."""
    import torch

    import gopf_gb300 as G
    from gopf_gb300.synthetic import uniform_field
    from oracle import oracle as O

    dims, n, steps = [128, 128], 128 * 128, 1000
    c0 = uniform_field(0, n, 0.5, 0.05)
    ref = np.load(os.path.join(HERE, "tests", "golden", "ch2d_128.npz"))["field"]

    def run(prec):
        m = G.Model(dims, prec, device=0)
        m.set_option(G._lib.OPT_CHECK_FINITE, 0)
        m.add_field("conc")
        m.add_scalar("gamma", 1.0)
        m.add_scalar("M", 1.0)
        m.add_scalar("m1", -1.0)
        m.add_equation(CH_EQ)
        m.init()
        m.set_stepper("euler", 0.1)
        m.upload(0, c0)
        m.prepare_graphs(steps)
        m.step(warmup_steps(args))
        m.upload(0, c0)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        m.step(steps)
        m.synchronize()
        rate = steps / (time.perf_counter() - t0)
        err = float(np.linalg.norm(m.download_real(0) - ref) / np.linalg.norm(ref))
        return rate, err

    r64, e64 = run("fp64")
    r32, e32 = run("fp32")
    O.build()
    o = O.cahn_hilliard(dims, gamma=1.0, M=1.0)
    o.set_field(0, c0)
    t0 = time.perf_counter()
    o.step_euler(0.1, steps)
    cpu = steps / (time.perf_counter() - t0)
    out = {"metric": "2D CH 128^2 steps/s (1000 steps) and rel-L2 vs the FP64 oracle fixture",
           "workload": "cahn_hilliard_2d_128_gamma1_dt0.1", "fp64_steps_per_s": r64, "fp64_rel_l2": e64,
           "fp32_steps_per_s": r32, "fp32_rel_l2": e32,
           "cpu_baseline": {"value": cpu, "unit": "steps/s", "cores": O.num_threads(), "kind": "port",
                            "sample": "the same 1000 FP64 Euler steps on the host cores"},
           "note": "16k cells: L2-resident, launch/latency-bound"}
    print(json.dumps(out))
    return 0


def run_precision(args):
    """3D CH 256^3: FP64 device mode steps/s, FP64 device vs the FP64 oracle at full size (few steps),
    FP32 vs FP64 device rel-L2 and mass drift after --check-steps steps."""
    import torch

    import gopf_gb300 as G
    from gopf_gb300.synthetic import uniform_field
    from oracle import oracle as O

    n = 256 ** 3
    c0 = uniform_field(SEED, n, 0.0, 0.1)

    def mk(prec):
        m = G.Model(DIMS, prec, device=0)
        m.set_option(G._lib.OPT_CHECK_FINITE, 0)
        m.add_field("conc")
        m.add_scalar("gamma", GAMMA)
        m.add_scalar("M", M)
        m.add_scalar("m1", -M)
        m.add_equation(CH_EQ)
        m.init()
        m.set_stepper("euler", DT)
        m.upload(0, c0)
        return m

    m64 = mk("fp64")
    m64.step(3)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    m64.step(args.steps)
    m64.synchronize()
    fp64_rate = args.steps / (time.perf_counter() - t0)
    # FP64 device against the FP64 oracle at full size
    k = 5
    a = mk("fp64")
    a.step(k)
    o = O.cahn_hilliard(DIMS, gamma=GAMMA, M=M)
    o.set_field(0, c0)
    o.step_euler(DT, k)
    ref = o.field(0).real
    fp64_vs_oracle = float(np.linalg.norm(a.download_real(0) - ref) / np.linalg.norm(ref))
    del o
    # FP32 vs FP64 device after check_steps
    S = args.check_steps if args.check_steps > 0 else 1000
    a32, a64 = mk("fp32"), mk("fp64")
    hist = []
    done = 0
    for s in sorted(set([10, 50, 100, 200, 500, S])):
        if s > S:
            continue
        a32.step(s - done)
        a64.step(s - done)
        done = s
        d32, d64 = a32.download_real(0), a64.download_real(0)
        hist.append({"step": s, "rel_l2_fp32_vs_fp64": float(np.linalg.norm(d32 - d64) / np.linalg.norm(d64))})
    out = {"metric": "CH 256^3: FP64 device steps/s and FP32-vs-FP64 accuracy", "fp64_steps_per_s": fp64_rate,
           "fp64_vs_oracle": {"steps": k, "rel_l2": fp64_vs_oracle},
           "fp32_vs_fp64": hist, "mass_drift_per_cell": {"fp32": abs(a32.mass(0) - c0.sum()) / n,
                                                         "fp64": abs(a64.mass(0) - c0.sum()) / n}}
    print(json.dumps(out))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=500)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--cpu-seconds", type=float, default=20.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-monitors", action="store_true", help="skip the monitor timings (config.monitors)")
    ap.add_argument("--no-precision", action="store_true",
                    help="skip the FP64 rate and the FP32-vs-FP64 / FP64-vs-oracle checks of the default line")
    ap.add_argument("--precision-steps", type=int, default=1000,
                    help="steps of the FP32-vs-FP64 device comparison in the default line")
    ap.add_argument("--grid", type=int, default=256, help="cube side (256 is the benchmark workload)")
    ap.add_argument("--workload", default="ch3d", choices=["ch3d", "sweep", "adjoint", "elastic", "precision", "c1"])
    ap.add_argument("--x-rows", type=int, default=None, choices=[16, 32],
                    help="rows per tile of the 256-column x pass (the library's default when omitted)")
    ap.add_argument("--z-lines", type=int, default=None, choices=[8, 16],
                    help="lines per tile of the 256-point z pass (the library's default when omitted)")
    ap.add_argument("--tma", type=int, default=None, choices=[0, 1],
                    help="tile movement of the 256-point kernels: 0 plain loads, 1 TMA")
    ap.add_argument("--pdl", type=int, default=None, choices=[0, 1],
                    help="programmatic dependent launches in the 3D step (the library's default when omitted)")
    ap.add_argument("--no-tune", action="store_true", help="sweep: keep the built-in kernel choices")
    ap.add_argument("--batch-mode", default="auto", choices=["auto", "persistent", "chains"],
                    help="sweep: one persistent kernel per captured graph, or a launch per class and pass")
    ap.add_argument("--check-steps", type=int, default=-1,
                    help="sweep: per-instance rel-L2 against FP64 after this many steps (-1: the configuration's "
                         "2000; 0: no check)")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "sweep":
        return run_sweep(args)
    if args.workload == "adjoint":
        return run_adjoint(args)
    if args.workload == "elastic":
        return run_elastic(args)
    if args.workload == "precision":
        return run_precision(args)
    if args.workload == "c1":
        return run_c1(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
