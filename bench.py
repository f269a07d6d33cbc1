"""Benchmark of the GB300 BT-MZ / SP-MZ ADI time step.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                    [--workload bt-c|sp-c|bt-b|sp-b|sp-a|lu-c|lu-b|lu-a]

A step is one time step of the node loop -- exch_qbc over all zones, then adi
(compute_rhs, x/y/z line solves, add) over all zones -- on the workload's
resident state.  The default workload is BT-MZ on the 480x320x28 grid split
16x16 into geometrically growing zones (area ratio 20.8, 256 zones, dt 1e-4):
the largest configuration, run batched (one launch per phase for all zones),
with FP32 line solves refined against an FP64 residual, replayed as one CUDA
graph per step.  Inputs are seeded synthetic manufactured solutions.

`value` is Mgridpt-steps/s with the state resident in HBM (5.4 GB with the
line scratch, far larger than the 129 MB L2, so no flush is needed); `e2e` is
the same metric through the C ABI with the reference-layout arrays in
page-locked host memory, copied in and out every step (npbmz_step_inout).
With N > 1 GPUs each rank runs an independent replica; the zone sharding of
one problem over several GPUs (npbmz.shard) is not what this times.

The lu-* workloads time LU-MZ's SSOR iteration instead (a step is one
iteration: exch_qbc + ssor of every zone, src/LU/lu-node.jl:233-270), FP64
throughout, bit-exact with the oracle, replayed as one CUDA graph.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
for _p in (ROOT, ROOT / "npbapps.jl_gb300"):
    if str(_p) not in sys.path:
        sys.path.insert(0, str(_p))

import numpy as np  # noqa: E402

WORKLOADS = {
    # name: (kind, class geometry, description)
    "bt-c": ("BT", "C", "BT-MZ 480x320x28, 16x16 geometric zones (area ratio 20.8), dt 1e-4"),
    "sp-c": ("SP", "C", "SP-MZ 480x320x28, 16x16 equal zones (30x20x28), dt 6.7e-4"),
    "bt-b": ("BT", "B", "BT-MZ 304x208x17, 8x8 geometric zones (area ratio 20.05), dt 3e-4"),
    "sp-b": ("SP", "B", "SP-MZ 304x208x17, 8x8 equal zones (38x26x17), dt 1e-3"),
    "sp-a": ("SP", "A", "SP-MZ 128x128x16, 4x4 equal zones (32x32x16), dt 1.5e-3"),
    "lu-c": ("LU", "C", "LU-MZ 480x320x28, 4x4 equal zones (120x80x28), dt 2.0, omega 1.2"),
    "lu-b": ("LU", "B", "LU-MZ 304x208x17, 4x4 equal zones (76x52x17), dt 2.0, omega 1.2"),
    "lu-a": ("LU", "A", "LU-MZ 128x128x16, 4x4 equal zones (32x32x16), dt 2.0, omega 1.2"),
}
# LU-MZ: algorithmic HBM bytes per grid point of each phase (FP64, every
# point of the zones): jac reads u and 1/u1 (48 B) and writes 120 planes of
# blocks and factors per interior point (960 B); the sweeps read rsd and the
# 66 planes of their direction (rsd in, rsd out: 80 B + 528 B); rhs reads u,
# frct and ten planes of flux quantities and writes rsd (200 B); update reads
# u and rsd and writes u and the flux quantities (200 B).
LU_BYTES_PER_POINT = {"jac": 1008.0, "lower": 608.0, "upper": 608.0, "rhs": 200.0, "update": 200.0, "exch": 0.0}
LU_KERNELS = {"jac": "k_lu_jac", "lower": "k_lu_lower<1>", "upper": "k_lu_upper", "rhs": "k_lu_rhs<0>",
              "update": "k_lu_pointwise<1>", "exch": "k_lu_pack+k_lu_unpack"}
SEED = 20261203
# Algorithmic HBM bytes per grid point of each phase (the 600 B/pt-step model:
# FP64 state, intermediates and line-solve scratch kept out of the count):
# compute_rhs reads u and forcing and writes rhs; each sweep reads u and rhs
# and writes rhs; the z sweep also updates u (add); the primitive kernel reads u.
BYTES_PER_POINT = {"prim": 40.0, "rhs": 120.0, "x": 120.0, "y": 120.0, "z": 160.0, "exch": 0.0}
# Kernels of each phase of the batched step (for the per-kernel ncu figures).
_SWEEPS = {
    "BT": {"x": ["k_bt_mixed_pl<0>", "k_bt_refine_pl<0, 1>", "k_xline_back"],
           "y": ["k_bt_mixed_pl<1>", "k_bt_refine_pl<1, 1>"],
           "z": ["k_bt_mixed_pl<2>", "k_bt_refine_pl<2, 0>"]},
    "SP": {"x": ["k_sp_mixed_pl<0>", "k_sp_refine_pl<0, 1>", "k_xline_back"],
           "y": ["k_sp_mixed_pl<1>", "k_sp_refine_pl<1, 1>"],
           "z": ["k_sp_mixed_pl<2>", "k_sp_refine_pl<2, 0>"]},
}
PHASE_KERNELS = {
    ("BT", "mixed"): {"prim": ["k_prim_w<0>", "k_xline_copy<0>"], "rhs": ["k_rhs_flux<0, 0>"], **_SWEEPS["BT"]},
    ("SP", "mixed"): {"prim": ["k_prim_w<1>", "k_xline_copy<1>"], "rhs": ["k_rhs_flux<1, 0>"], **_SWEEPS["SP"]},
    ("BT", "mixed-dfrhs"): {"prim": ["k_prim_df<0>", "k_xline_copy<0>"], "rhs": ["k_rhs_df<0, 0, 1>"], **_SWEEPS["BT"]},
    ("SP", "mixed-dfrhs"): {"prim": ["k_prim_df<1>", "k_xline_copy<1>"], "rhs": ["k_rhs_df<1, 0, 1>"], **_SWEEPS["SP"]},
}


def workload_config(desc, pts, nzones, world, variant, seed=None, escale=None):
    """The `config` object of both arms' JSON lines: the same keys and values
    for the GPU arm and the reference arm, except `variant`."""
    cfg = {"workload": desc, "points_per_gpu": pts, "zones": nzones, "variant": variant,
           "l2": f"u, rhs and forcing {3 * 40 * pts / 1e9:.2f} GB > 129 MB L2; no flush",
           "parallelism": f"replicas x{world}"}
    if seed is not None:
        cfg["seed"] = seed
        cfg["energy_row_scale"] = 2 ** escale
    else:
        cfg["ce"] = "the reference's table"
    return cfg


def plural(n, noun):
    return f"{n} {noun}" + ("" if n == 1 else "s")


def env_rank():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("LOCAL_RANK", "0"))


def peaks():
    try:
        return json.loads((ROOT / "MEASURED_PEAKS.json").read_text())
    except Exception:
        return {}


def geometry(npbmz, kind, cls):
    niter, dt, ratio, xz, yz, gx, gy, gz = npbmz.CLASSES[kind][cls]
    k = npbmz.KINDS[kind]
    nx, ny, nz, nbr = npbmz.zone_setup(k, gx, gy, gz, xz, yz, ratio)
    return npbmz.Geometry(k, nx, ny, nz, nbr, gx, gy, gz, xz, yz), dt


class ClockSampler:
    """nvidia-smi samples (every 20 ms) while the timed region runs; entering
    waits for the first sample so that sampling covers the region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap,clocks.mem,clocks.max.mem")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "20"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
            t0 = time.time()
            while not self.lines and time.time() - t0 < 5.0 and self.proc.poll() is None:
                time.sleep(0.01)
            self.lines.clear()  # samples from before the region starts
        except Exception:
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
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, mem, memx, reasons = [], [], [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            try:
                mem.append(float(f[9]))
                memx.append(float(f[10]))
            except (ValueError, IndexError):
                pass
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)), "reasons": sorted(reasons),
                "samples": len(sm), "mem_mhz": float(np.median(mem)) if mem else None,
                "mem_max_mhz": float(max(memx)) if memx else None}


def time_steps(p, torch, stream, steps, warmup, dist=None):
    p.step(warmup)
    stream.synchronize()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    p.step(steps)
    e1.record(stream)
    e1.synchronize()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    return e0.elapsed_time(e1)


def whole_job(ms_local, pts, steps, world, dist=None, device="cuda"):
    """Replicas: every rank runs the workload on its own GPU; the job's time is
    the slowest rank's (max over ranks) and its value counts the points of
    all ranks.  Returns (ms_max, Mgridpt-steps/s)."""
    import torch

    t = torch.tensor([float(ms_local)], dtype=torch.float64, device=device)
    if dist is not None:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    ms_max = float(t.item())
    return ms_max, pts * world * steps / (ms_max * 1e-3) / 1e6


def phase_times(p, nsteps):
    """Per-phase device time of the batched step -- the kernels the timed
    steps run -- from CUDA events the library records around each phase on
    its stream (npbmz_step_profile)."""
    p.step_profile(1)  # warm
    return p.step_profile(nsteps)


def kernel_metrics(workload, variant):
    """Per-point ncu figures of the step kernels (profiles/ncu_kernel_metrics.json):
    from a capture of this workload, else of the class-B workload of the same
    kind (same kernels, 1.07 M points), per point."""
    try:
        allm = json.loads((ROOT / "profiles" / "ncu_kernel_metrics.json").read_text())
    except Exception:
        return None, None
    for w in (workload, workload[:2] + "-b"):
        m = allm.get(w, {}).get(variant)
        if m:
            return m, w
    return None, None


def cpu_baseline(kind, cls, ce, target_s=15.0):
    """The oracle (CPU restatement of the reference path) on the host cores,
    OpenMP over zones like the reference's Threads.@threads: a bounded sample
    of the same workload."""
    from oracle import oracle

    import npbmz

    niter, dt, ratio, xz, yz, gx, gy, gz = npbmz.CLASSES[kind][cls]
    k = npbmz.KINDS[kind]
    nx, ny, nz, nbr = oracle.zone_setup(k, gx, gy, gz, xz, yz, ratio)
    pts = int(np.sum(nx.astype(np.int64) * ny * nz))
    o = oracle.Oracle(k, nx, ny, nz, nbr, dt, gx, gy, gz, xz, yz, ce)
    t0 = time.perf_counter()
    o.step(1)
    t1 = time.perf_counter() - t0
    n = max(1, min(50, int(target_s / max(t1, 1e-3))))
    t0 = time.perf_counter()
    o.step(n)
    t = time.perf_counter() - t0
    cores = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    return {"value": pts * n / t / 1e6, "unit": "Mgridpt-steps/s", "cores": cores, "kind": "port",
            "sample": f"{plural(n, 'full time step')} of the {kind}-MZ class {cls} grid ({pts} points, all zones) "
                      "after 1 untimed step"}


def lu_cpu_run(cls, warmup, steps):
    """The LU-MZ oracle on the host cores (OpenMP over zones, like the
    reference's Threads.@threads): seconds for `steps` iterations after
    `warmup`, and the point count."""
    from oracle import oracle

    import npbmz

    niter, dt, ratio, xz, yz, gx, gy, gz = npbmz.CLASSES["LU"][cls]
    g = oracle.lu_zone_setup(gx, gy, gz, xz, yz, ratio)
    pts = int(np.sum(g[0].astype(np.int64) * g[1] * g[2]))
    o = oracle.LuOracle(*g, dt, faces_npb=False)
    o.iterate(warmup)
    t0 = time.perf_counter()
    o.iterate(steps)
    return time.perf_counter() - t0, pts, len(g[0])


def lu_cpu_baseline(cls, target_s=15.0):
    t1, pts, _ = lu_cpu_run(cls, 0, 1)
    n = max(1, min(50, int(target_s / max(t1, 1e-3))))
    t, pts, _ = lu_cpu_run(cls, 1, n)
    cores = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    return {"value": pts * n / t / 1e6, "unit": "Mgridpt-steps/s", "cores": cores, "kind": "port",
            "sample": f"{plural(n, 'SSOR iteration')} of the LU-MZ class {cls} grid ({pts} points, all zones) "
                      "after 1 untimed iteration"}


def run_reference(args):
    rank, world, _ = env_rank()
    if rank != 0:
        return 0
    import npbmz

    kind, cls, desc = WORKLOADS[args.workload]
    if kind == "LU":
        t, pts, nzones = lu_cpu_run(cls, args.warmup, args.steps)
        value = pts * args.steps / t / 1e6
        cores = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
        line = {
            "impl": "reference", "metric": "Mgridpt-steps/s", "value": value, "unit": "Mgridpt-steps/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": t / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": workload_config(desc, pts, nzones, world, "reference CPU path (LU-MZ oracle port), FP64"),
            "cpu_baseline": {"value": value, "unit": "Mgridpt-steps/s", "cores": cores, "kind": "port",
                             "sample": f"{plural(args.steps, 'SSOR iteration')} after "
                                       f"{plural(args.warmup, 'warm-up iteration')}"},
            "e2e": {"value": value, "unit": "Mgridpt-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        }
        print(json.dumps(line), flush=True)
        return 0
    niter, dt, ratio, xz, yz, gx, gy, gz = npbmz.CLASSES[kind][cls]
    from oracle import oracle

    # the oracle alone: zone set-up, seeded coefficients and the time steps
    # (no product library is loaded in this arm)
    k = npbmz.KINDS[kind]
    nx, ny, nz, nbr = oracle.zone_setup(k, gx, gy, gz, xz, yz, ratio)
    ce, escale = oracle.seeded_coefficients(SEED, nx, ny, nz, gx, gy, gz, xz, yz)
    pts = int(np.sum(nx.astype(np.int64) * ny * nz))
    o = oracle.Oracle(k, nx, ny, nz, nbr, dt, gx, gy, gz, xz, yz, ce)
    o.step(args.warmup)
    t0 = time.perf_counter()
    o.step(args.steps)
    t = time.perf_counter() - t0
    value = pts * args.steps / t / 1e6
    cores = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    line = {
        "impl": "reference", "metric": "Mgridpt-steps/s", "value": value, "unit": "Mgridpt-steps/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": t / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": workload_config(desc, pts, len(nx), world, "reference CPU path (oracle port), FP64", SEED, escale),
        "cpu_baseline": {"value": value, "unit": "Mgridpt-steps/s", "cores": cores, "kind": "port",
                         "sample": f"{plural(args.steps, 'full time step')} after {plural(args.warmup, 'warm-up step')}"},
        "e2e": {"value": value, "unit": "Mgridpt-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def run_gpu_lu(args, cls, desc):
    """LU-MZ: one step = one SSOR iteration of every zone (exch_qbc + ssor)."""
    import torch

    import npbmz
    from npbmz import lu

    rank, world, local = env_rank()
    dist = None
    if world > 1:
        import torch.distributed as tdist

        tdist.init_process_group("nccl")
        dist = tdist
    torch.cuda.set_device(local)
    stream = torch.cuda.Stream()
    flags = lu.GRAPH | (lu.FMA if args.variant == "fma-graph" else 0)

    def make(fl):
        p = lu.LuProblem.from_class(cls, fl)
        p.set_stream(stream.cuda_stream)
        p.setup()
        return p

    p = make(flags)
    pts = p.points

    def timed(q, steps, warmup):
        q.iterate(warmup)
        stream.synchronize()
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        q.iterate(steps)
        e1.record(stream)
        e1.synchronize()
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        return e0.elapsed_time(e1)

    with ClockSampler(local) as clk:
        ms = timed(p, args.steps, args.warmup)
    ms_max, value = whole_job(ms, pts, args.steps, world, dist)
    extra = {}
    nprof = max(2, min(args.steps, 5))
    if rank == 0 and args.quick:
        extra["phase_ms"] = {k: v / nprof for k, v in p.profile(nprof).items()}
    elif rank == 0:
        # per-iteration device time of each phase (events around the phases
        # of nprof iterations, direct launches)
        ph = {k: v / nprof for k, v in p.profile(nprof).items()}
        extra["phase_ms"] = ph
        top = max((k for k in ph if k != "exch"), key=lambda k: ph[k])
        pk = peaks()
        hbm = float(pk.get("hbm_gbs", 6800.0))
        interior = int(np.sum((p.nx.astype(np.int64) - 2) * (p.ny - 2) * (p.nz - 2)))
        units = interior if top in ("jac", "lower", "upper") else pts
        achieved = LU_BYTES_PER_POINT[top] * units / (ph[top] * 1e-3) / 1e9
        fp64 = npbmz.fp64_peak_gflops()
        km = None
        try:
            km = json.loads((ROOT / "profiles" / "ncu_kernel_metrics.json").read_text()).get(args.workload, {}).get("lu")
        except Exception:
            km = None
        kn = LU_KERNELS[top]
        traffic = fp64_obj = None
        if km and kn in km:
            traffic = km[kn]["dram_bytes_per_point"] * units
            fl = km[kn]["fp64_flops_per_point"]
            fa = fl * units / (ph[top] * 1e-3) / 1e9
            fp64_obj = {"achieved": fa, "peak": fp64, "unit": "GFLOP/s", "frac": fa / fp64, "flops_per_point": fl,
                        "pipe_active_ncu": km[kn]["fp64_pipe_active"],
                        "peak_source": "npbmz_fp64_peak: FP64 FMA chains on this GPU, measured in this run"}
        hbm_obj = {"achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                   "bytes_per_point": LU_BYTES_PER_POINT[top],
                   "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)" if "hbm_gbs" in pk else "fallback 6800 GB/s"}
        binding = "fp64" if fp64_obj and fp64_obj["pipe_active_ncu"] > 0.6 else "hbm"
        head = fp64_obj if binding == "fp64" else hbm_obj
        extra["roofline"] = {"bound": binding, "kernel": kn, "phase": top, "achieved": head["achieved"],
                             "peak": head["peak"], "unit": head["unit"], "frac": head["frac"], "traffic": traffic,
                             "traffic_source": ("ncu dram__bytes_read.sum + dram__bytes_write.sum per point of this "
                                                "workload's capture (profiles/ncu_kernel_metrics.json), times its points")
                             if traffic is not None else None,
                             "points": f"{units} ({'interior' if units == interior else 'all'} points per launch)",
                             "launch_ms": ph[top], "hbm": hbm_obj, "fp64": fp64_obj}
        extra["fp64_peak_gflops_measured"] = fp64
        var = {}
        for name, fl in (("fp64_batched", 0), ("fp64_batched_graph", lu.GRAPH),
                         ("fp64_batched_graph_npb_faces", lu.GRAPH | lu.FACES_NPB),
                         ("fp64_fma_batched_graph (not bit-exact)", lu.GRAPH | lu.FMA)):
            q = make(fl)
            mv = timed(q, max(2, min(args.steps, 5)), 1)
            var[name] = pts * max(2, min(args.steps, 5)) / (mv * 1e-3) / 1e6
            q.close()
        extra["variants_mgridpt_steps_per_s"] = var
        # e2e through the C ABI: the reference-layout u of every zone in
        # page-locked host memory, uploaded and downloaded every iteration
        sizes = [lu.ref_elems(int(p.nx[z]), int(p.ny[z]), int(p.nz[z])) for z in range(p.nzones)]
        host = torch.empty(int(sum(sizes)), dtype=torch.float64, pin_memory=True)
        L = lu.lib()
        ptr = host.data_ptr()
        assert L.npbmz_lu_download(p._h, -1, lu.U, npbmz.LAYOUT_REF, ptr) == 0
        for _ in range(args.warmup):
            assert L.npbmz_lu_upload(p._h, -1, lu.U, npbmz.LAYOUT_REF, ptr) == 0
            p.iterate(1)
            assert L.npbmz_lu_download(p._h, -1, lu.U, npbmz.LAYOUT_REF, ptr) == 0
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            assert L.npbmz_lu_upload(p._h, -1, lu.U, npbmz.LAYOUT_REF, ptr) == 0
            p.iterate(1)
            assert L.npbmz_lu_download(p._h, -1, lu.U, npbmz.LAYOUT_REF, ptr) == 0
        te = time.perf_counter() - t0
        moved = 5 * 8 * pts  # the interior points of the reference arrays, each way
        extra["e2e"] = {"value": pts * world * args.steps / te / 1e6, "unit": "Mgridpt-steps/s",
                        "h2d_bytes_per_step": moved, "d2h_bytes_per_step": moved, "step_groups": best_g,
                        "ms_per_call_by_step_groups": {str(k): round(v, 3) for k, v in e2e_groups.items()},
                        "path": "npbmz_lu_upload + npbmz_lu_iterate(1) + npbmz_lu_download (zone=-1, "
                                "NPBMZ_LAYOUT_REF) on page-locked reference-layout u, read and written in place "
                                "(interior points only) by one kernel per zone each way"}
        if not args.no_cpu_baseline:
            extra["cpu_baseline"] = lu_cpu_baseline(cls)
    if rank == 0:
        line = {
            "metric": "Mgridpt-steps/s", "value": value, "unit": "Mgridpt-steps/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": workload_config(desc, pts, p.nzones, world,
                                      "fma-graph (not bit-exact)" if flags & lu.FMA else "fp64-graph (bit-exact)"),
            "variant_detail": {"batched": True, "cuda_graph": True, "exch_planes": "reference (k = 1..nz-2)"},
            "gpu_launches": p.launches_per_iteration() * args.steps,
            "clocks": clk.summary(),
        }
        line.update(extra)
        print(json.dumps(line), flush=True)
    p.close()
    if dist:
        dist.barrier()
        dist.destroy_process_group()
    return 0


def run_gpu(args):
    import torch

    import npbmz

    kind_, cls_, desc_ = WORKLOADS[args.workload]
    if kind_ == "LU":
        return run_gpu_lu(args, cls_, desc_)
    rank, world, local = env_rank()
    dist = None
    if world > 1:
        import torch.distributed as tdist

        tdist.init_process_group("nccl")
        dist = tdist
    torch.cuda.set_device(local)
    stream = torch.cuda.Stream()
    kind, cls, desc = WORKLOADS[args.workload]
    g, dt = geometry(npbmz, kind, cls)
    pts = g.points
    ce, escale = npbmz.seeded_coefficients(SEED, g.nx, g.ny, g.nz, g.gx, g.gy, g.gz, g.x_zones, g.y_zones)
    flags = {"mixed-graph": npbmz.MIXED | npbmz.GRAPH, "fp64-graph": npbmz.GRAPH,
             "mixed-dfrhs-graph": npbmz.MIXED | npbmz.RHS_DF | npbmz.GRAPH,
             "mixed": npbmz.MIXED, "fp64": 0}[args.variant]

    def make(fl):
        p = npbmz.Problem(g, dt, fl)
        p.set_stream(stream.cuda_stream)
        p.setup(ce)
        return p

    p = make(flags)
    tuned = None
    if not args.quick and not args.no_autotune:
        # launch shapes, zone-group branches and persistent kernels, chosen by
        # timing whole steps on this handle (results unchanged)
        p.autotune()
        p.setup(ce)
        d = p.describe()
        tuned = {k: d[k] for k in ("lines_per_cta", "zone_size_buckets", "step_groups", "fp64_priority",
                                   "sweep_ctas_per_sm", "persistent", "copy_fusion")}
    with ClockSampler(local) as clk:
        ms = time_steps(p, torch, stream, args.steps, args.warmup, dist)
    ms_max, value = whole_job(ms, pts, args.steps, world, dist)
    # the step kernels of every timed step, and the one state-check kernel
    # that ends the npbmz_step call
    launches = p.launches_per_step * args.steps + 1

    extra = {}
    if rank == 0 and args.quick:
        ph = phase_times(p, max(3, min(args.steps, 10)))
        extra["phase_ms"] = ph
    elif rank == 0:
        # per-phase device times of the timed variant's kernels -> dominant kernel roofline
        ph = phase_times(p, max(3, min(args.steps, 10)))
        top = max((k for k in ph if k != "exch"), key=lambda k: ph[k])
        pk = peaks()
        hbm = float(pk.get("hbm_gbs", 6800.0))
        achieved = BYTES_PER_POINT[top] * pts / (ph[top] * 1e-3) / 1e9
        fp64 = npbmz.fp64_peak_gflops()
        km, km_src = kernel_metrics(args.workload, args.variant)
        pk_key = (kind, "mixed-dfrhs" if flags & npbmz.RHS_DF else "mixed")
        knames = list(PHASE_KERNELS.get(pk_key, {}).get(top, [])) if flags & npbmz.MIXED else []
        # the state copy made by the compute_rhs launch (npbmz_set_copy_fusion):
        # its ncu figures count with compute_rhs, not with the primitive phase
        fused_copy = bool(p.describe().get("copy_fusion")) and not flags & npbmz.RHS_DF
        copy_k = [k for k in PHASE_KERNELS.get(pk_key, {}).get("prim", []) if k.startswith("k_xline_copy")]
        if fused_copy and top == "prim":
            knames = [k for k in knames if k not in copy_k]
        elif fused_copy and top == "rhs":
            knames += copy_k
        traffic = None
        issue_obj = None
        fp64_obj = None
        if km and knames and all(k in km for k in knames):
            traffic = sum(km[k]["dram_bytes_per_point"] for k in knames) * pts
            flops_pt = sum(km[k]["fp64_flops_per_point"] for k in knames)
            if flops_pt > 1.0:
                fp64_ach = flops_pt * pts / (ph[top] * 1e-3) / 1e9
                fp64_obj = {"achieved": fp64_ach, "peak": fp64, "unit": "GFLOP/s", "frac": fp64_ach / fp64,
                            "flops_per_point": flops_pt,
                            "pipe_active_ncu": max(km[k]["fp64_pipe_active"] for k in knames),
                            "peak_source": "npbmz_fp64_peak: FP64 FMA chains on this GPU, measured in this run"}
            if all("inst_per_point" in km[k] for k in knames):
                # instruction issue: 4 schedulers per SM, one warp instruction per cycle each
                inst_pt = sum(km[k]["inst_per_point"] for k in knames)
                nsm = torch.cuda.get_device_properties(local).multi_processor_count
                mhz = clk.summary().get("sm_mhz") or 2070.0
                peak_gi = 4 * nsm * mhz * 1e-3
                ach_gi = inst_pt / 32 * pts / (ph[top] * 1e-3) / 1e9
                issue_obj = {"achieved": ach_gi, "peak": peak_gi, "unit": "G warp-inst/s", "frac": ach_gi / peak_gi,
                             "inst_per_point": inst_pt,
                             "issue_active_ncu": {k: km[k]["issue_active"] for k in knames},
                             "warps_per_sm_ncu": {k: km[k]["warps_per_sm"] for k in knames},
                             "peak_source": "4 warp instructions per SM cycle x SMs x median SM clock of the timed run"}
        hbm_obj = {"achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                   "bytes_per_point": BYTES_PER_POINT[top],
                   "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)" if "hbm_gbs" in pk else "fallback 6800 GB/s"}
        binding = ("fp64" if fp64_obj and fp64_obj["pipe_active_ncu"] > 0.6
                   else "issue" if issue_obj and issue_obj["frac"] > hbm_obj["frac"] else "hbm")
        head = {"fp64": fp64_obj, "issue": issue_obj, "hbm": hbm_obj}[binding]
        kname = "+".join(knames) if knames else top
        if fused_copy and top == "rhs" and knames:
            kname = f"k_rhs_flux_xc (one launch: {kname})"
        extra["roofline"] = {"bound": binding, "kernel": kname, "phase": top,
                             "achieved": head["achieved"], "peak": head["peak"], "unit": head["unit"],
                             "frac": head["frac"], "launch_ms": ph[top], "points": pts,
                             "traffic": traffic,
                             "traffic_source": (f"ncu dram__bytes_read.sum + dram__bytes_write.sum per point, {km_src} "
                                                "capture (profiles/ncu_kernel_metrics.json), times this workload's points")
                             if traffic is not None else None,
                             "hbm": hbm_obj, "fp64": fp64_obj, "issue": issue_obj}
        # the whole step against both ceilings: the 600 B/pt HBM model and the
        # FP64 instructions of every kernel of the step (ncu, per point)
        step_ms = ms_max / args.steps
        step_obj = {"ms_per_step": step_ms, "points": pts, "bytes_per_point": 600.0,
                    "hbm_achieved_gbs": 600.0 * pts / (step_ms * 1e-3) / 1e9, "hbm_peak_gbs": hbm}
        step_obj["hbm_frac"] = step_obj["hbm_achieved_gbs"] / hbm
        step_obj["hbm_floor_ms"] = 600.0 * pts / (hbm * 1e9) * 1e3
        kall = [k for k in (km or {}) if not k.startswith("_")] if flags & npbmz.MIXED else []
        if kall:
            fl_step = sum(km[k]["fp64_flops_per_point"] for k in kall)
            step_obj.update({"fp64_flops_per_point": fl_step, "fp64_peak_gflops": fp64,
                             "fp64_floor_ms": fl_step * pts / (fp64 * 1e9) * 1e3,
                             "fp64_kernels": sorted(kall)})
            step_obj["fp64_floor_frac"] = step_obj["fp64_floor_ms"] / step_ms
        extra["roofline_step"] = step_obj
        extra["phase_ms"] = ph
        extra["fp64_peak_gflops_measured"] = fp64
        # variants (fewer steps each)
        var = {}
        nv = max(3, min(args.steps, 10))
        for name, fl in (("fp64_batched", 0), ("fp64_exact_batched", npbmz.EXACT),
                         ("mixed_batched", npbmz.MIXED), ("mixed_batched_graph", npbmz.MIXED | npbmz.GRAPH),
                         ("fp64_batched_graph", npbmz.GRAPH),
                         ("mixed_batched_graph_persistent", npbmz.MIXED | npbmz.GRAPH | npbmz.PERSIST),
                         ("mixed_double_float_rhs_batched_graph (compute_rhs not FP64)",
                          npbmz.MIXED | npbmz.RHS_DF | npbmz.GRAPH),
                         ("fp64_perzone", npbmz.PERZONE)):
            q = make(fl)
            steps_v = 2 if fl & npbmz.PERZONE else nv
            mv = time_steps(q, torch, stream, steps_v, 1)
            var[name] = pts * steps_v / (mv * 1e-3) / 1e6
            q.close()
        extra["variants_mgridpt_steps_per_s"] = var
        # accuracy of the timed variant against the plain FP64 GPU path (which
        # the parity tests hold to the oracle) over the measured number of steps
        nacc = args.warmup + args.steps
        a = make(0)
        a.step(nacc)
        xa = np.concatenate(a.verify())
        a.close()
        b = make(flags)
        b.step(nacc)
        xb = np.concatenate(b.verify())
        b.close()
        extra["accuracy"] = {"steps": nacc, "max_rel_err_final_norms_vs_fp64": float(np.max(np.abs(xb - xa) / np.abs(xa)))}
        # e2e through the C ABI: reference-layout u in page-locked host memory,
        # uploaded and downloaded every step
        sizes = [npbmz.ref_elems(g.kind, npbmz.U, int(g.nx[z]), int(g.ny[z]), int(g.nz[z])) for z in range(g.nzones)]
        host = torch.empty(int(sum(sizes)), dtype=torch.float64, pin_memory=True)
        q = p  # the timed (tuned) handle
        q.transfer_raw(npbmz.U, -1, npbmz.LAYOUT_REF, host.data_ptr(), False)
        ptr = host.data_ptr()
        # the zone-group count of the overlapped copies: more groups start the
        # compute sooner after the copy in and leave less to copy out at the
        # end; chosen by timing 4 calls per candidate (results unchanged)
        e2e_groups = {}
        for G in (2, 4, 6, 8):
            q.set_step_groups(G)
            q.step_inout(1, npbmz.LAYOUT_REF, ptr, ptr)
            t0 = time.perf_counter()
            for _ in range(4):
                q.step_inout(1, npbmz.LAYOUT_REF, ptr, ptr)
            e2e_groups[G] = (time.perf_counter() - t0) / 4 * 1e3
        best_g = min(e2e_groups, key=e2e_groups.get)
        q.set_step_groups(best_g)
        for _ in range(args.warmup):
            q.step_inout(1, npbmz.LAYOUT_REF, ptr, ptr)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            q.step_inout(1, npbmz.LAYOUT_REF, ptr, ptr)
        te = time.perf_counter() - t0
        moved = 5 * 8 * pts
        extra["e2e"] = {"value": pts * world * args.steps / te / 1e6, "unit": "Mgridpt-steps/s",
                        "h2d_bytes_per_step": moved, "d2h_bytes_per_step": moved, "step_groups": best_g,
                        "ms_per_call_by_step_groups": {str(k): round(v, 3) for k, v in e2e_groups.items()},
                        "path": "npbmz_step_inout(1, NPBMZ_LAYOUT_REF) per step on one page-locked buffer holding "
                                "every zone's reference-layout u: the planes exch_qbc reads by a kernel from host "
                                "memory, then each zone group's arrays by the copy engine while earlier groups "
                                "compute (group branches at priorities falling with the group number, so groups "
                                "finish in arrival order), and each group back by the copy engine when its last z "
                                "sweep is done (halo bytes travel unchanged; the counts above are the interior "
                                "points)"}
        if not args.no_cpu_baseline:
            extra["cpu_baseline"] = cpu_baseline(kind, cls, ce)
    if rank == 0:
        line = {
            "metric": "Mgridpt-steps/s", "value": value, "unit": "Mgridpt-steps/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64+f32" if flags & npbmz.MIXED else "f64",
            "data": "synthetic",
            "config": workload_config(desc, pts, g.nzones, world, args.variant, SEED, escale),
            "variant_detail": {"batched": True, "cuda_graph": bool(flags & npbmz.GRAPH),
                               "line_solves": ("fp32 + double-float-residual refinement; primitives and compute_rhs "
                                               + ("double-float" if flags & npbmz.RHS_DF else "fp64"))
                               if flags & npbmz.MIXED else "fp64",
                               "autotuned": tuned, "device_bytes": p.device_bytes},
            "gpu_launches": launches,
            "clocks": clk.summary(),
        }
        line.update(extra)
        print(json.dumps(line), flush=True)
    p.close()
    if dist:
        dist.barrier()
        dist.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="bt-c", choices=sorted(WORKLOADS))
    ap.add_argument("--variant", default="mixed-graph",
                    choices=["mixed-graph", "fp64-graph", "mixed-dfrhs-graph", "mixed", "fp64", "fma-graph"],
                    help="BT/SP step variant; lu-* workloads: fma-graph times NPBMZ_LU_FMA, anything else the "
                         "bit-exact build")
    ap.add_argument("--no-autotune", action="store_true",
                    help="time the default launch configuration (the timed handle is autotuned otherwise)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--quick", action="store_true",
                    help="only the timed variant and its phase times (for profiler runs)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
