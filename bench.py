"""Benchmark: GDoF/s of the matrix-free hexahedral operator action on GB300.

Workload (the benchmark configuration the headline metric is quoted on):
stiffness action, degree P=4 (125 DOFs/cell), Q=6 Gauss points per axis,
32768 cells, affine Jacobians J = I + 0.1 N(0,1), G = detJ w J^-1 J^-T as 6
components per point, u ~ U(-1,1); FP64 storage and arithmetic (the plain
FP64 path).  The same workload is also timed in FP32 and reported under
"variants".  Inputs (405 MB in FP64) exceed the 129 MB L2, so no L2 flush is
needed between steps.

A step is one operator application over all cells.  `value` is timed with
inputs resident in HBM; `e2e` goes through the host-buffer C-ABI entry point
(femtc_stiffness_apply_host) with pinned host buffers, so each step includes
the host->device copy of u and G and the device->host copy of y.

The default run also measures the other benchmark configurations in the
same process and reports them under "extra": mass P=3 at 4096 cells, the
precision workload (stiffness P=6, Q=8, 131072 cells, every form's error
against the FP64 oracle), the 64-mesh batch (one graph launch) and the
serving stream (p50/p99).  --extra none skips them.

--impl reference times the CPU implementation of the same operator on the
host cores instead (the reference's algorithm restated in C, OpenMP over
cells, FP64, built with the reference's -Ofast and native-ISA flags): that is
the reference arm.  It loads nothing of the GPU library.

Multi-GPU: cells are independent (the operator is block diagonal), so N
ranks run N independent replicas of the workload (weak scaling, no data
exchange); the step time is the max over ranks.  --gpus N without a
launcher's environment starts the N ranks itself (torch.distributed.run).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import tempfile
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

PEAKS_FILE = os.path.join(ROOT, "MEASURED_PEAKS.json")
# FP64 FMA throughput of a GB300, measured with an FMA-throughput kernel
# (8 independent FMA chains per thread on every SM, CUDA events); the
# measured-peaks file (HBM copy, bf16 GEMM) carries no FP64 figure.
FP64_PEAK_TFLOPS = 1.20
FALLBACK_HBM_GBS = 6800.0
L2_BYTES = 129e6  # GB300 L2


def flops_per_cell(op: int, n: int, q: int) -> float:
    if op == 0:
        return 4.0 * q * n * (n * n + q * n + q * q) + q ** 3
    return 4.0 * q * n * (2 * n * n + 3 * q * n + 3 * q * q) + 15.0 * q ** 3


def _eo_mv_flops(m: int, k: int, sig: int) -> int:
    """FP64 operations (FMA = 2) of one even-odd contraction, M outputs from
    K inputs, as the kernels' mv_eo executes it."""
    m2, mm, k2, km = m // 2, m % 2, k // 2, k % 2
    mid = (2 * (k2 + km) - 1) if sig > 0 else (2 * k2 - 1)
    return 2 * k2 + m2 * (4 * k2 + 2 * km) + mm * mid


def flops_per_cell_even_odd(op: int, n: int, q: int) -> float:
    """Operations the even-odd kernels execute per cell (forward_eo, fused
    pass, backward_eo in cell_kernel.cuh); the achieved rate of the FP64 pipe
    is this count over the kernel time."""
    grad = op != 0
    n2, nm, q2, qm = n // 2, n % 2, q // 2, q % 2
    mv_f = lambda s: _eo_mv_flops(q, n, s)   # N -> Q
    mv_b = lambda s: _eo_mv_flops(n, q, s)   # Q -> N
    # forward, per slab
    emit = mv_f(1) + (mv_f(-1) + mv_f(1) if grad else 0)
    pair_row = (4 * n2 + 2 * nm) * (2 if grad else 1)
    mid_row = (2 * (n2 + nm) - 1) + ((2 * n2 - 1) if grad else 0)
    fwd = n * 2 * n2 + q2 * (n * pair_row + 2 * emit) + qm * (n * mid_row + emit)
    # fused, per pencil
    if grad:
        fused = 3 * mv_f(1) + 15 * q + 3 * mv_b(1)
    else:
        fused = mv_f(1) + q + mv_b(1)
    # backward, per slab
    col = mv_b(1) + ((mv_b(-1) + n + mv_b(1)) if grad else 0)
    pair_acc = n * ((2 + 4 * n2 + 2 * nm) * (2 if grad else 1))
    mid_col = n * (2 * n2 * (2 if grad else 1) + 2 * nm)
    bwd = q2 * (2 * col + pair_acc) + qm * (col + mid_col) + n * 2 * n2
    return float(n * fwd + q * q * fused + n * bwd)


def _eo_mv_instr(m: int, k: int, sig: int) -> int:
    """Arithmetic instructions (FMA, MUL, ADD: one each) of mv_eo."""
    m2, mm, k2, km = m // 2, m % 2, k // 2, k % 2
    mid = (k2 + km) if sig > 0 else k2
    return 2 * k2 + m2 * (2 * k2 + km + 2) + mm * mid


def pipe_instr_per_cell(op: int, n: int, q: int, even_odd: bool, affine: bool = False) -> float:
    """FP64-pipe instructions per cell: every FMA, MUL and ADD takes one
    issue slot of the pipe, so this (not the flop count) is what the pipe's
    busy fraction measures.  Plain kernels: one FMA per multiply-add plus
    the point-wise work; even-odd kernels: as their code runs.  Affine mass
    scales each pencil's N inputs by detJ instead of its Q points."""
    grad = op != 0
    pw = (9 * q ** 3) if grad else (n ** 3 if affine else q ** 3)  # point-wise work
    if not even_odd:
        macs = flops_per_cell(op, n, q) - (15 if grad else 1) * q ** 3
        return macs / 2 + pw
    n2, nm, q2, qm = n // 2, n % 2, q // 2, q % 2
    mv_f = lambda s: _eo_mv_instr(q, n, s)
    mv_b = lambda s: _eo_mv_instr(n, q, s)
    emit = mv_f(1) + (mv_f(-1) + mv_f(1) if grad else 0)
    pair_row = (2 * n2 + nm + 2) * (2 if grad else 1)
    mid_row = (n2 + nm) + (n2 if grad else 0)
    fwd = n * 2 * n2 + q2 * (n * pair_row + 2 * emit) + qm * (n * mid_row + emit)
    fused = (3 * mv_f(1) + 3 * mv_b(1)) if grad else (mv_f(1) + mv_b(1))
    col = mv_b(1) + ((mv_b(-1) + n + mv_b(1)) if grad else 0)
    pair_acc = n * ((2 + 2 * n2 + nm) * (2 if grad else 1))
    mid_col = n * (n2 * (2 if grad else 1) + nm)
    bwd = q2 * (2 * col + pair_acc) + qm * (col + mid_col) + n * 2 * n2
    return float(n * fwd + q * q * fused + pw + n * bwd)


def bytes_per_cell(op: int, n: int, q: int, es: int, affine: bool = False) -> float:
    """u in, y out, and the geometry: per point, or one set per cell (affine)."""
    return es * (2 * n ** 3 + (1 if op == 0 else 6) * (1 if affine else q ** 3))


# DRAM bytes (read + write) of one launch of the headline kernels, from one
# ncu capture (dram__bytes_read.sum + dram__bytes_write.sum) of each kernel on
# the full workload
MEASURED_TRAFFIC = {("stiffness_p4", 32768, 0): 399.7e6, ("stiffness_p4", 32768, 1): 196.7e6}


def traffic_for(workload, ncells, dtype):
    return MEASURED_TRAFFIC.get((workload, ncells, dtype))


def roofline(head, ach_tf, ach_gbs, hbm, hbm_src, traffic=None, flop_count=None, pipe_frac=None):
    """The binding roof of the headline kernel: the FP64 pipe for FP64 (its
    arithmetic intensity puts it far above the FP64 ridge), HBM otherwise."""
    hbm_part = {"achieved": ach_gbs, "peak": hbm, "unit": "GB/s", "frac": ach_gbs / hbm,
                "peak_source": hbm_src}
    if head == 0:
        return {"bound": "fp64", "achieved": ach_tf, "peak": FP64_PEAK_TFLOPS, "unit": "TFLOP/s",
                "frac": ach_tf / FP64_PEAK_TFLOPS, "flop_count": flop_count,
                "fp64_pipe_instruction_frac": pipe_frac, "traffic": traffic,
                "traffic_unit": "DRAM bytes per launch (ncu dram__bytes_read.sum + "
                                "dram__bytes_write.sum, one capture of this kernel on this workload)",
                "peak_source": "measured FP64 FMA rate of a GB300 (FMA-throughput kernel, "
                               "CUDA events)",
                "hbm": hbm_part}
    return {"bound": "hbm", "achieved": ach_gbs, "peak": hbm, "unit": "GB/s", "frac": ach_gbs / hbm,
            "traffic": traffic, "peak_source": hbm_src}


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi clock/throttle sampling during the timed region."""

    def __init__(self, index: int):
        self.proc = None
        self.index = index
        self.path = os.path.join(tempfile.gettempdir(), f"femtc_clocks_{os.getpid()}_{index}.csv")

    def __enter__(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index),
                 "--query-gpu=index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=self.fh, stderr=subprocess.DEVNULL)
            time.sleep(0.3)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.fh.close()

    def summary(self):
        if self.proc is None or not os.path.exists(self.path):
            return None
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for name, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def host_link_gbs(dev, nbytes=1 << 30, reps=5):
    """Pinned host<->device copy bandwidth (GB/s, each direction alone),
    timed with CUDA events, best of `reps` copies (the link is shared with
    the host's other traffic): the ceiling of every host-buffer call."""
    import torch
    h = torch.empty(nbytes, dtype=torch.uint8, pin_memory=True)
    h.fill_(1)  # touch every page before timing
    d = torch.empty(nbytes, dtype=torch.uint8, device=dev)
    s = torch.cuda.current_stream()
    out = []
    for dst, src in ((d, h), (h, d)):
        dst.copy_(src, non_blocking=True)
        torch.cuda.synchronize()
        best = 0.0
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(s)
            dst.copy_(src, non_blocking=True)
            e1.record(s)
            torch.cuda.synchronize()
            best = max(best, nbytes / (e0.elapsed_time(e1) * 1e-3) / 1e9)
        out.append(best)
    del h, d
    return out[0], out[1]


def peaks():
    try:
        with open(PEAKS_FILE) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


def metric_name(base: int, degree: int, nquad: int) -> str:
    return f"GDoF/s {'stiffness' if base == 1 else 'mass'} action (P={degree}, Q={nquad})"


def workload_config(w, world: int, es: int) -> dict:
    """The `config` of an operator workload's line (both arms)."""
    bpc = bytes_per_cell(w.base_op, w.n, w.nquad, es, w.affine)
    flush = bpc * w.ncells < 1.5 * L2_BYTES
    return {"workload": w.name, "cells": w.ncells, "degree": w.degree, "nquad": w.nquad,
            "dofs": w.ndofs, "parallelism": f"replicas{world}",
            "geometry": ("affine: one factor set per cell, weights in the backward tables"
                         if w.affine else "per quadrature point"),
            "l2": (f"inputs {bpc * w.ncells / 1e6:.0f} MB "
                   + ("< 1.5 x 129 MB L2: a 512 MB write between launches flushes it; "
                      "time = sum of the launches' events" if flush
                      else "> 1.5 x 129 MB L2, no flush"))}


def _cpu_fn(base):
    import oracle
    return oracle.mass if base == 0 else oracle.stiffness


def cpu_sample(w, fn, cores, seconds):
    """Cells per call for a call of about `seconds` on `cores` threads,
    calibrated on a short call."""
    import oracle
    c0 = int(min(w.ncells, max(64, 32 * cores)))
    g = w.point_geometry(c0)
    fn(oracle.EXACT, w.degree, w.nquad, w.tables, w.u[:c0], g, nthreads=cores, fast=True)
    t0 = time.perf_counter()
    fn(oracle.EXACT, w.degree, w.nquad, w.tables, w.u[:c0], g, nthreads=cores, fast=True)
    per_cell = max((time.perf_counter() - t0) / c0, 1e-9)
    return int(min(w.ncells, max(c0, seconds / per_cell)))


def run_reference(args, rank, world):
    """CPU arm: the oracle's C restatement of the reference's algorithm,
    built with the reference's -Ofast and native-ISA flags, OpenMP over
    cells on every host core; tables from the oracle's own tabulation, so
    nothing of the GPU library is loaded.  Rank 0 only."""
    if rank != 0:
        return
    import oracle
    from femtc_gb300 import workloads as W
    if args.workload in ("batch64", "serve"):
        print(json.dumps({"impl": "reference", "unavailable":
                          "the reference has no batched or serving path (one operator of one "
                          "degree per call, src/mass.hpp:196-219)"}), flush=True)
        return
    w = W.make(args.workload, ncells=args.cells, tabulate=oracle.tabulate)
    n, q = w.n, w.nquad
    cores = os.cpu_count() or 1
    fn = _cpu_fn(w.op)
    # bounded sample per step: about 1.5 s of CPU work on all host cores
    sample = cpu_sample(w, fn, cores, 1.5)
    u, g = w.u[:sample], w.geo[:sample]
    times = []
    for i in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        fn(oracle.EXACT, w.degree, q, w.tables, u, g, nthreads=cores, fast=True)
        t1 = time.perf_counter()
        if i >= args.warmup:
            times.append(t1 - t0)
    t = float(np.mean(times))
    gdofs = sample * n ** 3 / t / 1e9
    line = {
        "metric": metric_name(w.op, w.degree, q),
        "value": gdofs, "unit": "GDoF/s", "impl": "reference", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": t * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "config": workload_config(w, world, 8),
        "cpu_baseline": {"value": gdofs, "unit": "GDoF/s", "cores": cores, "kind": "port",
                         "sample": f"{sample} of {w.ncells} cells per step, FP64, exact "
                                   f"operator, OpenMP over cells",
                         "flags": oracle.fast_flags()},
        "e2e": {"value": gdofs, "unit": "GDoF/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def cpu_baseline(w, seconds=10.0):
    """Time the oracle's C restatement (its -Ofast native-ISA build) on the
    host cores on a bounded sample (affine workloads: the per-point operator
    on the same mesh, the only form the reference has), and on one core."""
    import oracle
    cores = os.cpu_count() or 1
    fn = _cpu_fn(w.base_op)
    sample = cpu_sample(w, fn, cores, 0.5)
    u, g = w.u[:sample], w.point_geometry(sample)
    reps, t0 = 0, time.perf_counter()
    while True:
        fn(oracle.EXACT, w.degree, w.nquad, w.tables, u, g, nthreads=cores, fast=True)
        reps += 1
        el = time.perf_counter() - t0
        if el >= seconds:
            break
    v = reps * sample * w.n ** 3 / el / 1e9
    # one core on a 1/16 sample, for the per-core figure
    s1 = max(16, sample // 16)
    u1, g1 = u[:s1], g[:s1]
    reps1, t0 = 0, time.perf_counter()
    while True:
        fn(oracle.EXACT, w.degree, w.nquad, w.tables, u1, g1, nthreads=1, fast=True)
        reps1 += 1
        el1 = time.perf_counter() - t0
        if el1 >= seconds / 4:
            break
    return {"value": v, "unit": "GDoF/s", "cores": cores, "kind": "port",
            "sample": f"{reps} x {sample} cells of the workload, FP64, exact operator, "
                      f"OpenMP over cells, {el:.1f} s",
            "flags": oracle.fast_flags(),
            "value_1core": reps1 * s1 * w.n ** 3 / el1 / 1e9,
            "sample_1core": f"{reps1} x {s1} cells, one thread, {el1:.1f} s"}


def run_batch(args, rank, world, dev, pg):
    """64 meshes of mixed degree and operator in one persistent launch
    (CUDA graph), against the same meshes as 64 single-mesh launches."""
    import torch
    import femtc_gb300 as F
    from femtc_gb300 import workloads as W
    spec = W.batch64_spec()
    if args.cells:  # scale the cell counts down (small meshes / profiling)
        spec = [(op, P, max(1, n * args.cells // 100000)) for op, P, n in spec]
    gen = torch.Generator(device=dev).manual_seed(1004)
    rng = np.random.default_rng(1004)
    meshes, meshes64 = [], []
    for op, P, n in spec:
        Q = P + 2
        tables, _, wts, _ = F.tabulate(P, Q)
        J = torch.from_numpy(W.random_jacobians(rng, n).reshape(n, 9)).to(dev)
        u = torch.rand(n, (P + 1) ** 3, device=dev, generator=gen, dtype=torch.float32) * 2 - 1
        y = torch.empty_like(u)
        shape = (n, Q ** 3) if op == F.MASS else (n, Q ** 3, 6)
        geo = torch.empty(shape, device=dev, dtype=torch.float32)
        geo64 = torch.empty(shape, device=dev, dtype=torch.float64)
        for dt, g in ((F.F32, geo), (F.F64, geo64)):
            if op == F.MASS:
                F.geometry(dt, Q, wts, J, g, None, n)
            else:
                F.geometry(dt, Q, wts, J, None, g, n)
        meshes.append((op, P, Q, tables.astype(np.float32), u, y, geo, n))
        u64 = u.double()
        meshes64.append((op, P, Q, tables, u64, torch.empty_like(u64), geo64, n))
    torch.cuda.synchronize()
    ndofs = sum(n * (P + 1) ** 3 for _, P, n in spec)
    nbytes = sum(4 * (2 * (P + 1) ** 3 + (1 if op == 0 else 6) * (P + 2) ** 3) * n for op, P, n in spec)
    stream = torch.cuda.current_stream()
    out = {}

    def timed(step):
        for _ in range(args.warmup):
            step()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            step()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / args.steps

    # the plain FP64 path on the same meshes, one launch per mesh: the
    # denominator of the mixed-precision speed-up and the accuracy reference
    def step64():
        for op, P, Q, tables, u64, y64, geo64, n in meshes64:
            F.apply(op, F.F64, F.EXACT, P, Q, tables, u64, y64, geo64, n, stream)
    ms64 = timed(step64)
    out["f64"] = {"separate": {"ms": ms64, "gdofs": ndofs / ms64 / 1e6,
                               "hbm_gbs": 2 * nbytes / ms64 / 1e6}}

    # every mesh's error against the FP64 oracle on its first cells (the
    # FP64 geometry the GPU computed, copied back)
    import oracle
    err_cells = [min(n, 128) for _, _, n in spec]
    oracle_y = []
    for (op, P, Q, tables, u64, y64, geo64, n), k in zip(meshes64, err_cells):
        fn = oracle.mass if op == F.MASS else oracle.stiffness
        oracle_y.append(fn(oracle.EXACT, P, Q, tables, u64[:k].cpu().numpy(),
                           geo64[:k].cpu().numpy()))

    def max_rel_err():
        worst = 0.0
        for m32, yo, k in zip(meshes, oracle_y, err_cells):
            y = m32[5][:k].double().cpu().numpy()
            worst = max(worst, float(np.abs(y - yo).max() / np.abs(yo).max()))
        return worst

    for dtype in (F.F32, F.BF16X3, F.F16X2):
        b = F.Batch(dtype, meshes, tune=not args.no_batch_tune)
        res = {}
        for mode in ("graph", "eager", "separate"):
            def step():
                if mode == "graph":
                    b.launch(stream)
                elif mode == "eager":
                    b.launch_eager(stream)
                else:
                    for op, P, Q, tab, u, y, geo, n in meshes:
                        F.apply(op, dtype, F.EXACT, P, Q, tab, u, y, geo, n, stream)
            ms = timed(step)
            res[mode] = {"ms": ms, "gdofs": ndofs / ms / 1e6, "hbm_gbs": nbytes / ms / 1e6}
            if mode == "graph":
                res["max_rel_err_vs_fp64_oracle"] = max_rel_err()
        res["speedup_vs_f64_plain"] = res["graph"]["gdofs"] / out["f64"]["separate"]["gdofs"]
        res["info"] = b.info()
        b.close()
        if not args.no_batch_tune:
            # the untuned plan: every mesh in one persistent kernel, one graph
            # launch (the tuner's split plan above may hold several kernels)
            b1 = F.Batch(dtype, meshes, tune=False)
            ms = timed(lambda: b1.launch(stream))
            res["one_kernel_graph"] = {"ms": ms, "gdofs": ndofs / ms / 1e6,
                                       "hbm_gbs": nbytes / ms / 1e6}
            b1.close()
        out[F.DTYPE_NAMES[dtype]] = res
    if F.device_status() != 0:
        raise RuntimeError("device fault word set during the batch benchmark")
    if rank == 0:
        head = out["f32"]["graph"]
        hbm, src = peaks()
        line = {
            "metric": "GDoF/s batched mixed-degree action (64 meshes, one persistent graph launch)",
            "value": head["gdofs"] * world, "unit": "GDoF/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": head["ms"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "batch64", "meshes": len(spec), "dofs": ndofs,
                       "degrees": sorted({P for _, P, _ in spec}),
                       "bytes_per_step": nbytes},
            "roofline": {"bound": "hbm", "achieved": head["hbm_gbs"], "peak": hbm, "unit": "GB/s",
                         "frac": head["hbm_gbs"] / hbm, "traffic": None, "peak_source": src},
            "forms": out,
        }
        return line
    return None


def run_serve(args, rank, world, dev, pg):
    """Serving: a Poisson stream (mean 2000 req/s) of matrix-free solves of
    (M + sigma K) x = b, sigma ~ U(0.1, 10), P ~ U{2..7} (Q = P+2), cells
    log-uniform in [1e3, 2e5], b ~ N(0,1), Jacobi, rel. tol 1e-8 through the
    mixed-precision operator inside FP64 iterative refinement; admission by
    HBM budget, continuous batching.  Latency = completion - arrival."""
    import threading
    import femtc_gb300 as F
    from femtc_gb300 import workloads as W
    rng = np.random.default_rng(1005 + rank)
    nreq = args.requests
    inner = {"f32": F.F32, "f16x2": F.F16X2, "bf16x3": F.BF16X3}[args.inner_dtype]
    probs = []
    for _ in range(nreq):
        P = int(rng.integers(2, 8))
        n = int(round(10 ** rng.uniform(3.0, np.log10(2e5))))
        if args.cells:
            n = max(1, n * args.cells // 200000)
        sigma = float(rng.uniform(0.1, 10.0))
        J = W.random_jacobians(rng, n).reshape(-1, 9)
        b = rng.standard_normal((n, (P + 1) ** 3))
        probs.append(F.Problem(P, P + 2, J, b, alpha=1.0, beta=sigma, rtol=1e-8,
                               inner_dtype=inner))
    # optional operator applications in the same stream (FP64, mass or
    # stiffness, the solves' degree and cell distributions)
    apps = []
    for _ in range(args.serve_applications):
        P = int(rng.integers(2, 8))
        n = int(round(10 ** rng.uniform(3.0, np.log10(2e5))))
        if args.cells:
            n = max(1, n * args.cells // 200000)
        op = int(rng.integers(0, 2))
        w = W.make_custom("serve_apply", op, P, P + 2, n, seed=int(rng.integers(1 << 30)))
        apps.append(F.Application(op, F.F64, F.EXACT, P, P + 2, w.tables, w.u, w.geo))
    kinds = [0] * nreq + [1] * len(apps)
    rng.shuffle(kinds)
    reqs, ia, ip = [], 0, 0
    for k in kinds:
        if k:
            reqs.append(apps[ia])
            ia += 1
        else:
            reqs.append(probs[ip])
            ip += 1
    arrivals = np.cumsum(rng.exponential(1.0 / 2000.0, size=len(reqs)))
    free = torch_free_bytes(dev)
    budget = int(min(free * 0.6, 120e9))
    # warm the kernels used by the solves (setup, outside the timed region)
    for P in range(2, 8):
        wp = F.Problem(P, P + 2, np.tile(np.eye(3).reshape(1, 9), (8, 1)), np.ones((8, (P + 1) ** 3)),
                       inner_dtype=inner)
        F.solve(wp)
    policy = F.SERVE_FIFO if args.serve_policy == "fifo" else F.SERVE_SHORTEST_FIRST
    srv = F.Server(budget, max_active=8, policy=policy)
    tickets = [None] * len(reqs)
    t0 = time.perf_counter()

    def feeder():
        for i, p in enumerate(reqs):
            delay = arrivals[i] - (time.perf_counter() - t0)
            if delay > 0:
                time.sleep(delay)
            tickets[i] = srv.submit_apply(p) if kinds[i] else srv.submit(p)

    th = threading.Thread(target=feeder)
    th.start()
    th.join()
    all_results = [srv.wait(t, 3600.0) for t in tickets]
    wall = time.perf_counter() - t0
    st = srv.stats()
    srv.close()
    results = [r for r, k in zip(all_results, kinds) if not k]
    app_results = [r for r, k in zip(all_results, kinds) if k]
    lat = np.array([r["t_done_ms"] - r["t_submit_ms"] for r in results])
    svc = np.array([r["ms_total"] for r in results])
    ok = sum(1 for r in results if r["rc"] == 0)
    dofs = sum(p.b.size for p in probs)
    if rank == 0:
        line = {
            "metric": "p50/p99 solve latency ms (serving, Poisson 2000 req/s)",
            "value": float(np.percentile(lat, 50)), "unit": "ms", "n_gpus": world,
            "steps": nreq, "warmup": 6, "ms_per_step": wall * 1e3 / nreq,
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
            "dtype": f"{args.inner_dtype}+f64",
            "data": "synthetic",
            "config": {"workload": "serve", "requests": nreq, "arrival_rate_per_s": 2000,
                       "degrees": "2..7", "cells": "log-uniform [1e3, 2e5]", "rtol": 1e-8,
                       "hbm_budget_bytes": budget, "max_active": 8,
                       "admission": args.serve_policy},
            "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
            "service_p50_ms": float(np.percentile(svc, 50)),
            "service_p99_ms": float(np.percentile(svc, 99)),
            "throughput_req_s": nreq / wall, "solved_dofs_per_s": dofs / wall,
            "converged": ok, "max_relres": float(max(r["relres"] for r in results)),
            "max_concurrent": st["max_concurrent"], "peak_hbm_bytes": st["peak_in_use_bytes"],
            "mean_outer_iters": float(np.mean([r["outer_iters"] for r in results])),
            "mean_inner_iters": float(np.mean([r["inner_iters"] for r in results])),
        }
        if app_results:
            alat = np.array([r["t_done_ms"] - r["t_submit_ms"] for r in app_results])
            line["applications"] = {
                "requests": len(app_results), "dtype": "f64",
                "completed_ok": sum(1 for r in app_results if r["rc"] == 0),
                "p50_ms": float(np.percentile(alat, 50)),
                "p99_ms": float(np.percentile(alat, 99)),
                "service_p50_ms": float(np.percentile([r["ms_total"] for r in app_results], 50)),
                "dofs": int(sum(a.u.size for a in apps)),
            }
            line["config"]["operator_applications"] = len(app_results)
        return line
    return None


def box_shape(ncells: int):
    """nx >= ny >= nz with nx*ny*nz = ncells, as near a cube as the factors allow."""
    best = (ncells, 1, 1)
    for nz in range(1, int(round(ncells ** (1 / 3))) + 2):
        if ncells % nz:
            continue
        rest = ncells // nz
        for ny in range(nz, int(rest ** 0.5) + 2):
            if rest % ny == 0 and rest // ny >= ny:
                cand = (rest // ny, ny, nz)
                if max(cand) < max(best):
                    best = cand
    return best


def run_assembled(args, rank, world, dev, pg):
    """The workload's cells as a box mesh with shared (continuous) DOFs,
    through femtc_assembled_apply: gather by the DOF map, the cell operator,
    and the deterministic sum per global DOF.  GDoF/s counts global DOFs."""
    import torch
    import femtc_gb300 as F
    from femtc_gb300 import workloads as W
    w = W.make(args.workload, ncells=args.cells)
    shape = box_shape(w.ncells)
    dm, nd = W.box_dofmap(*shape, w.degree)
    off, ent = F.dofmap_transpose(dm, nd)
    stream = torch.cuda.current_stream()
    n, q, op = w.n, w.nquad, w.op
    forms = {}
    launches = 0
    for dtype in (F.F64, F.F32):
        tdt = torch.float64 if dtype == F.F64 else torch.float32
        dmd, offd, entd = (torch.from_numpy(a).to(dev) for a in (dm, off, ent))
        x = torch.from_numpy(np.random.default_rng(w.seed).uniform(-1, 1, nd)).to(dev, tdt)
        y = torch.empty_like(x)
        g = torch.from_numpy(w.geo).to(dev, tdt)
        work = torch.empty(F.assembled_work_bytes(dtype, w.degree, w.ncells), device=dev,
                           dtype=torch.uint8)
        u = torch.empty((w.ncells, n ** 3), device=dev, dtype=tdt)
        F.autotune(op, dtype, F.EXACT, w.degree, q, w.tables, u, torch.empty_like(u), g, w.ncells,
                   stream)
        del u

        def step():
            F.assembled_apply(op, dtype, F.EXACT, w.degree, q, w.tables, dmd, offd, entd, nd, x, y,
                              g, w.ncells, work, stream)

        for _ in range(args.warmup):
            step()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        l0 = F.operator_launches()
        e0.record(stream)
        for _ in range(args.steps):
            step()
        e1.record(stream)
        torch.cuda.synchronize()
        launches += F.operator_launches() - l0
        ms = replicas_max(e0.elapsed_time(e1), dev, world) / args.steps
        forms[F.DTYPE_NAMES[dtype]] = {"ms": ms, "global_gdofs": world * nd / ms / 1e6,
                                       "cell_gdofs": world * w.ndofs / ms / 1e6}
    if rank == 0:
        head = forms["f64"]
        hbm, src = peaks()
        print(json.dumps({
            "metric": f"GDoF/s assembled {'stiffness' if op == 1 else 'mass'} action "
                      f"(global DOFs, P={w.degree}, Q={q})",
            "value": head["global_gdofs"], "unit": "GDoF/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": head["ms"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": f"{args.workload}_assembled", "cells": w.ncells, "box": shape,
                       "global_dofs": nd, "cell_dofs": w.ndofs, "parallelism": f"replicas{world}"},
            "gpu_launches": launches, "forms": forms, "peak_hbm_gbs": hbm, "peak_source": src,
        }), flush=True)


def replicas_max(x, dev, world):
    if world == 1:
        return x
    from femtc_gb300 import replicas
    return replicas.max_over_ranks(x, device=dev)


def torch_free_bytes(dev):
    import torch
    free, _ = torch.cuda.mem_get_info(dev)
    return free


def run_operator(args, name, dtypes_arg, rank, world, dev, pg, local, e2e_on=True,
                 cpu_seconds=10.0, ncells=None, clocks=True):
    """One operator workload: every form in `dtypes_arg` (the first is the
    headline) with inputs resident in HBM, the host-buffer entry point (e2e)
    and the CPU baseline; returns the line (rank 0) or None."""
    import torch
    import femtc_gb300 as F
    from femtc_gb300 import workloads as W
    from femtc_gb300 import replicas

    w = (W.make_affine if args.geometry == "affine" else W.make)(name, ncells=ncells)
    # op: the entry point's operator code; base: mass (0) or stiffness (1)
    n, q, op, base = w.n, w.nquad, w.op, w.base_op
    tabs = w.op_tables()
    stream = torch.cuda.current_stream()
    names = {v: k for k, v in F.DTYPE_NAMES.items()}
    # "f64plain": FP64 with the even-odd contractions switched off (the plain
    # sum-factorized kernels), for comparison with the default FP64 form
    F64PLAIN = -1
    names["f64plain"] = F64PLAIN
    dname = dict(F.DTYPE_NAMES)
    dname[F64PLAIN] = "f64plain"
    dtypes = [names[d] for d in dtypes_arg.split(",")]
    head = dtypes[0]

    def barrier():
        if pg is not None:
            pg.barrier()
        torch.cuda.synchronize()

    def maxreduce(x):
        return replicas.max_over_ranks(x, device=dev)

    # FP64 oracle on a slice of the workload: every form states its error
    err_cells = min(w.ncells, 2048)
    y_oracle = None
    if rank == 0:
        import oracle
        fn = oracle.mass if base == 0 else oracle.stiffness
        y_oracle = fn(oracle.EXACT, w.degree, q, w.tables, w.u[:err_cells],
                      w.point_geometry(err_cells))

    tuned = False
    if args.tile_db and os.path.exists(args.tile_db):
        F.tile_db_load(args.tile_db)
        tuned = True
    launches_timed = [0]
    results = {}
    for key in dtypes:
        dtype = F.F64 if key == F64PLAIN else key
        if not F.supported(op, dtype, F.EXACT, w.degree, q):
            continue
        F.set_even_odd(key != F64PLAIN)
        tdt = torch.float64 if dtype in F.FP64_STORAGE else torch.float32
        u = torch.from_numpy(w.u).to(dev, tdt)
        g = torch.from_numpy(w.geo).to(dev, tdt)
        y = torch.empty_like(u)

        def step():
            F.apply(op, dtype, F.EXACT, w.degree, q, tabs, u, y, g, w.ncells, stream)

        if not tuned and key != F64PLAIN:  # the project's autotuner, outside the timed region
            F.autotune(op, dtype, F.EXACT, w.degree, q, tabs, u, y, g, w.ncells, stream)
        tile = F.get_tile_config(op, dtype, F.EXACT, w.degree, q)

        # inputs under 1.5x the L2 could be served from it in part by the
        # previous launch: a 512 MB write between launches evicts them, and
        # the time is the sum of the launches' own events
        es = 8 if dtype in F.FP64_STORAGE else 4
        flush = None
        if bytes_per_cell(base, n, q, es, w.affine) * w.ncells < 1.5 * L2_BYTES:
            flush = torch.empty(512 << 20, dtype=torch.uint8, device=dev)
        for _ in range(args.warmup):
            step()
        barrier()
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
              for _ in range(args.steps)]
        sampler = ClockSampler(local) if (key == head and clocks) else None
        if sampler:
            sampler.__enter__()
        barrier()
        t_start = torch.cuda.Event(enable_timing=True)
        t_end = torch.cuda.Event(enable_timing=True)
        l0 = F.operator_launches()
        t_start.record(stream)
        for i in range(args.steps):
            # per-launch events only where a flush separates the launches;
            # back-to-back launches are timed as one region (an event
            # between two launches of ~50 us would add its own gap)
            if flush is not None:
                flush.fill_(i & 255)
                ev[i][0].record(stream)
            step()
            if flush is not None:
                ev[i][1].record(stream)
        t_end.record(stream)
        if key == head:
            launches_timed[0] += F.operator_launches() - l0
        barrier()
        if sampler:
            sampler.__exit__(None, None, None)
        if flush is None:
            total_ms = maxreduce(t_start.elapsed_time(t_end))
            kern_ms = t_start.elapsed_time(t_end) / args.steps
        else:
            total_ms = maxreduce(sum(a.elapsed_time(b) for a, b in ev))
            kern_ms = statistics.mean(a.elapsed_time(b) for a, b in ev)
        err = None
        if y_oracle is not None:
            yo = y[:err_cells].double().cpu().numpy()
            err = float(np.abs(yo - y_oracle).max() / np.abs(y_oracle).max())
        results[key] = dict(total_ms=total_ms, kern_ms=kern_ms, err=err, tile=tile,
                            clocks=sampler.summary() if sampler else None,
                            l2_flush=flush is not None)
        del flush
        F.set_even_odd(True)
        if F.device_status() != 0:
            raise RuntimeError("device fault word set during the benchmark")
        del u, g, y
        torch.cuda.empty_cache()

    if args.tile_db and not tuned and rank == 0:
        F.tile_db_save(args.tile_db)

    # end-to-end through the host-buffer C-ABI entry point, pinned buffers:
    # mode 0 lets the kernel stream the host buffers over the coherent
    # Grace-Blackwell link (zero-copy), mode 1 stages them through device
    # copies; both include every byte's host->device and device->host move
    e2e = {}
    for dtype in ([head] if e2e_on else []):
        npdt = np.float64 if dtype in F.FP64_STORAGE else np.float32
        uh = torch.from_numpy(w.u.astype(npdt)).pin_memory()
        gh = torch.from_numpy(w.geo.astype(npdt)).pin_memory()
        yh = torch.empty_like(uh).pin_memory()

        def estep():
            F.apply_host(op, dtype, F.EXACT, w.degree, q, tabs, uh, yh, gh, w.ncells)

        # tile tuning of the zero-copy path (setup, outside the timed region)
        F.autotune_host(op, dtype, F.EXACT, w.degree, q, tabs, uh, yh, gh, w.ncells)
        for mode in (0, 2, 1):  # auto (tuned choice), zero-copy, staging pipeline
            F.set_host_path(mode)
            for _ in range(args.warmup):
                estep()
            barrier()
            l0 = F.operator_launches()
            t0 = time.perf_counter()
            marks = [t0]
            for _ in range(args.steps):
                estep()  # synchronous: returns when y is written on the host
                marks.append(time.perf_counter())
            barrier()
            el = maxreduce(time.perf_counter() - t0)
            if mode == 0:
                launches_timed[0] += F.operator_launches() - l0
            # per-call rates: the spread of the host-link rate between calls
            per = sorted(w.ndofs / (b - a) / 1e9 for a, b in zip(marks, marks[1:]))
            e2e[(dtype, mode)] = dict(gdofs=world * args.steps * w.ndofs / el / 1e9,
                                      h2d=uh.numel() * uh.element_size() + gh.numel() * gh.element_size(),
                                      d2h=yh.numel() * yh.element_size(),
                                      per_call=[per[0], per[len(per) // 2], per[-1]])
        F.set_host_path(0)

    r = results[head]
    value = world * args.steps * w.ndofs / (r["total_ms"] * 1e-3) / 1e9
    fpc = flops_per_cell(base, n, q)
    # the FP64 pipe's roof counts the operations the kernel runs: the even-odd
    # kernels execute fewer than the reference's flop convention
    head_eo = head == F.F64 and F.even_odd_used(op, F.F64, F.EXACT, w.degree, q, tabs)
    fpc_head = flops_per_cell_even_odd(base, n, q) if head_eo else fpc
    bpc = bytes_per_cell(base, n, q, 8 if head == F.F64 else 4, w.affine)
    ach_tf = fpc_head * w.ncells / (r["kern_ms"] * 1e-3) / 1e12
    # FP64 pipe: instructions issued per second against its peak (half the
    # FMA flop rate: one FMA = two flops = one instruction)
    pipe_frac = (pipe_instr_per_cell(base, n, q, head_eo, w.affine) * w.ncells / (r["kern_ms"] * 1e-3)
                 / (FP64_PEAK_TFLOPS * 1e12 / 2)) if head == F.F64 else None
    ach_gbs = bpc * w.ncells / (r["kern_ms"] * 1e-3) / 1e9
    hbm, hbm_src = peaks()
    variants = {}
    for key, res in results.items():
        dtype = F.F64 if key == F64PLAIN else key
        es = 8 if dtype in F.FP64_STORAGE else 4
        variants[dname[key]] = {
            "gdofs": world * args.steps * w.ndofs / (res["total_ms"] * 1e-3) / 1e9,
            "kernel_ms": res["kern_ms"],
            "hbm_gbs": bytes_per_cell(base, n, q, es, w.affine) * w.ncells / (res["kern_ms"] * 1e-3) / 1e9,
            "tflops_reference_convention": fpc * w.ncells / (res["kern_ms"] * 1e-3) / 1e12,
            "max_rel_err_vs_fp64_oracle": res["err"],
            "tile": {"cells": res["tile"][0], "geo_staged": res["tile"][1], "threads": res["tile"][2],
                     "lanes_per_slab": res["tile"][3]},
        }
    if "f64plain" in variants:
        base_g = variants["f64plain"]["gdofs"]
        for k, v in variants.items():
            v["vs_f64_plain"] = v["gdofs"] / base_g
    if rank != 0:
        return None
    line = {
        "metric": metric_name(base, w.degree, q),
        "value": value, "unit": "GDoF/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": r["total_ms"] / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": F.DTYPE_NAMES[head], "data": "synthetic",
        "config": workload_config(w, world, 8 if head in F.FP64_STORAGE else 4),
        "roofline": roofline(head, ach_tf, ach_gbs, hbm, hbm_src,
                             traffic_for(w.name, w.ncells, head),
                             flop_count=("even-odd kernel operations per cell "
                                         f"{fpc_head:.0f} (reference convention {fpc:.0f})")
                             if head == F.F64 else None, pipe_frac=pipe_frac),
        "gpu_launches": launches_timed[0],
        "clocks": r["clocks"],
        "variants": variants,
    }
    if (head, 0) in e2e:
        a, z, c = e2e[(head, 0)], e2e[(head, 2)], e2e[(head, 1)]
        h2d_gbs, d2h_gbs = host_link_gbs(dev)
        link_s = max(a["h2d"] / (h2d_gbs * 1e9), a["d2h"] / (d2h_gbs * 1e9))
        line["e2e"] = {"value": a["gdofs"], "unit": "GDoF/s",
                       "h2d_bytes_per_step": a["h2d"], "d2h_bytes_per_step": a["d2h"],
                       "path": "femtc_*_apply_host, pinned host buffers, host-path mode "
                               "auto (tuned: zero-copy or staging pipeline)",
                       "per_call_gdofs_min_median_max": a["per_call"],
                       "zero_copy_gdofs": z["gdofs"], "staging_pipeline_gdofs": c["gdofs"],
                       "host_link_gbs": {"h2d": h2d_gbs, "d2h": d2h_gbs},
                       "host_link_ceiling_gdofs": w.ndofs / link_s / 1e9}
    if cpu_seconds > 0:
        line["cpu_baseline"] = cpu_baseline(w, cpu_seconds)
    return line


def self_launch(args) -> None:
    """--gpus N > 1 outside a launcher: start N local ranks through
    torch.distributed.run (one per GPU, rendezvous on 127.0.0.1) and exit
    with their status."""
    import socket
    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        port = sk.getsockname()[1]
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1",
           f"--nproc-per-node={args.gpus}", "--master-addr", "127.0.0.1",
           "--master-port", str(port), os.path.abspath(__file__), *sys.argv[1:]]
    sys.exit(subprocess.call(cmd))


EXTRA_DEFAULT = "mass_p3,stiffness_p6,batch64,serve"


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="femtc", choices=["femtc", "reference"])
    ap.add_argument("--workload", default="stiffness_p4",
                    choices=["stiffness_p4", "mass_p3", "stiffness_p6", "batch64", "serve"])
    ap.add_argument("--extra", default=None,
                    help="comma list of further workloads measured in the same run and "
                         f"reported under 'extra' (default with the default workload: "
                         f"{EXTRA_DEFAULT}; 'none' for none)")
    ap.add_argument("--requests", type=int, default=48, help="serve: number of requests")
    ap.add_argument("--serve-applications", type=int, default=0,
                    help="serve: operator applications (FP64 mass or stiffness) mixed into "
                         "the request stream, reported under 'applications'")
    ap.add_argument("--serve-policy", default="shortest", choices=["shortest", "fifo"],
                    help="serve: admission order (shortest estimated work first, with aging; "
                         "or arrival order)")
    ap.add_argument("--inner-dtype", default="f32", choices=["f32", "f16x2", "bf16x3"],
                    help="serve: operator form of the inner CG (FP64 refinement outside)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-batch-tune", action="store_true",
                    help="batch64: built-in tile layouts (no autotuning launches; profiling)")
    ap.add_argument("--cells", type=int, default=None, help="override the cell count (profiling)")
    ap.add_argument("--assembled", action="store_true",
                    help="the workload's cells as a box mesh with shared DOFs, through the "
                         "assembled (global-DOF) entry point, F64 and F32")
    ap.add_argument("--geometry", default="per-point", choices=["per-point", "affine"],
                    help="affine: the same degree and cell count on affine cells through the "
                         "affine operator forms (one geometry set per cell), F64 and F32")
    ap.add_argument("--dtypes", default="f64,f32,f16x2,bf16x3,f64e,f64plain",
                    help="comma list of forms to time; the first is the headline")
    ap.add_argument("--tile-db", default=None,
                    help="tile configuration file: loaded if it exists (no tuning), "
                         "else written after autotuning")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        self_launch(args)
    rank, world, local = dist_env()

    if args.impl == "reference":
        run_reference(args, rank, world)
        return

    import torch
    import femtc_gb300 as F

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    pg = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=dev)
        pg = dist
    F.load()

    def finish(line):
        if line is not None:
            print(json.dumps(line), flush=True)
        if pg is not None:
            pg.destroy_process_group()

    if args.workload in ("batch64", "serve"):
        finish((run_batch if args.workload == "batch64" else run_serve)(args, rank, world, dev, pg))
        return
    if args.assembled:
        run_assembled(args, rank, world, dev, pg)
        finish(None)
        return

    line = run_operator(args, args.workload, args.dtypes, rank, world, dev, pg, local,
                        e2e_on=not args.no_e2e,
                        cpu_seconds=0.0 if args.no_cpu_baseline else 10.0, ncells=args.cells)
    extra = args.extra
    if extra is None:
        extra = (EXTRA_DEFAULT if args.workload == "stiffness_p4" and args.cells is None
                 and args.geometry == "per-point" else "none")
    extras = {}
    for name in [e for e in extra.split(",") if e and e != "none"]:
        t0 = time.perf_counter()
        if name in ("batch64", "serve"):
            x = (run_batch if name == "batch64" else run_serve)(args, rank, world, dev, pg)
        else:
            x = run_operator(args, name, "f64,f32,f16x2,bf16x3,f64e,f64plain", rank, world, dev,
                             pg, local, e2e_on=(name == "mass_p3" and not args.no_e2e),
                             cpu_seconds=0.0 if args.no_cpu_baseline else 3.0, clocks=False)
        if x is not None:
            x["wall_s"] = time.perf_counter() - t0
            extras[name] = x
    if line is not None and extras:
        line["extra"] = extras
    finish(line)


if __name__ == "__main__":
    main()
