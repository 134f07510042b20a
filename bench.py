#!/usr/bin/env python3
"""Benchmark of the melt_IBM RK3 step on GB300 (one JSON line on stdout).

A "step" is one iteration of the reference time loop (gcurv.f90:151-172):
cfl -> get_dt -> tschem (3 RK3 substeps: explicit terms, factored implicit
line solves, MLS immersed-boundary forcing with melting, FFT pressure
projection).  Metric: Mcell-steps/s = N^3 * steps / seconds.

value      device time of K steps with every field resident in HBM (CUDA events
           on the library's stream, synchronised on both sides), plain FP64 form.
fp32_refined
           the same K steps in the precision form (FP32 explicit terms, line
           solves and FFTs on FP64 fields, projection refined on the FP64
           divergence residual) from identical inputs; per-field relative L2
           error against the FP64 run after the same number of steps.
e2e        the same K steps driven the way a Fortran host drives the C-ABI:
           every step copies u, v, w, T, p and the vertex coordinates from host
           arrays to the device (mibm_sync_from_host_), runs cfl_/get_dt_/tschem_
           and copies the five fields and the vertices back (mibm_sync_to_host_);
           wall-clock time, after W warm-up iterations of the same calls.
roofline   the dominant kernel's algorithmic bytes per launch / its average
           launch time, both measured live in the timed region (per-kernel CUDA
           events on the launching stream, second timed pass), against the
           measured HBM copy bandwidth.
cpu_baseline / --impl reference
           the CPU oracle (C++ restatement of the reference's algorithm, OpenMP,
           all host threads) on the same workload: the reference itself (Fortran +
           MPI + FFTW + HDF5) cannot be built on this machine or the GPU machine.

Inputs are larger than L2 (each field is N^3 doubles; > 30 fields resident).
Multi-GPU: independent replicas, one per rank (a case runs on one GPU);
value = all ranks' cell-steps / max time over ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

from melt_ibm_gb300 import abi  # noqa: E402
from melt_ibm_gb300.case import Case, CaseConfig  # noqa: E402
from melt_ibm_gb300.workloads import WORKLOAD_TEXT, WORKLOADS  # noqa: E402

# Algorithmic bytes per launch of the kernels that can be dominant (FP64,
# compulsory field reads + writes of that kernel, in passes of N^3 doubles).
ALGO_PASSES = {
    "fused_rhs": 7.0,      # x/y/z/T average: reads u,v,w(,T),p,ru ; writes rhs, ru
    # one launch for u, v, w (3 fields), one for T: mean of 3x and 1x the field passes
    "solve_x": 4.0, "solve_y": 4.0, "solve_z": 8.0,
    "fft_x_fwd": 1.0 + 1.125, "fft_y": 2.25, "fft_z_solve": 2.25, "fft_x_inv": 1.125 + 1.0,
    "divg": 4.0, "updvp": 7.0, "prcalc": 3.0, "hdnl": 6.0,
}


def step_bytes_per_cell(form: str, forcing: bool, tagging: bool, nproj: int = 2) -> dict:
    """Compulsory bytes per cell-step of the routine-boundary model: every
    C-ABI routine of one RK3 step reads and writes each N^3 field it touches
    once (surface-sized work ignored), at the width the form stores it.

    FP64 form, per substep (passes of 8 B): tagging 4 (moving or melting body
    only); hdnl1/2/3/te 6+6+7+6; invtr1/2/3 with solxi/j/k 3 x (6+2+2+3);
    invtrte with its solves 5+7; the IBM field part 19 (zeroing for_* 4,
    velforce 12, tempforce 3); divg 4, phcalc 10, updvp 7, prcalc 3.  Per step
    3 substeps + cfl 3 + forcing 3 passes: 375 passes = 3000 B with forcing
    and tagging.

    Precision form: the explicit terms read the FP32 mirrors of u, v, w, T, p
    (4 B) and the FP64 VOF and forcing fields (8 B) and produce FP32 terms;
    the RHS, RK histories and line-solve right-hand sides are FP32; the z
    solve adds into the FP64 field (read + write 16 B) and writes the T
    mirror; the IBM field part is FP64 as above (+ the T mirror); every
    projection pass forms the FP64 divergence residual (u, v, w 24 B, FP32
    residual 4 B), solves in FP32 (10 FP32 passes), and updates the FP64
    velocity (phi 4 B + read/write u, v, w 48 B) and pressure (4 + 16 B); the
    last pass also writes the u, v, w, p mirrors (16 B)."""
    if form == "f64":
        tag = 4 if tagging else 0
        sub = tag + (6 + 6 + 7 + 6) + 3 * (6 + 2 + 2 + 3) + (5 + 7) + 19 + (4 + 10 + 7 + 3)
        passes = 3 * sub + 3 + (3 if forcing else 0)
        return {"bytes": 8.0 * passes, "passes": passes}
    tag = 32 if tagging else 0
    hdnl = (12 + 8 + 8 + 4) * 2 + (16 + 8 + 8 + 4) + (16 + 8 + 4)
    invtr = 3 * 6 * 4 + 5 * 4
    solves = 4 * (8 + 8 + (4 + 16)) + 4
    ibm = 19 * 8 + 4
    proj = nproj * ((24 + 4) + 10 * 4 + (4 + 48) + (4 + 16)) + 16
    sub = tag + hdnl + invtr + solves + ibm + proj
    total = 3 * sub + 24 + (24 if forcing else 0)
    return {"bytes": float(total), "passes": total / 8.0}


# DRAM bytes per launch of the kernel that dominates the FP64 step, measured
# with ncu (dram__bytes_read.sum + dram__bytes_write.sum, one pass, over the
# launches of one timed step: the mean of its u, v, w, T launches), per
# workload; a workload without its own figure scales the nearest one by the
# cell count (the traffic is per-cell).
NCU_TRAFFIC = {
    "melt256_c2": {"fused_rhs": {"bytes_per_launch": 1.2905e9, "measured_at": "256^3 (melt256_c2)"}},
    "melt128_c1": {"fused_rhs": {"bytes_per_launch": 139.6e6, "measured_at": "128^3 (melt128_c1)"}},
}

# FP64 warp instructions of one step (ncu sm__inst_executed_pipe_fp64.sum
# summed over every kernel launch of one timed step of the workload).  The
# FP64 form is bounded by the FP64 issue rate (one warp instruction per 16
# clocks per SM on this part): this count over that rate is the step's FP64
# floor.
FP64_CENSUS = {"melt256_c2": {"warp_instructions_per_step": 404.58e6, "clocks_per_instruction_per_sm": 16},
               "melt128_c1": {"warp_instructions_per_step": 51.88e6, "clocks_per_instruction_per_sm": 16}}

FIELDS = {"u": abi.MIBM_F_VX, "v": abi.MIBM_F_VY, "w": abi.MIBM_F_VZ, "T": abi.MIBM_F_TEMP, "p": abi.MIBM_F_PR}
FIELD_MASK = sum(1 << f for f in FIELDS.values())
MESH_MASK = 1 << (32 + abi.MIBM_M_XYZV)


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def measured_peaks() -> dict:
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        d = json.load(open(path))
        return {"hbm_gbs": float(d["hbm_gbs"]), "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def __enter__(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self) -> dict:
        if not self.path or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


class Nvtx:
    """An NVTX range around a timed region (`bench_f64`, `bench_f32`), so that
    an ncu capture can select exactly the timed steps with --nvtx
    --nvtx-include "bench_f64/".  No-op without torch."""

    def __init__(self, name: str):
        self.name = name
        try:
            import torch
            self.nvtx = torch.cuda.nvtx
        except Exception:  # noqa: BLE001
            self.nvtx = None

    def __enter__(self):
        if self.nvtx is not None:
            self.nvtx.range_push(self.name)
        return self

    def __exit__(self, *exc):
        if self.nvtx is not None:
            self.nvtx.range_pop()


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class Dist:
    """Barrier / max-reduce over ranks (gloo over the loopback; replicas only)."""

    def __init__(self):
        self.ws, self.rank, self.local = dist_env()
        self.pg = None
        if self.ws > 1:
            import torch.distributed as td
            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            td.init_process_group("gloo")
            self.td = td

    def barrier(self):
        if self.ws > 1:
            self.td.barrier()

    def max(self, v: float) -> float:
        if self.ws == 1:
            return v
        import torch
        t = torch.tensor([v], dtype=torch.float64)
        self.td.all_reduce(t, op=self.td.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.ws > 1:
            self.td.destroy_process_group()


def cpu_baseline(workload: str, steps: int, threads: int | None = None) -> dict:
    """Time the CPU oracle on a bounded sample of the same workload."""
    import oracle
    if threads:
        os.environ["OMP_NUM_THREADS"] = str(threads)
    lib = abi.Lib(oracle.build())
    case = Case(CaseConfig(**WORKLOADS[workload]))
    case.attach(lib)
    case.step(lib, 1)                       # warm-up step (also the reference's ntime = 1)
    t0 = time.perf_counter()
    for nt in range(2, 2 + steps):
        case.step(lib, nt)
    dt = time.perf_counter() - t0
    n3 = case.n1m * case.n2m * case.n3m
    nthreads = int(lib.dll.oracle_num_threads())
    case.detach(lib)
    return {"value": n3 * steps / dt / 1e6, "unit": "Mcell-steps/s", "cores": nthreads, "kind": "port",
            "sample": f"{steps} RK3 steps of {workload} after 1 warm-up step, {dt:.1f} s, "
                      f"CPU oracle (C++ restatement, not the reference binary), {nthreads} OpenMP threads"}


def workload_config(workload: str, n_gpus: int) -> dict:
    """The `config` object of the JSON line: identical in both arms."""
    w = WORKLOADS[workload]
    n = w["n"]
    return {"workload": workload, "description": WORKLOAD_TEXT[workload], "grid": [n, n, n],
            "triangles": 20 * 4 ** w["mesh_level"],
            "parallelism": f"replicas x{n_gpus}" if n_gpus > 1 else "single GPU",
            "l2": "inputs larger than L2 (>30 fields of N^3 doubles resident)"}


def step_model(workload: str, form: str, nproj: int = 2) -> dict:
    w = WORKLOADS[workload]
    moving = w.get("imlsstr", 0) == 1 or w.get("imelt", 1) == 1
    return step_bytes_per_cell(form, bool(w.get("forcing", 0)), moving, nproj)


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    steps = args.steps
    base = cpu_baseline(args.workload, steps)
    line = {"metric": "Mcell-steps/s", "value": base["value"], "unit": "Mcell-steps/s", "n_gpus": args.gpus,
            "steps": steps, "warmup": args.warmup, "ms_per_step": None, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "impl": "reference",
            "config": workload_config(args.workload, args.gpus),
            "cpu_baseline": {"value": base["value"], "unit": base["unit"], "cores": base["cores"],
                             "kind": base["kind"], "sample": base["sample"]},
            "e2e": {"value": base["value"], "unit": "Mcell-steps/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    n3 = WORKLOADS[args.workload]["n"] ** 3
    line["ms_per_step"] = 1e3 * n3 / (base["value"] * 1e6)
    print(json.dumps(line), flush=True)


def autotune_shapes(lib, case, args):
    """The library's autotuner on the bound case before its timed steps (as a
    host does once per grid and form): line-solve chunk lengths and the
    explicit-term block height; returns the chosen shapes."""
    if args.no_autotune:
        return None
    case.bind(lib)
    if lib.mibm_autotune_() != 0:
        lib.check("autotune")
    got = np.zeros(4, dtype=np.int32)
    lib.mibm_autotune_get_(got.ctypes.data)
    return {"chunk_x": int(got[0]), "chunk_y": int(got[1]), "chunk_z": int(got[2]), "rhs_block_y": int(got[3])}


def run_gpu(args):
    from melt_ibm_gb300 import build as mbuild
    dist = Dist()
    lib = abi.Lib(mbuild.build())
    ndev = lib.mibm_device_count_()
    if ndev < 1:
        raise SystemExit("bench: no CUDA device visible (libmibm.so needs a GPU)")
    dev = dist.local % ndev
    lib.mibm_select_device_(abi.ref_int(dev))
    cfg = CaseConfig(**WORKLOADS[args.workload])
    case = Case(cfg)
    case32 = case.clone()                  # identical inputs for the precision form
    case.attach(lib)
    lib.check("attach")
    shapes64 = autotune_shapes(lib, case, args)
    n3 = case.n1m * case.n2m * case.n3m
    nt = 1
    for _ in range(args.warmup):
        case.step(lib, nt)
        nt += 1
    case.sync_to_host(lib, 0)               # drains the stream
    # ---------------- timed region: device-resident ----------------
    dist.barrier()
    l0 = lib.mibm_launch_count_()
    with ClockSampler(dev) as clk, Nvtx("bench_f64"):
        lib.mibm_timer_mark_(abi.ref_int(0))
        t0 = time.perf_counter()
        for _ in range(args.steps):
            case.step(lib, nt)
            nt += 1
        lib.mibm_timer_mark_(abi.ref_int(1))
        ms = lib.mibm_timer_ms_(abi.ref_int(0), abi.ref_int(1))
        wall = time.perf_counter() - t0
    launches = int(lib.mibm_launch_count_() - l0)
    lib.check("timed steps")
    div64 = lib.mibm_divergence_max_()
    diag = np.zeros(abi.MIBM_NDIAG)
    diagnostics = None
    if lib.mibm_diagnostics_(diag.ctypes.data) == 0:
        diagnostics = {"re_lambda": float(diag[abi.MIBM_D_RE_LAMBDA]), "dissipation": float(diag[abi.MIBM_D_DISS]),
                       "kinetic_energy": float(diag[abi.MIBM_D_KENERG]), "eta": float(diag[abi.MIBM_D_ETA]),
                       "after_steps": nt - 1}
    case.sync_to_host(lib, FIELD_MASK)
    snap64 = {k: case.interior(f).copy() for k, f in FIELDS.items()}
    dist.barrier()
    ms_max = dist.max(ms)
    value = dist.ws * n3 * args.steps / (ms_max * 1e-3) / 1e6
    clocks = clk.summary()
    # ---------------- per-kernel pass (roofline of the dominant kernel) ----------------
    lib.mibm_profile_(abi.ref_int(1))
    for _ in range(args.steps):
        case.step(lib, nt)
        nt += 1
    lib.mibm_profile_(abi.ref_int(0))
    prof = lib.profile()
    total = sum(v[0] for v in prof.values()) or 1.0
    dominant = max(prof.items(), key=lambda kv: kv[1][0])
    dname, (dms, dcnt) = dominant
    avg_ms = dms / max(1, dcnt)
    passes = ALGO_PASSES.get(dname)
    peaks = measured_peaks()
    roofline = None
    if passes is not None:
        algo_bytes = passes * 8.0 * n3
        achieved = algo_bytes / (avg_ms * 1e-3) / 1e9
        tr = NCU_TRAFFIC.get(args.workload, {}).get(dname)
        traffic = tr["bytes_per_launch"] if tr else None
        if tr is None:                       # scale the nearest measurement by the cell count
            for wl, kk in NCU_TRAFFIC.items():
                if dname in kk:
                    tr = kk[dname]
                    traffic = tr["bytes_per_launch"] * n3 / WORKLOADS[wl]["n"] ** 3
                    break
        roofline = {"bound": "hbm", "kernel": dname, "achieved": achieved, "peak": peaks["hbm_gbs"],
                    "unit": "GB/s", "frac": achieved / peaks["hbm_gbs"], "traffic": traffic,
                    "traffic_source": (f"ncu dram bytes per launch measured at {tr['measured_at']}"
                                       + ("" if args.workload in tr["measured_at"] else ", scaled by cells"))
                    if tr else None,
                    "algo_bytes_per_launch": algo_bytes, "avg_launch_ms": avg_ms,
                    "peak_source": f"{peaks['source']} (MEASURED_PEAKS.json hbm_gbs)",
                    "note": "FP64 stencils are bounded by the FP64 issue rate (about 1.2 TFLOP/s of FP64 FMA "
                            "measured on this part), not HBM"}
    model = step_model(args.workload, "f64")
    step_ms = ms_max / args.steps
    step_gbs = model["bytes"] * n3 * dist.ws / (step_ms * 1e-3) / 1e9
    step_roofline = {"bound": "hbm", "achieved": step_gbs, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                     "frac": step_gbs / peaks["hbm_gbs"], "bytes_per_cell_step": model["bytes"],
                     "model": "routine-boundary compulsory bytes of one RK3 step (FP64: 375 passes of N^3 "
                              "doubles with forcing and tagging)",
                     "peak_source": f"{peaks['source']} (MEASURED_PEAKS.json hbm_gbs)"}
    kernels = {k: {"ms_per_step": v[0] / args.steps, "launches_per_step": v[1] / args.steps,
                   "share": v[0] / total} for k, v in sorted(prof.items(), key=lambda kv: -kv[1][0])}
    # ---------------- e2e: host buffers, copies inside the timed region ----------------
    h2d = 0
    d2h = 0
    for fid in (abi.MIBM_F_VX, abi.MIBM_F_VY, abi.MIBM_F_VZ, abi.MIBM_F_TEMP, abi.MIBM_F_PR):
        a = case.fields[fid]
        h2d += a.nbytes                                  # whole Fortran array (mibm_sync_from_host_)
        wx = case.n1m + 1 if fid == abi.MIBM_F_VX else case.n1m     # owned cells (+ padding read by cfl)
        hy = case.n2m + 1 if fid == abi.MIBM_F_VY else case.n2m
        d2h += 8 * wx * hy * a.shape[2]
    h2d += case.mesh_arrays[abi.MIBM_M_XYZV].nbytes
    d2h += case.mesh_arrays[abi.MIBM_M_XYZV].nbytes
    case.sync_to_host(lib, FIELD_MASK | MESH_MASK)
    pinned = lib.mibm_pin_host_(abi.ref_int(1)) == 0      # page-locked host arrays: DMA copies
    # warm-up through the same calls: the per-kernel pass above ran without
    # step graphs, so the first steps after it capture them again
    for _ in range(args.warmup):
        case.sync_from_host(lib, FIELD_MASK | MESH_MASK)
        case.step(lib, nt)
        nt += 1
        case.sync_to_host(lib, FIELD_MASK | MESH_MASK)
    dist.barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        case.sync_from_host(lib, FIELD_MASK | MESH_MASK)
        case.step(lib, nt)
        nt += 1
        case.sync_to_host(lib, FIELD_MASK | MESH_MASK)
    e2e_s = dist.max(time.perf_counter() - t0)
    e2e_value = dist.ws * n3 * args.steps / e2e_s / 1e6
    lib.check("e2e")
    case.detach(lib)
    # ---------------- precision form: FP32 compute, FP64 fields, refined projection ----------------
    fp32 = None
    if not args.no_fp32:
        case32.attach(lib)
        case32.bind(lib)
        lib.mibm_set_precision_(abi.ref_int(1), abi.ref_int(args.nproj))
        lib.check("set_precision")
        shapes32 = autotune_shapes(lib, case32, args)
        nt32 = 1
        for _ in range(args.warmup):
            case32.step(lib, nt32)
            nt32 += 1
        case32.sync_to_host(lib, 0)
        dist.barrier()
        with Nvtx("bench_f32"):
            lib.mibm_timer_mark_(abi.ref_int(2))
            for _ in range(args.steps):
                case32.step(lib, nt32)
                nt32 += 1
            lib.mibm_timer_mark_(abi.ref_int(3))
        ms32 = dist.max(lib.mibm_timer_ms_(abi.ref_int(2), abi.ref_int(3)))
        lib.check("precision form")
        div32 = lib.mibm_divergence_max_()
        case32.sync_to_host(lib, FIELD_MASK)
        errs = {}
        for k, f in FIELDS.items():
            a, b = case32.interior(f), snap64[k]
            errs[k] = float(np.sqrt(np.sum((a - b) ** 2)) / np.sqrt(np.sum(b * b)))
        lib.mibm_profile_(abi.ref_int(1))
        for _ in range(args.steps):
            case32.step(lib, nt32)
            nt32 += 1
        lib.mibm_profile_(abi.ref_int(0))
        prof32 = lib.profile()
        tot32 = sum(v[0] for v in prof32.values()) or 1.0
        kern32 = {k: {"ms_per_step": v[0] / args.steps, "launches_per_step": v[1] / args.steps, "share": v[0] / tot32}
                  for k, v in sorted(prof32.items(), key=lambda kv: -kv[1][0])}
        case32.detach(lib)
        v32 = dist.ws * n3 * args.steps / (ms32 * 1e-3) / 1e6
        model32 = step_model(args.workload, "f32", args.nproj)
        gbs32 = model32["bytes"] * n3 * dist.ws / (ms32 / args.steps * 1e-3) / 1e9
        pk = measured_peaks()
        roof32 = {"bound": "hbm", "achieved": gbs32, "peak": pk["hbm_gbs"], "unit": "GB/s",
                  "frac": gbs32 / pk["hbm_gbs"], "bytes_per_cell_step": model32["bytes"],
                  "model": "routine-boundary compulsory bytes of one RK3 step at the precision form's field "
                           "widths (FP32 mirrors, terms, RHS and Poisson solves; FP64 u, v, w, T, p, VOF, "
                           f"forcing and IBM fields; {args.nproj} projection passes per substep)",
                  "peak_source": f"{pk['source']} (MEASURED_PEAKS.json hbm_gbs)"}
        fp32 = {"value": v32, "unit": "Mcell-steps/s", "ms_per_step": ms32 / args.steps, "roofline": roof32,
                "speedup_vs_fp64": v32 / value, "nproj": args.nproj,
                "rel_l2_vs_fp64": errs, "divergence_max": div32, "divergence_max_fp64": div64,
                "compared_after_steps": args.warmup + args.steps, "kernels": kern32, "autotuned_shapes": shapes32,
                "dtype": "f32 compute, f64 fields (u, v, w, T, p), f64 MLS / Stefan / divergence residual"}
    dist.barrier()
    if dist.rank != 0:
        dist.close()
        return
    line = {"metric": "Mcell-steps/s", "value": value, "unit": "Mcell-steps/s", "n_gpus": dist.ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_max / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded random-phase velocity, tanh temperature, generated icosphere)",
            "config": workload_config(args.workload, dist.ws), "step_roofline": step_roofline,
            "e2e": {"value": e2e_value, "unit": "Mcell-steps/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h, "host_arrays_pinned": pinned},
            "roofline": roofline, "gpu_launches": launches, "clocks": clocks, "fp32_refined": fp32,
            "diagnostics": diagnostics,
            "host_wall_ms_per_step": 1e3 * wall / args.steps, "kernels": kernels, "autotuned_shapes": shapes64}
    census = FP64_CENSUS.get(args.workload)
    if census is not None and clocks and clocks.get("sm_mhz"):
        import torch
        sms = torch.cuda.get_device_properties(dev).multi_processor_count
        floor_ms = (census["warp_instructions_per_step"] * census["clocks_per_instruction_per_sm"]
                    / (sms * clocks["sm_mhz"] * 1e6) * 1e3)
        line["fp64_issue"] = {"bound": "fp64", "step_floor_ms": floor_ms, "step_ms": ms_max / args.steps,
                              "frac": floor_ms / (ms_max / args.steps),
                              "warp_instructions_per_step": census["warp_instructions_per_step"],
                              "source": "ncu sm__inst_executed_pipe_fp64.sum summed over the launches of one "
                                        "step of this workload, at the sampled SM clock"}
    if dist.ws == 1 and args.extra_workload and args.extra_workload != args.workload:
        line["extra_workload"] = extra_workload_measurement(lib, args.extra_workload, args.steps, args.warmup,
                                                            args.nproj)
    if dist.ws == 1 and args.remesh_steps > 0:
        line["config1_remesh"] = remesh_measurement(lib, args.remesh_steps)
    if dist.ws == 1 and args.relambda_steps > 0:
        line["config1_re_lambda"] = relambda_measurement(lib, args.relambda_steps)
    if dist.ws == 1 and not args.no_batch:
        line["batched"] = batched_measurement(lib, args.batch_steps, args.warmup)
    if dist.ws == 1 and not args.no_serve:
        line["serving"] = serving_measurement(lib, args.serve_seconds, args.serve_steps, args.serve_budget_gb)
    if dist.ws == 1 and not args.no_cpu:
        try:
            line["cpu_baseline"] = cpu_baseline(args.workload, args.cpu_steps)
        except Exception as e:  # noqa: BLE001
            line["cpu_baseline"] = {"value": None, "error": str(e)}
    print(json.dumps(line), flush=True)
    dist.close()


def extra_workload_measurement(lib, workload: str, steps: int, warmup: int, nproj: int) -> dict:
    """Device-resident K steps of a second workload in both forms (CUDA
    events on the library's stream, as for the headline), same inputs."""
    case = Case(CaseConfig(**WORKLOADS[workload]))
    n3 = case.n1m * case.n2m * case.n3m
    out = {"workload": workload, "description": WORKLOAD_TEXT[workload], "steps": steps, "warmup": warmup}
    for form in ("f64", "f32"):
        c = case.clone()
        c.attach(lib)
        c.bind(lib)
        if form == "f32":
            lib.mibm_set_precision_(abi.ref_int(1), abi.ref_int(nproj))
        lib.check("extra workload")
        nt = 1
        for _ in range(warmup):
            c.step(lib, nt)
            nt += 1
        c.sync_to_host(lib, 0)
        lib.mibm_timer_mark_(abi.ref_int(4))
        for _ in range(steps):
            c.step(lib, nt)
            nt += 1
        lib.mibm_timer_mark_(abi.ref_int(5))
        ms = lib.mibm_timer_ms_(abi.ref_int(4), abi.ref_int(5))
        lib.check("extra workload steps")
        model = step_model(workload, form, nproj)
        pk = measured_peaks()
        gbs = model["bytes"] * n3 / (ms / steps * 1e-3) / 1e9
        out[form] = {"value": n3 * steps / (ms * 1e-3) / 1e6, "unit": "Mcell-steps/s", "ms_per_step": ms / steps,
                     "step_roofline_frac": gbs / pk["hbm_gbs"], "divergence_max": lib.mibm_divergence_max_()}
        c.detach(lib)
    out["speedup_f32_vs_f64"] = out["f32"]["value"] / out["f64"]["value"]
    return out


def remesh_measurement(lib, steps: int) -> dict:
    """The 128^3 free-body configuration with remeshing on (melt128_c1_remesh),
    `steps` steps timed with CUDA events (a step that may remesh runs without
    a step graph and reads the trigger once per substep).  A run that
    reaches the reference's exit condition (the body melted below 27 cell
    volumes) or a remesher abort stops there and says so."""
    workload = "melt128_c1_remesh"
    case = Case(CaseConfig(**WORKLOADS[workload]))
    n3 = case.n1m * case.n2m * case.n3m
    case.attach(lib)
    case.use_library_remesher(lib)
    lib.check("remesher")
    v0 = case.S(abi.MIBM_S_VOLUME)
    nt = 1
    lib.mibm_timer_mark_(abi.ref_int(6))
    stopped = None
    try:
        for _ in range(steps):
            case.step(lib, nt)
            nt += 1
    except RuntimeError as e:
        stopped = f"after {nt - 1} steps: {e}"
    lib.mibm_timer_mark_(abi.ref_int(7))
    ms = lib.mibm_timer_ms_(abi.ref_int(6), abi.ref_int(7))
    done = nt - 1
    out = {"workload": workload, "description": WORKLOAD_TEXT[workload], "steps": done,
           "value": n3 * done / (ms * 1e-3) / 1e6 if done else 0.0, "unit": "Mcell-steps/s",
           "ms_per_step": ms / max(1, done), "remesh_events": int(lib.mibm_remesh_count_()),
           "volume_over_initial": case.S(abi.MIBM_S_VOLUME) / v0, "stopped": stopped}
    stats = np.zeros(8)
    lib.mibm_remesh_stats_(stats.ctypes.data)
    out["last_remesh"] = {"edge_collapses": stats[0], "vertex_deletions": stats[1], "edge_relaxations": stats[2],
                          "volume_residual": stats[5] - stats[3], "largest_drift": stats[6]}
    case.detach(lib)
    return out


def relambda_measurement(lib, steps: int, every: int = 250) -> dict:
    """Where the linear forcing takes Re_lambda: the 128^3 configuration's
    fluid (nu = 0.005, C_HIT of melt128_c1) with the body held solid, `steps`
    steps, Re_lambda every `every` steps and its mean over the second half."""
    w = dict(WORKLOADS["melt128_c1"])
    w.update(imelt=0, imlsstr=0)
    case = Case(CaseConfig(**w))
    case.attach(lib)
    diag = np.zeros(abi.MIBM_NDIAG)
    series = []
    for nt in range(1, steps + 1):
        case.step(lib, nt)
        if nt % every == 0 and lib.mibm_diagnostics_(diag.ctypes.data) == 0:
            series.append({"step": nt, "time": case.S(abi.MIBM_S_TIME),
                           "re_lambda": float(diag[abi.MIBM_D_RE_LAMBDA]),
                           "kinetic_energy": float(diag[abi.MIBM_D_KENERG])})
    case.detach(lib)
    late = [p["re_lambda"] for p in series if p["step"] > steps // 2]
    return {"c_hit": w["c_hit"], "nu": 1.0 / w["ren"], "steps": steps, "series": series,
            "re_lambda_mean_second_half": float(np.mean(late)) if late else None,
            "body": "held solid (imelt = 0, imlsstr = 0)"}


def batched_measurement(lib, steps: int, warmup: int, seed: int = 100) -> dict:
    """Batched form on the batched configuration's mix: 32 cases (12 x 48^3,
    10 x 64^3, 6 x 96^3, 4 x 128^3), radius 0.3-0.6 uniform, icosphere level
    2-4 by the resolution rule of serve.resolved_level, St log-uniform in
    [0.5, 4], nu uniform in [0.005, 0.02], seeds 100-131, precision form,
    shapes autotuned; timed against stepping the
    same cases one after another.  Host wall clock around whole batch steps
    (each ends with a device synchronisation)."""
    from melt_ibm_gb300.batch import BatchRunner
    from melt_ibm_gb300.serve import resolved_level
    rng = np.random.default_rng(seed)
    sizes = [48] * 12 + [64] * 10 + [96] * 6 + [128] * 4
    cfgs = []
    for q, n in enumerate(sizes):
        rad = float(rng.uniform(0.3, 0.6))
        cfgs.append(CaseConfig(n=n, mesh_level=resolved_level(n, rad), rad_p=rad,
                               ren=float(1.0 / rng.uniform(0.005, 0.02)),
                               latheat=float(1.0 / np.exp(rng.uniform(np.log(0.5), np.log(4.0)))), seed=seed + q,
                               v_on_ve=27.0))
    t0 = time.perf_counter()
    proto = [Case(c) for c in cfgs]
    setup_s = time.perf_counter() - t0
    cells = sum(n ** 3 for n in sizes)

    def attached():
        out = []
        for p in proto:
            c = p.clone()
            c.attach(lib)
            c.bind(lib)
            lib.mibm_set_precision_(abi.ref_int(1), abi.ref_int(2))
            lib.check("precision")
            out.append(c)
        return out

    cs = attached()
    with BatchRunner(lib, cs, autotune=True) as b:
        b.run(warmup)
        t0 = time.perf_counter()
        b.run(steps)
        t_batch = time.perf_counter() - t0
    launches = lib.mibm_launch_count_()
    for c in cs:
        c.detach(lib)
    cs = attached()
    for c in cs:
        c.run(lib, warmup)
    t0 = time.perf_counter()
    for s in range(steps):
        for c in cs:
            c.step(lib, warmup + 1 + s)
    t_seq = time.perf_counter() - t0
    for c in cs:
        c.detach(lib)
    shapes = {}
    for n in sorted(set(sizes)):
        c = proto[sizes.index(n)].clone()
        c.attach(lib)
        c.bind(lib)
        lib.mibm_set_precision_(abi.ref_int(1), abi.ref_int(2))
        lib.mibm_autotune_()
        got = np.zeros(4, dtype=np.int32)
        lib.mibm_autotune_get_(got.ctypes.data)
        shapes[f"{n}^3"] = {"chunk_x": int(got[0]), "chunk_y": int(got[1]), "chunk_z": int(got[2]),
                            "rhs_block_y": int(got[3])}
        c.detach(lib)
    return {"value": cells * steps / t_batch / 1e6, "unit": "Mcell-steps/s", "cases": len(sizes),
            "cells": cells, "steps": steps, "warmup": warmup, "ms_per_step": 1e3 * t_batch / steps,
            "sequential_value": cells * steps / t_seq / 1e6, "speedup_vs_sequential": t_seq / t_batch,
            "autotuned_shapes": shapes, "host_setup_s": setup_s, "form": "precision (f32 compute, f64 fields)",
            "config": "32 cases: 12x48^3, 10x64^3, 6x96^3, 4x128^3; r 0.3-0.6, level 2-4 by the mesh-resolution "
                      "rule, St log-U[0.5,4], nu U[0.005,0.02], seeds 100-131",
            "timing": "host wall clock around batch steps (each ends synchronised)"}


def serving_measurement(lib, seconds: float, steps: int, budget_gb: float, seed: int = 7,
                        step_cells: int | None = 8 << 20) -> dict:
    """Serving form: Poisson arrivals at 2 cases/s for `seconds`, grids
    {64, 96, 128, 192}^3 with probabilities {0.4, 0.3, 0.2, 0.1}, the batched
    configuration's parameter laws, `steps` steps per case in the precision
    form, admission against an HBM budget of `budget_gb` GB, a work budget
    of `step_cells` cells per batch step (the cases that waited longest,
    at least one); the run lasts until every request has completed."""
    from melt_ibm_gb300.serve import DeviceExecutor, Server, serving_requests
    reqs = serving_requests(seconds, rate=2.0, seed=seed, steps=steps)
    ex = DeviceExecutor(lib)
    try:
        stats = Server(ex, int(budget_gb * 1e9), prepare_workers=4, step_cells=step_cells).run(reqs)
    finally:
        ex.close()
    out = stats.summary()
    out.update({"requests": len(reqs), "arrival_window_s": seconds, "rate_per_s": 2.0, "steps_per_case": steps,
                "hbm_budget_gb": budget_gb, "step_cells_budget": step_cells, "seed": seed,
                "form": "precision (f32 compute, f64 fields)",
                "unit_cell_steps": "cell-steps/s over the whole run (first arrival to last completion)"})
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["mibm", "reference"], default="mibm")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="melt256_c2")
    ap.add_argument("--extra-workload", choices=sorted(WORKLOADS) + [""], default="melt128_c1",
                    help="a second workload timed in both forms (device-resident), '' for none")
    ap.add_argument("--cpu-steps", type=int, default=3)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-fp32", action="store_true", help="skip the precision-form measurement")
    ap.add_argument("--nproj", type=int, default=2, help="Poisson solves per substep in the precision form")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched-form measurement")
    ap.add_argument("--no-autotune", action="store_true",
                    help="time the headline case at the default shapes instead of the autotuned ones")
    ap.add_argument("--remesh-steps", type=int, default=100,
                    help="steps of the 128^3 free-body configuration with remeshing (0: skip)")
    ap.add_argument("--relambda-steps", type=int, default=3500,
                    help="steps of the Re_lambda series under the linear forcing (0: skip)")
    ap.add_argument("--batch-steps", type=int, default=10)
    ap.add_argument("--no-serve", action="store_true", help="skip the serving measurement")
    ap.add_argument("--serve-seconds", type=float, default=30.0,
                    help="arrival window of the serving run (the serving configuration uses 600; the default "
                         "is shortened so that the bench ends within minutes, and the line says so)")
    ap.add_argument("--serve-steps", type=int, default=300,
                    help="steps per served case (the serving configuration's 300)")
    ap.add_argument("--serve-budget-gb", type=float, default=150.0)
    args = ap.parse_args()
    if args.warmup < 3:
        log("bench: warm-up raised to 3 steps")
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
