"""Serving form: a request loop with continuous batching on one GPU.

Requests (one melting case each: grid, mesh, parameters, number of steps)
arrive over time.  The server

* prepares each arrived request's host state (mesh, seeded initial fields)
  in worker threads, off the device loop;
* admits prepared requests first come, first served while their device
  footprint fits the HBM budget (a request that does not fit blocks those
  behind it, so none is starved), attaching each as its own context whose
  fields and mesh stay resident on the device until the case completes;
* advances the resident cases by one time step per loop iteration through
  one persistent batch (`mibm_batch_step_`), whose members change as cases
  join or leave (`mibm_batch_add_` / `mibm_batch_remove_`); each case's own
  step graph is launched on its own stream, so a membership change rebuilds
  nothing -- new work joins the running mix at the next step, finished
  cases free their memory at once;
* with a work budget per batch step (``step_cells``), advances in each
  iteration the resident cases that have waited longest, as many as fit
  the budget in cells (at least one): the latency of a batch step then
  follows the budget rather than how much work happens to be resident,
  while every case still gets its steps in order and the GPU stays busy;
* records the latency of every batch step (and which steps carried an
  admission: a case's first two steps run its direct launches and its graph
  capture) and the completion time of every case (completion - arrival:
  preparation, queueing and steps).

Faults are handled per case, on the host, without touching the others:

* ``Server.cancel(rid)`` drops a request that has not been admitted, or
  detaches a resident case between two batch steps;
* an admission that runs out of device memory (:class:`DeviceOOM`, raised by
  the library's allocation failure or by an executor's simulated capacity)
  puts the request back at the head of the queue until a resident case has
  completed; with nothing resident it is refused;
* a case that fails inside a batch step (e.g. a non-finite field caught by the
  CFL guard) is left out of that step by the library and detached as failed,
  while the other cases complete the step exactly as they would alone;
* a case whose body has melted below the volume threshold (the reference's
  exit condition, particle.f90:218-224: V < V_ON_VE cell volumes) ends there
  and counts as completed.

The device executor is one implementation of a small interface; the tests
drive the same scheduler with a host-only executor to check the admission
and fault policy without a GPU.
"""
from __future__ import annotations

import concurrent.futures as cf
import threading
import time
from collections import deque
from dataclasses import dataclass, field

import numpy as np

from . import abi
from .case import Case, CaseConfig


@dataclass
class Request:
    rid: int
    arrival: float              # seconds after the server starts
    cfg: CaseConfig
    steps: int
    precision: int = 1          # 1 = FP32 + refined projection, 0 = FP64


@dataclass
class Finished:
    rid: int
    n: int
    arrival: float
    admitted: float
    completed: float
    steps: int
    melted: bool = False        # ended early: the body melted below the volume threshold


class DeviceOOM(MemoryError):
    """An admission ran out of device memory (real or simulated)."""


@dataclass
class ServeStats:
    wall_s: float
    step_ms: list = field(default_factory=list)        # latency of every batch step
    admission: list = field(default_factory=list)      # the step carried an admission (first two steps of a case)
    active: list = field(default_factory=list)         # cases in each batch step
    stepped_cells: list = field(default_factory=list)   # cells advanced by each batch step
    cell_steps: float = 0.0
    finished: list = field(default_factory=list)
    admitted: int = 0
    peak_bytes: int = 0
    cancelled: list = field(default_factory=list)      # rids cancelled (queued or resident)
    failed: dict = field(default_factory=dict)         # rid -> reason (failed inside a step, or refused)
    oom_retries: int = 0                               # admissions put back after running out of memory

    def summary(self) -> dict:
        st = np.array(self.step_ms) if self.step_ms else np.zeros(1)
        adm = np.array(self.admission, dtype=bool) if self.admission else np.zeros(len(st), dtype=bool)
        steady = st[~adm] if (~adm).any() else st
        # latency per Mcell advanced: the step of a mix of grids 64^3..256^3
        # lasts as long as its work, so p99/p50 of the raw latency measures
        # the mix; this ratio measures the jitter at a given load
        cells = np.array(self.stepped_cells, dtype=float) if len(self.stepped_cells) == len(st) else None
        if cells is not None and (cells > 0).all():
            per = st / (cells / 1e6)
            per_steady = per[~adm] if (~adm).any() else per
        else:
            per_steady = np.zeros(1)
        ct = np.array([f.completed - f.arrival for f in self.finished]) if self.finished else np.zeros(1)
        qt = np.array([f.admitted - f.arrival for f in self.finished]) if self.finished else np.zeros(1)
        return {
            "wall_s": self.wall_s,
            "cases_completed": len(self.finished),
            "cases_melted_out": sum(1 for f in self.finished if f.melted),
            "cases_admitted": self.admitted,
            "cases_cancelled": len(self.cancelled),
            "cases_failed": len(self.failed),
            "oom_retries": self.oom_retries,
            "batch_steps": len(self.step_ms),
            "admission_steps": int(adm.sum()),
            "step_latency_ms": {"p50": float(np.percentile(st, 50)), "p99": float(np.percentile(st, 99)),
                                "max": float(st.max())},
            "step_latency_ms_outside_admission": {"p50": float(np.percentile(steady, 50)),
                                                  "p99": float(np.percentile(steady, 99)),
                                                  "max": float(steady.max())},
            "step_latency_us_per_mcell_outside_admission": {
                "p50": float(np.percentile(per_steady, 50)), "p99": float(np.percentile(per_steady, 99))},
            "case_completion_s": {"p50": float(np.percentile(ct, 50)), "p99": float(np.percentile(ct, 99))},
            "admission_wait_s": {"p50": float(np.percentile(qt, 50)), "p99": float(np.percentile(qt, 99))},
            "mean_active_cases": float(np.mean(self.active)) if self.active else 0.0,
            "cell_steps_per_s": self.cell_steps / self.wall_s if self.wall_s > 0 else 0.0,
            "peak_resident_bytes": int(self.peak_bytes),
        }


def resolved_level(n: int, rad_p: float, length: float = 2.0 * np.pi, levels=(2, 3, 4)) -> int:
    """The icosphere level, among `levels`, whose mean edge is closest to 1.5
    grid cells, i.e. triangles about one cell face in area.  That is the
    resolution the MLS forcing needs: its coefficient cfac = sur h / celvol
    (initmls.f90:25) grows with the triangle area, and a mesh much coarser
    than the grid (cfac well above 1) overshoots and diverges within a few
    steps (e.g. a level-2 body of radius 0.44 on a 128^3 grid).  The unit
    icosphere's mean edge is about 1.2 / 2^level."""
    dx = length / n
    return min(levels, key=lambda lv: abs(np.log(1.2 * rad_p / 2 ** lv / dx / 1.5)))


def serving_requests(duration_s: float, rate: float = 2.0, seed: int = 7, steps: int = 300,
                     grids=(64, 96, 128, 192), probs=(0.4, 0.3, 0.2, 0.1)) -> list[Request]:
    """Poisson arrivals with the serving configuration's distributions:
    grid from `grids` with `probs`; radius 0.3-0.6 uniform; St log-uniform in
    [0.5, 4]; nu uniform in [0.005, 0.02]; icosphere level 2-4 by the
    resolution rule of :func:`resolved_level` (uniform levels include meshes
    too coarse for their grid, which diverge); the reference's volume
    threshold of 27 cell volumes (part.in V_ON_VE) ends a case whose body has
    melted away."""
    rng = np.random.default_rng(seed)
    out, t, rid = [], 0.0, 0
    while True:
        t += rng.exponential(1.0 / rate)
        if t > duration_s:
            return out
        n = int(rng.choice(grids, p=probs))
        st = float(np.exp(rng.uniform(np.log(0.5), np.log(4.0))))
        rad = float(rng.uniform(0.3, 0.6))
        cfg = CaseConfig(n=n, mesh_level=resolved_level(n, rad), rad_p=rad,
                         ren=float(1.0 / rng.uniform(0.005, 0.02)), latheat=1.0 / st, seed=1000 + rid,
                         v_on_ve=27.0)
        out.append(Request(rid=rid, arrival=t, cfg=cfg, steps=steps))
        rid += 1


class DeviceExecutor:
    """Resident cases on the GPU, advanced together by one persistent batch.

    ``launch`` = 1 launches each case's step graph on its own stream (no
    batch-graph rebuild when members change), 0 one batch graph.
    ``device_capacity`` (bytes) simulates a device with less memory than the
    server's budget: an admission beyond it raises :class:`DeviceOOM` before
    anything is allocated, as a failed cudaMalloc would after."""

    def __init__(self, lib: abi.Lib, launch: int = 1, device_capacity: int | None = None):
        self.lib = lib
        self.cases: dict[int, Case] = {}
        self.batch = 0
        self.launch = launch
        self.capacity = device_capacity
        self.bytes: dict[int, int] = {}
        self.age: dict[int, int] = {}
        self.members: set[int] = set()          # cases in the batch now
        self.measured: dict[tuple, int] = {}    # device bytes per (n, precision), measured at first admission

    @staticmethod
    def model_bytes(cfg: CaseConfig, precision: int) -> int:
        """Device footprint model: 26 FP64 fields + RHS scratch (4 FP64, or 15
        FP32 fields and the 3 FP64 velocity fields between projection sweeps
        in the precision form) + spectrum + reductions + mesh."""
        n3 = cfg.n * cfg.n * cfg.nz
        per_cell = 26 * 8 + (4 * 8 if precision == 0 else 15 * 4 + 3 * 8) + 8 + 16 + 16
        nf = 20 * 4 ** cfg.mesh_level
        return int(per_cell * n3 + 4000 * nf + (64 << 20))

    def estimate(self, req: Request) -> int:
        return self.measured.get((req.cfg.n, req.precision), self.model_bytes(req.cfg, req.precision))

    def free_bytes(self) -> int | None:
        try:
            import torch
            if torch.cuda.is_available():
                return int(torch.cuda.mem_get_info()[0])
        except Exception:
            pass
        return None

    def _ensure_batch(self) -> None:
        if self.batch:
            return
        self.batch = int(self.lib.mibm_batch_create_(None, abi.ref_int(0)))
        if self.batch <= 0:
            raise RuntimeError(f"batch_create: {self.lib.mibm_last_message().decode()}")
        if self.lib.mibm_batch_set_launch_(abi.ref_int(self.batch), abi.ref_int(self.launch)) != 0:
            raise RuntimeError(f"batch_set_launch: {self.lib.mibm_last_message().decode()}")

    def attach(self, req: Request, case: Case) -> None:
        need = self.estimate(req)
        if self.capacity is not None and sum(self.bytes.values()) + need > self.capacity:
            raise DeviceOOM(f"request {req.rid}: {need} B do not fit the device's {self.capacity} B")
        before = self.free_bytes()
        try:
            case.attach(self.lib)
            case.bind(self.lib)
            self.lib.mibm_set_precision_(abi.ref_int(req.precision), abi.ref_int(2))
            self.lib.check("set_precision")
        except RuntimeError as e:
            status = self.lib.mibm_last_status_()
            case.detach(self.lib)
            if status == abi.MIBM_ENOMEM:
                raise DeviceOOM(str(e)) from e
            raise
        self._ensure_batch()
        if self.lib.mibm_batch_add_(abi.ref_int(self.batch), abi.ref_int(case.ctx[self.lib.path])) != 0:
            case.detach(self.lib)
            raise RuntimeError(f"batch_add: {self.lib.mibm_last_message().decode()}")
        self.members.add(req.rid)
        self.cases[req.rid] = case
        self.bytes[req.rid] = need
        self.age[req.rid] = 0
        after = self.free_bytes()
        key = (req.cfg.n, req.precision)
        if before is not None and after is not None and key not in self.measured:
            # device memory of a context grows during its first step; the
            # model covers that part, the measurement the part seen here
            self.measured[key] = max(before - after, self.model_bytes(req.cfg, req.precision))

    def detach(self, rid: int) -> Case:
        case = self.cases.pop(rid)
        self.bytes.pop(rid, None)
        self.age.pop(rid, None)
        if self.batch and rid in self.members:
            self.lib.mibm_batch_remove_(abi.ref_int(self.batch), abi.ref_int(case.ctx[self.lib.path]))
        self.members.discard(rid)
        case.detach(self.lib)
        return case

    def _members(self, rids) -> None:
        """Make the batch's members exactly `rids` (launch mode 1 rebuilds
        nothing when members change)."""
        want = set(rids)
        for rid in list(self.members - want):
            self.lib.mibm_batch_remove_(abi.ref_int(self.batch), abi.ref_int(self.cases[rid].ctx[self.lib.path]))
            self.members.discard(rid)
        for rid in sorted(want - self.members):
            if self.lib.mibm_batch_add_(abi.ref_int(self.batch), abi.ref_int(self.cases[rid].ctx[self.lib.path])) != 0:
                raise RuntimeError(f"batch_add: {self.lib.mibm_last_message().decode()}")
            self.members.add(rid)

    def step(self, rids=None) -> dict:
        """One batch step of the resident cases `rids` (all when None).
        Returns whether the step carried an admission and the cases that
        failed in it."""
        self._ensure_batch()
        rids = list(self.cases) if rids is None else list(rids)
        self._members(rids)
        admission = any(self.age[r] < 2 for r in rids)
        st = int(self.lib.mibm_batch_step_(abi.ref_int(self.batch), abi.ref_int(0)))
        failed = {}
        if st != 0:
            for rid in rids:
                case = self.cases[rid]
                case.bind(self.lib)
                cst = int(self.lib.mibm_last_status_())
                if cst != 0:
                    failed[rid] = (cst, f"status {cst}: {self.lib.mibm_last_message().decode()}")
            if not failed:
                raise RuntimeError(f"batch_step ({st}): {self.lib.mibm_last_message().decode()}")
        for rid in rids:
            self.age[rid] += 1
        return {"admission": admission, "failed": failed}

    def close(self) -> None:
        for rid in list(self.cases):
            self.detach(rid)
        if self.batch:
            self.lib.mibm_batch_destroy_(abi.ref_int(self.batch))
            self.batch = 0


class Server:
    def __init__(self, executor, budget_bytes: int, prepare_workers: int = 2, keep_results: bool = False,
                 on_finish=None, on_step=None, step_cells: int | None = None):
        self.ex = executor
        self.budget = int(budget_bytes)
        self.step_cells = step_cells        # work budget of a batch step in cells (None: every resident case)
        self.workers = prepare_workers
        self.keep_results = keep_results
        self.on_finish = on_finish          # callback(request, case) before the case is detached
        self.on_step = on_step              # callback(server, batch step index) before each batch step
        self._lock = threading.Lock()
        self._cancel: set[int] = set()

    def cancel(self, rid: int) -> None:
        """Cancel request `rid` (thread-safe): dropped if still queued, detached
        between two batch steps if resident."""
        with self._lock:
            self._cancel.add(rid)

    def set_budget(self, budget_bytes: int) -> None:
        """Change the HBM budget while running (thread-safe).  Resident cases
        keep running; admissions wait until the used bytes fit the new budget."""
        with self._lock:
            self.budget = int(budget_bytes)

    def run(self, requests: list[Request], max_wall_s: float | None = None) -> ServeStats:
        pending = deque(sorted(requests, key=lambda r: r.arrival))
        futures: dict[int, cf.Future] = {}
        active: dict[int, list] = {}         # rid -> [request, steps done, admitted time, bytes, last stepped]
        used = 0
        oom_hold = False                     # an admission ran out of memory: wait for a completion
        stats = ServeStats(wall_s=0.0)
        t0 = time.perf_counter()
        now = lambda: time.perf_counter() - t0
        pool = cf.ThreadPoolExecutor(max_workers=self.workers)
        queued = list(pending)
        qi = 0
        nstep = 0
        dropped: set[int] = set()

        def release(rid):
            nonlocal used, oom_hold
            used -= active[rid][3]
            del active[rid]
            oom_hold = False

        try:
            while pending or active:
                t = now()
                if max_wall_s is not None and t > max_wall_s:
                    break
                with self._lock:
                    cancels, self._cancel = self._cancel, set()
                    budget = self.budget
                for rid in cancels:
                    if rid in active:
                        self.ex.detach(rid)
                        release(rid)
                        stats.cancelled.append(rid)
                    elif any(r.rid == rid for r in pending):
                        pending = deque(r for r in pending if r.rid != rid)
                        dropped.add(rid)
                        fut = futures.pop(rid, None)
                        if fut is not None:
                            fut.cancel()
                        stats.cancelled.append(rid)
                # start preparing every request that has arrived
                while qi < len(queued) and queued[qi].arrival <= t:
                    r = queued[qi]
                    if r.rid not in dropped:
                        futures[r.rid] = pool.submit(Case, r.cfg)
                    qi += 1
                # admit first come, first served while the budget allows
                while pending and pending[0].arrival <= t and not oom_hold:
                    r = pending[0]
                    need = self.ex.estimate(r)
                    if need > budget and not active:
                        # cannot fit even alone under the budget in force: refused
                        pending.popleft()
                        fut = futures.pop(r.rid, None)
                        if fut is not None:
                            fut.cancel()
                        stats.failed[r.rid] = f"needs {need} B, more than the budget of {budget} B"
                        continue
                    if used + need > budget or not futures[r.rid].done():
                        break
                    try:
                        self.ex.attach(r, futures[r.rid].result())
                    except DeviceOOM as e:
                        if not active:             # it cannot fit even alone: refuse it
                            pending.popleft()
                            futures.pop(r.rid)
                            stats.failed[r.rid] = f"out of device memory: {e}"
                            continue
                        stats.oom_retries += 1
                        oom_hold = True            # retry when a resident case has completed
                        break
                    pending.popleft()
                    futures.pop(r.rid)
                    used += need
                    stats.peak_bytes = max(stats.peak_bytes, used)
                    stats.admitted += 1
                    active[r.rid] = [r, 0, now(), need, -1]
                if not active:
                    # idle: wait for the next arrival or preparation
                    time.sleep(0.002)
                    continue
                if self.on_step is not None:
                    self.on_step(self, nstep)
                    if not active:
                        continue
                cells = lambda a: a[0].cfg.n * a[0].cfg.n * a[0].cfg.nz
                if self.step_cells is None:
                    chosen = list(active)
                else:
                    # the cases that have waited longest, as many as fit the budget
                    chosen, total = [], 0
                    for rid in sorted(active, key=lambda r: (active[r][4], r)):
                        if chosen and total + cells(active[rid]) > self.step_cells:
                            continue
                        chosen.append(rid)
                        total += cells(active[rid])
                ts = time.perf_counter()
                info = (self.ex.step(chosen) if self.step_cells is not None else self.ex.step()) or {}
                stats.step_ms.append((time.perf_counter() - ts) * 1e3)
                stats.admission.append(bool(info.get("admission", False)))
                stats.active.append(len(active))
                stats.stepped_cells.append(sum(cells(active[r]) for r in chosen))
                for rid in chosen:
                    active[rid][4] = nstep
                nstep += 1
                failed = info.get("failed", {})
                for rid, why in failed.items():
                    if rid not in active:
                        continue
                    status, msg = why if isinstance(why, tuple) else (None, why)
                    a = active[rid]
                    if status == abi.MIBM_EABORT:
                        # the body melted below the volume threshold: the
                        # reference's run ends there (particle.f90:218-224)
                        a[1] += 1
                        stats.cell_steps += a[0].cfg.n * a[0].cfg.n * a[0].cfg.nz
                        case = self.ex.cases.get(rid) if hasattr(self.ex, "cases") else None
                        if self.on_finish is not None:
                            self.on_finish(a[0], case)
                        stats.finished.append(Finished(rid, a[0].cfg.n, a[0].arrival, a[2], now(), a[1], True))
                    else:
                        stats.failed[rid] = msg
                    self.ex.detach(rid)
                    release(rid)
                for rid in chosen:
                    if rid not in active:
                        continue
                    a = active[rid]
                    a[1] += 1
                    stats.cell_steps += a[0].cfg.n * a[0].cfg.n * a[0].cfg.nz
                    if a[1] >= a[0].steps:
                        case = self.ex.cases.get(rid) if hasattr(self.ex, "cases") else None
                        if self.on_finish is not None:
                            self.on_finish(a[0], case)
                        self.ex.detach(rid)
                        release(rid)
                        stats.finished.append(Finished(rid, a[0].cfg.n, a[0].arrival, a[2], now(), a[1]))
        finally:
            stats.wall_s = now()
            pool.shutdown(wait=False, cancel_futures=True)
        return stats
