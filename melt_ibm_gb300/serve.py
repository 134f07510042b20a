"""Serving form: a request loop with continuous batching on one GPU.

Requests (one melting case each: grid, mesh, parameters, number of steps)
arrive over time.  The server

* prepares each arrived request's host state (mesh, seeded initial fields)
  in worker threads, off the device loop;
* admits prepared requests first come, first served while their device
  footprint fits the HBM budget (a request that does not fit blocks those
  behind it, so none is starved), attaching each as its own context whose
  fields and mesh stay resident on the device until the case completes;
* advances every resident case by one time step per loop iteration through
  the batched form (`mibm_batch_step_`: one batch graph, the device
  interleaves the cases), rebuilding the batch whenever cases join or leave
  -- new work joins the running mix at the next step, finished cases free
  their memory at once;
* records the latency of every batch step and the completion time of every
  case (completion - arrival: preparation, queueing and steps).

The device executor is one implementation of a small interface; the tests
drive the same scheduler with a host-only executor to check the admission
policy without a GPU.
"""
from __future__ import annotations

import concurrent.futures as cf
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


@dataclass
class ServeStats:
    wall_s: float
    step_ms: list = field(default_factory=list)        # latency of every batch step
    active: list = field(default_factory=list)         # cases in each batch step
    cell_steps: float = 0.0
    finished: list = field(default_factory=list)
    admitted: int = 0
    peak_bytes: int = 0

    def summary(self) -> dict:
        st = np.array(self.step_ms) if self.step_ms else np.zeros(1)
        ct = np.array([f.completed - f.arrival for f in self.finished]) if self.finished else np.zeros(1)
        qt = np.array([f.admitted - f.arrival for f in self.finished]) if self.finished else np.zeros(1)
        return {
            "wall_s": self.wall_s,
            "cases_completed": len(self.finished),
            "cases_admitted": self.admitted,
            "batch_steps": len(self.step_ms),
            "step_latency_ms": {"p50": float(np.percentile(st, 50)), "p99": float(np.percentile(st, 99)),
                                "max": float(st.max())},
            "case_completion_s": {"p50": float(np.percentile(ct, 50)), "p99": float(np.percentile(ct, 99))},
            "admission_wait_s": {"p50": float(np.percentile(qt, 50)), "p99": float(np.percentile(qt, 99))},
            "mean_active_cases": float(np.mean(self.active)) if self.active else 0.0,
            "cell_steps_per_s": self.cell_steps / self.wall_s if self.wall_s > 0 else 0.0,
            "peak_resident_bytes": int(self.peak_bytes),
        }


def serving_requests(duration_s: float, rate: float = 2.0, seed: int = 7, steps: int = 300,
                     grids=(64, 96, 128, 192), probs=(0.4, 0.3, 0.2, 0.1)) -> list[Request]:
    """Poisson arrivals with the serving configuration's distributions:
    grid from `grids` with `probs`; icosphere level 2-4 and radius 0.3-0.6
    uniform; St log-uniform in [0.5, 4]; nu uniform in [0.005, 0.02]."""
    rng = np.random.default_rng(seed)
    out, t, rid = [], 0.0, 0
    while True:
        t += rng.exponential(1.0 / rate)
        if t > duration_s:
            return out
        n = int(rng.choice(grids, p=probs))
        st = float(np.exp(rng.uniform(np.log(0.5), np.log(4.0))))
        cfg = CaseConfig(n=n, mesh_level=int(rng.integers(2, 5)), rad_p=float(rng.uniform(0.3, 0.6)),
                         ren=float(1.0 / rng.uniform(0.005, 0.02)), latheat=1.0 / st, seed=1000 + rid,
                         v_on_ve=0.0)
        out.append(Request(rid=rid, arrival=t, cfg=cfg, steps=steps))
        rid += 1


class DeviceExecutor:
    """Resident cases on the GPU, advanced together by the batched form."""

    def __init__(self, lib: abi.Lib):
        self.lib = lib
        self.cases: dict[int, Case] = {}
        self.batch = 0
        self.members: tuple = ()
        self.measured: dict[tuple, int] = {}    # device bytes per (n, precision), measured at first admission

    @staticmethod
    def model_bytes(cfg: CaseConfig, precision: int) -> int:
        """Device footprint model: 26 FP64 fields + RHS scratch (4 FP64 or 15
        FP32 fields in the precision form) + spectrum + reductions + mesh."""
        n3 = cfg.n * cfg.n * cfg.nz
        per_cell = 26 * 8 + (4 * 8 if precision == 0 else 15 * 4) + 8 + 16 + 16
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

    def attach(self, req: Request, case: Case) -> None:
        before = self.free_bytes()
        case.attach(self.lib)
        case.bind(self.lib)
        self.lib.mibm_set_precision_(abi.ref_int(req.precision), abi.ref_int(2))
        self.lib.check("set_precision")
        self.cases[req.rid] = case
        after = self.free_bytes()
        key = (req.cfg.n, req.precision)
        if before is not None and after is not None and key not in self.measured:
            # device memory of a context grows during its first step; the
            # model covers that part, the measurement the part seen here
            self.measured[key] = max(before - after, self.model_bytes(req.cfg, req.precision))

    def detach(self, rid: int) -> Case:
        case = self.cases.pop(rid)
        if self.batch:
            self.lib.mibm_batch_destroy_(abi.ref_int(self.batch))
            self.batch = 0
        case.detach(self.lib)
        return case

    def step(self) -> None:
        rids = tuple(sorted(self.cases))
        if rids != self.members or not self.batch:
            if self.batch:
                self.lib.mibm_batch_destroy_(abi.ref_int(self.batch))
            ids = np.array([self.cases[r].ctx[self.lib.path] for r in rids], dtype=np.int32)
            self.batch = int(self.lib.mibm_batch_create_(ids.ctypes.data, abi.ref_int(len(ids))))
            if self.batch <= 0:
                raise RuntimeError(f"batch_create: {self.lib.mibm_last_message().decode()}")
            self.members = rids
        st = int(self.lib.mibm_batch_step_(abi.ref_int(self.batch), abi.ref_int(0)))
        if st != 0:
            raise RuntimeError(f"batch_step ({st}): {self.lib.mibm_last_message().decode()}")

    def close(self) -> None:
        if self.batch:
            self.lib.mibm_batch_destroy_(abi.ref_int(self.batch))
            self.batch = 0
        for rid in list(self.cases):
            self.cases.pop(rid).detach(self.lib)


class Server:
    def __init__(self, executor, budget_bytes: int, prepare_workers: int = 2, keep_results: bool = False,
                 on_finish=None):
        self.ex = executor
        self.budget = int(budget_bytes)
        self.workers = prepare_workers
        self.keep_results = keep_results
        self.on_finish = on_finish          # callback(request, case) before the case is detached

    def run(self, requests: list[Request], max_wall_s: float | None = None) -> ServeStats:
        pending = deque(sorted(requests, key=lambda r: r.arrival))
        futures: dict[int, cf.Future] = {}
        active: dict[int, tuple] = {}        # rid -> (request, steps done, admitted time, bytes)
        used = 0
        stats = ServeStats(wall_s=0.0)
        t0 = time.perf_counter()
        now = lambda: time.perf_counter() - t0
        pool = cf.ThreadPoolExecutor(max_workers=self.workers)
        queued = list(pending)
        qi = 0
        try:
            while pending or active:
                t = now()
                if max_wall_s is not None and t > max_wall_s:
                    break
                # start preparing every request that has arrived
                while qi < len(queued) and queued[qi].arrival <= t:
                    r = queued[qi]
                    futures[r.rid] = pool.submit(Case, r.cfg)
                    qi += 1
                # admit first come, first served while the budget allows
                while pending and pending[0].arrival <= t:
                    r = pending[0]
                    need = self.ex.estimate(r)
                    if need > self.budget:
                        raise ValueError(f"request {r.rid} needs {need} B, more than the whole budget")
                    if used + need > self.budget or not futures[r.rid].done():
                        break
                    pending.popleft()
                    self.ex.attach(r, futures.pop(r.rid).result())
                    used += need
                    stats.peak_bytes = max(stats.peak_bytes, used)
                    stats.admitted += 1
                    active[r.rid] = [r, 0, now(), need]
                if not active:
                    # idle: wait for the next arrival or preparation
                    time.sleep(0.002)
                    continue
                ts = time.perf_counter()
                self.ex.step()
                stats.step_ms.append((time.perf_counter() - ts) * 1e3)
                stats.active.append(len(active))
                for rid, a in list(active.items()):
                    a[1] += 1
                    stats.cell_steps += a[0].cfg.n * a[0].cfg.n * a[0].cfg.nz
                    if a[1] >= a[0].steps:
                        case = self.ex.cases.get(rid) if hasattr(self.ex, "cases") else None
                        if self.on_finish is not None:
                            self.on_finish(a[0], case)
                        self.ex.detach(rid)
                        used -= a[3]
                        stats.finished.append(Finished(rid, a[0].cfg.n, a[0].arrival, a[2], now(), a[1]))
                        del active[rid]
        finally:
            stats.wall_s = now()
            pool.shutdown(wait=False, cancel_futures=True)
        return stats
