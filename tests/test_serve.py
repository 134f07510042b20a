"""Serving loop: admission and fault policy (host-only executor, no GPU)
and, on the GPU, every served case equals the same case run alone -- also
when other cases are cancelled, fail inside a step, or wait for memory."""
from __future__ import annotations

import time

import numpy as np
import pytest

from melt_ibm_gb300 import abi
from melt_ibm_gb300.case import CaseConfig
from melt_ibm_gb300.serve import DeviceExecutor, DeviceOOM, Request, Server, serving_requests
from tests.helpers import FIELDS_OUT, small_config


class HostExecutor:
    """Stands in for the device: footprint n^3 bytes, steps take 1 ms.
    `capacity` simulates a device smaller than the budget (admissions beyond
    it raise DeviceOOM); `fail_at` = {rid: k} makes case rid fail in its k-th
    step, as the library reports a case that failed inside a batch step."""

    def __init__(self, capacity=None, fail_at=None):
        self.cases, self.log, self.resident = {}, [], 0
        self.max_resident = 0
        self.capacity = capacity
        self.fail_at = dict(fail_at or {})
        self.steps = {}

    def estimate(self, req):
        return req.cfg.n ** 3

    def attach(self, req, case):
        if self.capacity is not None and self.resident + self.estimate(req) > self.capacity:
            self.log.append(("oom", req.rid))
            raise DeviceOOM(f"request {req.rid}")
        self.cases[req.rid] = case
        self.steps[req.rid] = 0
        self.resident += self.estimate(req)
        self.max_resident = max(self.max_resident, self.resident)
        self.log.append(("attach", req.rid))

    def detach(self, rid):
        case = self.cases.pop(rid)
        self.steps.pop(rid)
        self.resident -= case.cfg.n ** 3
        self.log.append(("detach", rid))

    def step(self):
        time.sleep(0.001)
        failed = {}
        for rid in self.steps:
            self.steps[rid] += 1
            if self.fail_at.get(rid) == self.steps[rid]:
                failed[rid] = "injected"
        return {"admission": False, "failed": failed}


def _requests():
    sizes = [16, 24, 16, 32, 24, 16]
    return [Request(rid=q, arrival=0.002 * q, cfg=small_config(n=n, level=2), steps=3 + q % 3)
            for q, n in enumerate(sizes)]


def test_admission_respects_budget_and_order():
    ex = HostExecutor()
    budget = 32 ** 3 + 24 ** 3          # never room for everything at once
    stats = Server(ex, budget).run(_requests())
    assert ex.max_resident <= budget
    assert len(stats.finished) == 6
    admitted = [rid for kind, rid in ex.log if kind == "attach"]
    assert admitted == sorted(admitted)                 # first come, first served
    s = stats.summary()
    assert s["cases_completed"] == 6 and s["step_latency_ms"]["p99"] >= s["step_latency_ms"]["p50"]


def test_request_too_large_for_budget_is_refused():
    stats = Server(HostExecutor(), 10).run(_requests()[:2])
    assert set(stats.failed) == {0, 1} and not stats.finished


def test_cancel_queued_and_resident_cases():
    ex = HostExecutor()
    reqs = _requests()
    reqs[5].arrival = 0.5                          # still queued when cancelled

    def on_step(server, k):
        if k == 1:
            server.cancel(0)                       # resident
            server.cancel(5)                       # queued, not yet arrived

    stats = Server(ex, 1 << 30, on_step=on_step).run(reqs)
    assert sorted(stats.cancelled) == [0, 5]
    assert sorted(f.rid for f in stats.finished) == [1, 2, 3, 4]
    assert ("attach", 5) not in ex.log
    assert ex.log.index(("detach", 0)) < len(ex.log) and not ex.cases


def _burst():
    """The same requests, all arrived at once and long enough to overlap:
    they compete for memory."""
    reqs = _requests()
    for r in reqs:
        r.arrival = 0.0
        r.steps += 60
    return reqs


def test_simulated_oom_is_retried_after_a_completion():
    ex = HostExecutor(capacity=32 ** 3 + 2 * 24 ** 3)
    stats = Server(ex, 1 << 30).run(_burst())          # the budget would admit everything
    ooms = [q for q, (kind, _) in enumerate(ex.log) if kind == "oom"]
    assert stats.oom_retries == len(ooms) >= 1
    assert len(stats.finished) == 6 and not stats.failed
    assert ex.max_resident <= ex.capacity
    # each retry came after a resident case had completed, and the request
    # was admitted in the end, still in arrival order
    for q in ooms[1:]:
        assert any(kind == "detach" for kind, _ in ex.log[ooms[0]:q])
    rid = ex.log[ooms[0]][1]
    at = ex.log.index(("attach", rid))
    assert any(kind == "detach" for kind, _ in ex.log[ooms[0]:at])
    admitted = [r for kind, r in ex.log if kind == "attach"]
    assert admitted == sorted(admitted)


def test_oom_with_nothing_resident_is_refused():
    ex = HostExecutor(capacity=10)
    stats = Server(ex, 1 << 30).run(_requests()[:2])
    assert set(stats.failed) == {0, 1}


def test_reduced_budget_holds_admissions():
    ex = HostExecutor()
    reduced = 32 ** 3                                  # the largest single request still fits
    after = []

    def on_step(server, k):
        if k == 0:
            server.set_budget(reduced)                 # below what is resident now
            after.append(len(ex.log))

    stats = Server(ex, 1 << 30, on_step=on_step).run(_burst())
    assert len(stats.finished) == 6 and not stats.failed
    # replay the log from the budget change: every admission made after it fits the new budget
    sizes = {r.rid: r.cfg.n ** 3 for r in _requests()}
    live = set()
    for q, (kind, rid) in enumerate(ex.log):
        if kind == "attach":
            live.add(rid)
            if q >= after[0]:
                assert sum(sizes[x] for x in live) <= reduced, (q, live)
        elif kind == "detach":
            live.discard(rid)


def test_failed_case_leaves_the_others_running():
    ex = HostExecutor(fail_at={2: 2})
    stats = Server(ex, 1 << 30).run(_requests())
    assert set(stats.failed) == {2}
    assert sorted(f.rid for f in stats.finished) == [0, 1, 3, 4, 5]


def test_serving_requests_follow_the_configured_laws():
    reqs = serving_requests(200.0, rate=2.0, seed=7, steps=5)
    assert abs(len(reqs) / 200.0 - 2.0) < 0.4
    ns = np.array([r.cfg.n for r in reqs])
    for n, p in zip((64, 96, 128, 192), (0.4, 0.3, 0.2, 0.1)):
        assert abs(np.mean(ns == n) - p) < 0.08
    assert all(2 <= r.cfg.mesh_level <= 4 and 0.3 <= r.cfg.rad_p <= 0.6 for r in reqs)
    assert all(0.5 - 1e-12 <= 1.0 / r.cfg.latheat <= 4.0 + 1e-12 for r in reqs)
    assert all(0.005 <= 1.0 / r.cfg.ren <= 0.02 for r in reqs)


@pytest.mark.gpu
@pytest.mark.parametrize("step_cells", [None, 32 ** 3])
def test_served_cases_equal_cases_run_alone(gpu_lib, step_cells):
    """Every case equals the same case run alone, with all resident cases in
    every batch step and with a work budget that advances a subset per step."""
    from melt_ibm_gb300.case import Case
    reqs = _requests()
    results = {}

    def keep(req, case):
        case.sync_to_host(gpu_lib, -1)
        results[req.rid] = {k: case.interior(f).copy() for k, f in FIELDS_OUT.items()}

    ex = DeviceExecutor(gpu_lib)
    stats = Server(ex, budget_bytes=1 << 40, on_finish=keep, step_cells=step_cells).run(reqs)
    ex.close()
    assert len(stats.finished) == len(reqs)
    assert max(stats.active) >= 2                      # the cases were resident together
    if step_cells is not None:
        assert max(stats.stepped_cells) <= max(step_cells, max(r.cfg.n ** 3 for r in reqs))
    for r in reqs:
        c = Case(r.cfg)
        c.attach(gpu_lib)
        c.bind(gpu_lib)
        gpu_lib.mibm_set_precision_(abi.ref_int(r.precision), abi.ref_int(2))
        c.run(gpu_lib, r.steps)
        c.sync_to_host(gpu_lib, -1)
        for k, f in FIELDS_OUT.items():
            assert np.array_equal(c.interior(f), results[r.rid][k]), (r.rid, k)
        c.detach(gpu_lib)


@pytest.mark.gpu
def test_faults_leave_other_cases_bitwise_unchanged(gpu_lib):
    """A cancelled resident case, a case whose velocity turns non-finite
    between two steps (the CFL guard fails it inside the batch step), and an
    admission that runs out of (simulated) device memory and waits for a
    completion: every case that completes equals the same case run alone,
    bit for bit."""
    from melt_ibm_gb300.case import Case
    reqs = _requests()
    results = {}

    def keep(req, case):
        case.sync_to_host(gpu_lib, -1)
        results[req.rid] = {k: case.interior(f).copy() for k, f in FIELDS_OUT.items()}

    ex = DeviceExecutor(gpu_lib)
    one = ex.model_bytes(reqs[0].cfg, 1)
    ex.capacity = int(2.5 * one)                       # room for two resident cases

    def on_step(server, k):
        if k == 1:
            server.cancel(1)
        if k == 2 and 0 in ex.cases:
            c = ex.cases[0]
            c.sync_to_host(gpu_lib, -1)
            c.fields[abi.MIBM_F_VX][3, 2, 4] = np.nan
            c.sync_from_host(gpu_lib, 1 << abi.MIBM_F_VX)

    stats = Server(ex, budget_bytes=1 << 40, on_finish=keep, on_step=on_step).run(reqs)
    ex.close()
    assert stats.cancelled == [1]
    assert list(stats.failed) == [0] and "status 10" in stats.failed[0]     # MIBM_ENONFINITE
    assert stats.oom_retries >= 1
    assert sorted(results) == [2, 3, 4, 5]
    for r in reqs:
        if r.rid not in results:
            continue
        c = Case(r.cfg)
        c.attach(gpu_lib)
        c.bind(gpu_lib)
        gpu_lib.mibm_set_precision_(abi.ref_int(r.precision), abi.ref_int(2))
        c.run(gpu_lib, r.steps)
        c.sync_to_host(gpu_lib, -1)
        for k, f in FIELDS_OUT.items():
            assert np.array_equal(c.interior(f), results[r.rid][k]), (r.rid, k)
        c.detach(gpu_lib)


class BudgetExecutor(HostExecutor):
    """HostExecutor that records which cases each batch step advanced."""

    def __init__(self):
        super().__init__()
        self.advanced = []

    def step(self, rids=None):
        rids = list(self.steps) if rids is None else list(rids)
        self.advanced.append(list(rids))
        for rid in rids:
            self.steps[rid] += 1
        return {"admission": False, "failed": {}}


def test_step_budget_round_robin_keeps_every_case_in_order():
    """With a work budget per batch step, each step advances the cases that
    waited longest within the budget (at least one), every case still gets
    exactly its steps, and no step exceeds the budget unless one case alone
    does."""
    reqs = [Request(rid=q, arrival=0.0, cfg=small_config(n=n), steps=5)
            for q, n in enumerate([32, 16, 24, 16, 32, 24])]
    ex = BudgetExecutor()
    budget = 32 ** 3 + 16 ** 3
    stats = Server(ex, budget_bytes=1 << 40, step_cells=budget).run(reqs)
    assert sorted(f.rid for f in stats.finished) == list(range(6))
    assert all(f.steps == 5 for f in stats.finished)
    size = {r.rid: r.cfg.n ** 3 for r in reqs}
    for rids in ex.advanced:
        assert len(rids) >= 1
        assert len(rids) == 1 or sum(size[r] for r in rids) <= budget
    # no starvation: the case that has waited longest is always advanced,
    # so no case waits more batch steps than there are resident cases
    last = {}
    for k, rids in enumerate(ex.advanced):
        for r in rids:
            assert r not in last or k - last[r] <= len(reqs), (r, k, last[r])
            last[r] = k
