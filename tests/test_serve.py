"""Serving loop: admission policy (host-only executor, no GPU) and, on the
GPU, every served case equals the same case run alone."""
from __future__ import annotations

import time

import numpy as np
import pytest

from melt_ibm_gb300 import abi
from melt_ibm_gb300.case import CaseConfig
from melt_ibm_gb300.serve import DeviceExecutor, Request, Server, serving_requests
from tests.helpers import FIELDS_OUT, small_config


class HostExecutor:
    """Stands in for the device: footprint n^3 bytes, steps take 1 ms."""

    def __init__(self):
        self.cases, self.log, self.resident = {}, [], 0
        self.max_resident = 0

    def estimate(self, req):
        return req.cfg.n ** 3

    def attach(self, req, case):
        self.cases[req.rid] = case
        self.resident += self.estimate(req)
        self.max_resident = max(self.max_resident, self.resident)
        self.log.append(("attach", req.rid))

    def detach(self, rid):
        case = self.cases.pop(rid)
        self.resident -= case.cfg.n ** 3
        self.log.append(("detach", rid))

    def step(self):
        time.sleep(0.001)


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
    with pytest.raises(ValueError):
        Server(HostExecutor(), 10).run(_requests()[:1])


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
def test_served_cases_equal_cases_run_alone(gpu_lib):
    from melt_ibm_gb300.case import Case
    reqs = _requests()
    results = {}

    def keep(req, case):
        case.sync_to_host(gpu_lib, -1)
        results[req.rid] = {k: case.interior(f).copy() for k, f in FIELDS_OUT.items()}

    ex = DeviceExecutor(gpu_lib)
    stats = Server(ex, budget_bytes=1 << 40, on_finish=keep).run(reqs)
    ex.close()
    assert len(stats.finished) == len(reqs)
    assert max(stats.active) >= 2                      # the cases did share batch steps
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
