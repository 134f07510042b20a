"""Parity at the configurations' own sizes, through the C-ABI, against the
CPU oracle.

* The plain configuration (64^3, 10 steps) on the reference's own mesh
  (gts/unitSphere_N3.gts, as a fixture) instead of the generated icosphere.
* The 128^3 configuration as the benchmark runs it (melt128_c1: free melting
  body under Newton-Euler, linear forcing, level-4 icosphere): u, v, w, T, p
  within 1e-10 relative L2 after 1 and 10 steps; the rigid state (vel_CM,
  omega_c, pos_CM, quat) within 1e-9 and the vertices within 1e-11.  The
  rigid state is bounded by the reference's own MLS noise: its loads come from
  moment matrices with condition numbers ~1e7 at 128^3, so a last-bit
  difference of the moving body's geometry (which carries the fluid solver's
  round-off) changes them by ~1e-9 of their size -- as a different MPI
  decomposition of the reference, which reorders its Allreduce of the loads,
  would.
* The 256^3 configuration (melt256_c2: spheroid, Eswaran-Pope forcing,
  Boussinesq, St = 2): the FP64 form within 1e-10 after 1 and 2 steps with
  post-projection divergence <= 1e-12; the precision form from identical
  inputs within 1e-6 of the oracle's FP64 run per field, divergence <= 1e-10.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from melt_ibm_gb300 import abi
from melt_ibm_gb300.case import Case, CaseConfig, CONFIG0
from melt_ibm_gb300.fields import discrete_divergence_max
from melt_ibm_gb300.workloads import WORKLOADS
from tests.helpers import FIELDS_OUT, rel_l2
from tests.test_mesh_fixture import reference_n3

pytestmark = pytest.mark.gpu
A = abi
ALL = -1
TOL_STEP = 1e-10
RIGID = {"vel_CM": (A.MIBM_S_VEL_CM, 3), "omega_c": (A.MIBM_S_OMEGA_C, 3), "pos_CM": (A.MIBM_S_POS_CM, 3),
         "quat": (A.MIBM_S_QUAT, 4)}


def _snap(case):
    return {k: case.interior(f).copy() for k, f in FIELDS_OUT.items()}


def _div(case, f):
    return discrete_divergence_max(f["vx"], f["vy"], f["vz"], case.xlen, case.ylen, case.zlen)


def _paired_runs(cfg: CaseConfig, oracle_lib, gpu_lib, checkpoints, precision=False):
    """Run the oracle and the GPU from identical inputs; snapshots of the
    fields (and rigid state, vertices) at each checkpoint step count."""
    case = Case(cfg)
    co, cg = case.clone(), case.clone()
    co.attach(oracle_lib)
    cg.attach(gpu_lib)
    cg.bind(gpu_lib)
    gpu_lib.mibm_set_precision_(C.byref(C.c_int(1 if precision else 0)), C.byref(C.c_int(2)))
    gpu_lib.check("set_precision")
    out, done = {}, 0
    for upto in checkpoints:
        co.run(oracle_lib, upto - done, start=done + 1)
        cg.run(gpu_lib, upto - done, start=done + 1)
        cg.sync_to_host(gpu_lib, ALL)
        out[upto] = {"oracle": _snap(co), "gpu": _snap(cg),
                     "rigid": {k: (co.sc[s, :w].copy(), cg.sc[s, :w].copy()) for k, (s, w) in RIGID.items()},
                     "xyzv": (co.mesh_arrays[A.MIBM_M_XYZV].copy(), cg.mesh_arrays[A.MIBM_M_XYZV].copy()),
                     "volume": (co.S(A.MIBM_S_VOLUME), cg.S(A.MIBM_S_VOLUME))}
        done = upto
    cg.detach(gpu_lib)
    co.detach(oracle_lib)
    return case, out


# ------------------------------------------------------------ plain, reference mesh
@pytest.fixture(scope="module")
def config0_reference_mesh(oracle_lib, gpu_lib):
    cfg = CaseConfig(**CONFIG0, mesh=reference_n3())
    return _paired_runs(cfg, oracle_lib, gpu_lib, (1, 10))


@pytest.mark.parametrize("after", [1, 10])
def test_config0_on_reference_mesh(config0_reference_mesh, after):
    case, out = config0_reference_mesh
    r = out[after]
    for k in FIELDS_OUT:
        err = rel_l2(r["gpu"][k], r["oracle"][k])
        assert err <= TOL_STEP, f"{k} after {after} steps: rel L2 {err:.3e}"
    vo, vg = r["volume"]
    assert abs(vg - vo) <= 1e-10 * abs(vo)
    assert _div(case, r["gpu"]) <= 1e-12


# ------------------------------------------------------------ 128^3 free body
@pytest.fixture(scope="module")
def config1_runs(oracle_lib, gpu_lib):
    return _paired_runs(CaseConfig(**WORKLOADS["melt128_c1"]), oracle_lib, gpu_lib, (1, 10))


@pytest.mark.parametrize("after", [1, 10])
def test_config1_128_fields(config1_runs, after):
    _, out = config1_runs
    r = out[after]
    for k in FIELDS_OUT:
        err = rel_l2(r["gpu"][k], r["oracle"][k])
        assert err <= TOL_STEP, f"{k} after {after} steps: rel L2 {err:.3e}"


@pytest.mark.parametrize("after", [1, 10])
def test_config1_128_rigid_state_and_vertices(config1_runs, after):
    _, out = config1_runs
    r = out[after]
    for k, (a, b) in r["rigid"].items():
        err = np.abs(b - a).max() / max(1.0, np.abs(a).max())
        assert err <= 1e-9, f"{k} after {after} steps: {err:.3e} ({a} vs {b})"
    xo, xg = r["xyzv"]
    assert rel_l2(xg, xo) <= 1e-11
    assert np.abs(r["rigid"]["vel_CM"][0]).max() > 0.0        # the body does move


# ------------------------------------------------------------ 256^3, both forms
@pytest.fixture(scope="module")
def config2_runs(oracle_lib, gpu_lib):
    cfg = CaseConfig(**WORKLOADS["melt256_c2"])
    case, out = _paired_runs(cfg, oracle_lib, gpu_lib, (1, 2))
    # the precision form from the same inputs; the oracle run above is its reference
    cp = case.clone()
    cp.attach(gpu_lib)
    cp.bind(gpu_lib)
    gpu_lib.mibm_set_precision_(C.byref(C.c_int(1)), C.byref(C.c_int(2)))
    gpu_lib.check("set_precision")
    done = 0
    for upto in (1, 2):
        cp.run(gpu_lib, upto - done, start=done + 1)
        cp.sync_to_host(gpu_lib, ALL)
        out[upto]["precision"] = _snap(cp)
        done = upto
    cp.detach(gpu_lib)
    return case, out


@pytest.mark.parametrize("after", [1, 2])
def test_config2_256_fp64(config2_runs, after):
    case, out = config2_runs
    r = out[after]
    for k in FIELDS_OUT:
        err = rel_l2(r["gpu"][k], r["oracle"][k])
        assert err <= TOL_STEP, f"{k} after {after} steps: rel L2 {err:.3e}"
    assert _div(case, r["gpu"]) <= 1e-12


@pytest.mark.parametrize("after", [1, 2])
def test_config2_256_precision_form(config2_runs, after):
    case, out = config2_runs
    r = out[after]
    for k in FIELDS_OUT:
        err = rel_l2(r["precision"][k], r["oracle"][k])
        assert err <= 1e-6, f"{k} after {after} steps: rel L2 {err:.3e}"
    assert _div(case, r["precision"]) <= 1e-10
