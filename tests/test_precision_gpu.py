"""The precision form (FP32 compute on FP64 fields, refined projection).

Acceptance bar: relative L2 error <= 1e-6 per field against the FP64 run
from identical inputs, and divergence <= 1e-10 after every step.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from melt_ibm_gb300 import abi
from melt_ibm_gb300.case import Case, CaseConfig, CONFIG0
from tests.helpers import FIELDS_OUT, pair, rel_l2, set_substep, small_config

pytestmark = pytest.mark.gpu
TOL_FIELD = 1e-6
TOL_DIV = 1e-10


def _run(case, lib, nsteps, precision, nproj=2, divs=None):
    c = case.clone()
    c.attach(lib)
    c.bind(lib)
    lib.mibm_set_precision_(C.byref(C.c_int(precision)), C.byref(C.c_int(nproj)))
    lib.check("set_precision")
    for nt in range(1, nsteps + 1):
        c.step(lib, nt)
        if divs is not None:
            divs.append(lib.mibm_divergence_max_())
    c.sync_to_host(lib, -1)
    out = {k: c.interior(f).copy() for k, f in FIELDS_OUT.items()}
    vol = c.S(abi.MIBM_S_VOLUME)
    c.detach(lib)
    return out, vol


@pytest.mark.parametrize("nsteps", [1, 10])
def test_precision_form_error_and_divergence(gpu_lib, nsteps):
    case = Case(CaseConfig(**CONFIG0))
    ref, _ = _run(case, gpu_lib, nsteps, 0)
    divs = []
    got, _ = _run(case, gpu_lib, nsteps, 1, divs=divs)
    errs = {k: rel_l2(got[k], ref[k]) for k in FIELDS_OUT}
    print("precision form errors vs FP64 after", nsteps, "steps:", errs, "max div", max(divs))
    for k, e in errs.items():
        assert e <= TOL_FIELD, f"{k}: {e:.3e}"
    assert max(divs) <= TOL_DIV


def test_precision_form_single_solve_is_not_enough(gpu_lib):
    """Without refinement the FP32 projection leaves divergence well above 1e-10."""
    case = Case(small_config(n=32, level=2))
    divs = []
    _run(case, gpu_lib, 2, 1, nproj=1, divs=divs)
    assert max(divs) > TOL_DIV


def test_precision_form_deterministic(gpu_lib):
    case = Case(small_config(n=32, level=3))
    a, _ = _run(case, gpu_lib, 2, 1)
    b, _ = _run(case, gpu_lib, 2, 1)
    for k in FIELDS_OUT:
        assert np.array_equal(a[k], b[k]), k


def _mls_pair(oracle_lib, gpu_lib):
    case = Case(small_config(n=24, level=2))
    co, cg = pair(case, oracle_lib, gpu_lib, initial_tag=True)
    cg.bind(gpu_lib)
    gpu_lib.mibm_set_precision_(C.byref(C.c_int(1)), C.byref(C.c_int(2)))
    gpu_lib.check("set_precision")
    return co, cg


def test_precision_mls_weights_match_oracle(oracle_lib, gpu_lib):
    """Shifted-basis, separable-moment MLS weights (precision form) against the
    reference construction: equal up to the reference's own conditioning error."""
    co, cg = _mls_pair(oracle_lib, gpu_lib)
    for c, lib in ((co, oracle_lib), (cg, gpu_lib)):
        c.bind(lib)
        lib.findcentroidindices_()
        lib.mlsweight_()
        lib.check("mlsweight")
    cg.sync_to_host(gpu_lib, -1)
    for mid in (abi.MIBM_M_PTXAB_Q1, abi.MIBM_M_PTXAB_Q2, abi.MIBM_M_PTXAB_Q3, abi.MIBM_M_PTXAB_TEMP):
        e = rel_l2(cg.mesh_arrays[mid], co.mesh_arrays[mid])
        assert e <= 1e-8, (mid, e)


def test_precision_heat_flux_matches_oracle(oracle_lib, gpu_lib):
    co, cg = _mls_pair(oracle_lib, gpu_lib)
    for c, lib in ((co, oracle_lib), (cg, gpu_lib)):
        c.bind(lib)
        set_substep(c, 0, dt=0.01)
        lib.findprobeindices_()
        lib.mls_heatflux_()
        lib.check("heat")
    cg.sync_to_host(gpu_lib, -1)
    for mid in (abi.MIBM_M_QW_O, abi.MIBM_M_QW_I, abi.MIBM_M_QW_OVERT, abi.MIBM_M_QW_IVERT):
        e = rel_l2(cg.mesh_arrays[mid], co.mesh_arrays[mid])
        assert e <= 1e-7, (mid, e)
