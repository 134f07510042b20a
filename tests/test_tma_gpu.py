"""Alternative data paths of the precision form against each other.

Staged line solves (bulk tensor copies into shared memory) against the same
solves reading global memory directly; the one-pass u, v, w explicit-term
kernel against the advection-products kernel followed by one RHS kernel per
component.

Both paths run the same arithmetic in the same order, so a step must give
the same bits either way: on grids whose width is a multiple of the 32-cell
tile and on one that is not (the last tile's missing columns are filled with
zeros by the copy), for z-lines of the longest staged length (256) and for
the velocity (three fields per launch) and temperature (one field and its
FP32 mirror) solves.  The precision form against the FP64 form stays within
its 1e-6 bar with the staged path on.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from melt_ibm_gb300 import abi
from melt_ibm_gb300.case import Case
from tests.helpers import FIELDS_OUT, randomize, rel_l2, small_config

pytestmark = pytest.mark.gpu


def _run(case, lib, nsteps, precision, tma, fused_uvw=1):
    c = case.clone()
    c.attach(lib)
    c.bind(lib)
    lib.mibm_set_precision_(C.byref(C.c_int(precision)), C.byref(C.c_int(2)))
    lib.check("set_precision")
    lib.mibm_set_tma_(C.byref(C.c_int(tma)))
    lib.mibm_set_fused_uvw_(C.byref(C.c_int(fused_uvw)))
    lib.check("set_tma")
    for nt in range(1, nsteps + 1):
        c.step(lib, nt)
    c.sync_to_host(lib, -1)
    out = {k: c.interior(f).copy() for k, f in FIELDS_OUT.items()}
    c.detach(lib)
    return out


def _case(n, n3, level, which_hit):
    if n == n3:
        return Case(small_config(n=n, level=level, forcing=1, which_hit=which_hit, c_hit=0.2, betagz=0.3))
    case = Case(small_config(n=n, n3=n3, level=level, velocity="rest", betagz=0.3))
    randomize(case, forcing=False)      # non-cubic grids start at rest: seeded noise in every field
    if which_hit:
        case.iv[abi.MIBM_I_FORCING] = 1
        case.iv[abi.MIBM_I_WHICH_HIT] = which_hit
    return case


@pytest.mark.parametrize("n,n3,level,which_hit", [(48, 256, 2, 0), (64, 64, 3, 3), (32, 128, 2, 1)])
def test_one_pass_uvw_bitwise_equal_products_path(gpu_lib, n, n3, level, which_hit):
    case = _case(n, n3, level, which_hit)
    one = _run(case, gpu_lib, 3, 1, 1, fused_uvw=1)
    two = _run(case, gpu_lib, 3, 1, 1, fused_uvw=0)
    for k in FIELDS_OUT:
        assert np.array_equal(one[k], two[k]), k


@pytest.mark.parametrize("n,n3,level,which_hit", [(48, 256, 2, 0), (64, 64, 3, 3), (32, 128, 2, 1)])
def test_staged_solves_bitwise_equal_direct(gpu_lib, n, n3, level, which_hit):
    case = _case(n, n3, level, which_hit)
    staged = _run(case, gpu_lib, 3, 1, 1)
    direct = _run(case, gpu_lib, 3, 1, 0)
    for k in FIELDS_OUT:
        assert np.array_equal(staged[k], direct[k]), k


def test_staged_precision_form_within_bar(gpu_lib):
    case = Case(small_config(n=48, level=3))
    ref = _run(case, gpu_lib, 4, 0, 1)
    got = _run(case, gpu_lib, 4, 1, 1)
    for k in FIELDS_OUT:
        assert rel_l2(got[k], ref[k]) <= 1e-6, k


def test_set_tma_rejects_bad_values(gpu_lib):
    case = Case(small_config(n=32, level=2))
    c = case.clone()
    c.attach(gpu_lib)
    c.bind(gpu_lib)
    gpu_lib.mibm_set_tma_(C.byref(C.c_int(2)))
    assert gpu_lib.mibm_last_status_() != 0
    c.detach(gpu_lib)
