"""Per-step diagnostics on the GPU (CalcDissipation diss.f90:11-201,
vorticity vorticity.f90:1-109, calcFluidVelAvgs calcSlipVels.f90:17-181)
against the oracle, through the C-ABI.

The sums run over the fully fluid cells in a different (fixed) order than
the reference's loop, so on identical fields the values agree to summation
round-off (1e-12 relative); after time steps they agree to the steps' own
parity.  The per-step mode must return the numbers of a direct call after
the same step and must not change the step's results (bitwise).
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from melt_ibm_gb300 import abi
from melt_ibm_gb300.case import Case
from tests.helpers import FIELDS_OUT, pair, small_config

pytestmark = pytest.mark.gpu
A = abi
ALL = -1


def _diag(case, lib):
    case.bind(lib)
    out = np.zeros(A.MIBM_NDIAG)
    st = lib.mibm_diagnostics_(out.ctypes.data)
    assert st == 0, lib.mibm_last_message()
    return out


def _close(a, b, tol=1e-12, floor=0.0):
    for q in range(A.MIBM_NDIAG):
        assert abs(a[q] - b[q]) <= tol * abs(b[q]) + floor, (q, a[q], b[q])


@pytest.mark.parametrize("imlsstr", [0, 1])
def test_diagnostics_parity_after_steps(oracle_lib, gpu_lib, imlsstr):
    case = Case(small_config(n=24, level=2, imlsstr=imlsstr, dens_ratio=2.0))
    co, cg = pair(case, oracle_lib, gpu_lib)
    for c, lib in ((co, oracle_lib), (cg, gpu_lib)):
        c.run(lib, 2)
    d_o, d_g = _diag(co, oracle_lib), _diag(cg, gpu_lib)
    # means of fields that agree to 1e-10; near-zero means (u, w_rel ...)
    # get an absolute floor of the same order times the rms.  With a moving
    # body the velocities relative to it carry the body's MLS noise (~1e-10
    # absolute after a few steps, whichever side computes it): floor 1e-9.
    floor = (1e-9 if imlsstr else 1e-10) * max(1.0, d_o[A.MIBM_D_URMS])
    _close(d_g, d_o, tol=1e-9, floor=floor)
    assert d_o[A.MIBM_D_NFLUID] == d_g[A.MIBM_D_NFLUID]
    assert 0 < d_o[A.MIBM_D_NFLUID] < case.n1m * case.n2m * case.n3m


def test_diagnostics_same_state(oracle_lib, gpu_lib):
    """Identical fields on both sides (no time stepping): summation round-off only."""
    case = Case(small_config(n=32, level=3))
    co, cg = pair(case, oracle_lib, gpu_lib)
    d_o = _diag(co, oracle_lib)
    _close(_diag(cg, gpu_lib), d_o, tol=1e-12, floor=1e-14 * max(1.0, d_o[A.MIBM_D_URMS]))


@pytest.mark.parametrize("precision", [0, 1])
def test_diagnostics_per_step_mode(gpu_lib, precision):
    case = Case(small_config(n=32, level=3, imlsstr=1, dens_ratio=2.0))
    runs = []
    for on in (0, 1):
        c = case.clone()
        c.attach(gpu_lib)
        c.bind(gpu_lib)
        gpu_lib.mibm_set_precision_(C.byref(C.c_int(precision)), C.byref(C.c_int(2)))
        gpu_lib.mibm_set_diagnostics_(C.byref(C.c_int(on)))
        gpu_lib.check("setup")
        per_step = []
        for nt in range(1, 4):
            c.step(gpu_lib, nt)
            if on:
                out = np.zeros(A.MIBM_NDIAG)
                assert gpu_lib.mibm_diagnostics_get_(out.ctypes.data) == 0
                per_step.append(out)
        direct = _diag(c, gpu_lib)
        c.sync_to_host(gpu_lib, ALL)
        runs.append(({k: c.interior(f).copy() for k, f in FIELDS_OUT.items()}, per_step, direct))
        c.detach(gpu_lib)
    (f0, _, d0), (f1, steps, d1) = runs
    for k in FIELDS_OUT:
        assert np.array_equal(f0[k], f1[k]), k         # diagnostics change nothing
    assert np.array_equal(steps[-1], d1)              # per-step value = direct call after the step
    assert np.array_equal(d0, d1)
    assert not np.array_equal(steps[0], steps[-1])
