"""Non-finite guard of the CFL reduction (cfl.f90:1-31 plus the library's
own check): a NaN or Inf in a velocity component or in the temperature of an
owned cell makes cfl_ report MIBM_ENONFINITE instead of a CFL number that
silently dropped it.  The oracle cases run on the CPU; the GPU cases put the
same poisoned fields on the device through mibm_sync_from_host_ and read the
status through the C-ABI, in both arithmetic forms and through the batched
step.  No device fault is involved: the kernel raises a flag that the host
reads after the reduction.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from melt_ibm_gb300 import abi as A
from melt_ibm_gb300.batch import BatchRunner
from melt_ibm_gb300.case import Case
from tests.helpers import small_config

ALL = -1


def _poison(case, fid, value, ijk=(3, 4, 5)):
    case.interior(fid)[ijk] = value
    case.fill_ghosts(fid)


@pytest.mark.parametrize("fid, value", [(A.MIBM_F_VX, np.nan), (A.MIBM_F_VZ, np.inf),
                                        (A.MIBM_F_TEMP, np.nan), (A.MIBM_F_TEMP, -np.inf)])
def test_oracle_cfl_flags_non_finite(oracle_lib, fid, value):
    case = Case(small_config(n=16, level=2))
    _poison(case, fid, value)
    case.attach(oracle_lib)
    case.bind(oracle_lib)
    oracle_lib.cfl_()
    assert oracle_lib.mibm_last_status_() == A.MIBM_ENONFINITE
    assert b"non-finite" in oracle_lib.mibm_last_message()
    case.detach(oracle_lib)


def test_oracle_cfl_clean_fields_pass(oracle_lib):
    case = Case(small_config(n=16, level=2))
    case.attach(oracle_lib)
    case.run(oracle_lib, 1)          # Case.step checks cfl_'s status
    assert np.isfinite(case.S(A.MIBM_S_CFLM)) and case.S(A.MIBM_S_CFLM) > 0
    case.detach(oracle_lib)


def test_oracle_step_stops_on_non_finite(oracle_lib):
    case = Case(small_config(n=16, level=2))
    case.attach(oracle_lib)
    case.run(oracle_lib, 1)
    _poison(case, A.MIBM_F_VY, np.nan)
    with pytest.raises(RuntimeError, match="status 10"):
        case.step(oracle_lib, 2)
    case.detach(oracle_lib)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("fid, value", [(A.MIBM_F_VX, np.nan), (A.MIBM_F_TEMP, np.inf)])
def test_gpu_cfl_flags_non_finite(gpu_lib, precision, fid, value):
    case = Case(small_config(n=24, level=2))
    case.attach(gpu_lib)
    case.bind(gpu_lib)
    gpu_lib.mibm_set_precision_(C.byref(C.c_int(precision)), C.byref(C.c_int(2)))
    case.run(gpu_lib, 2)                       # clean steps: no flag
    _poison(case, fid, value)
    case.sync_from_host(gpu_lib, ALL)
    gpu_lib.cfl_()
    assert gpu_lib.mibm_last_status_() == A.MIBM_ENONFINITE
    assert b"non-finite" in gpu_lib.mibm_last_message()
    case.detach(gpu_lib)


def _batch_stops(lib):
    cases = [Case(small_config(n=16, level=2, seed=s)) for s in (1, 2)]
    for c in cases:
        c.attach(lib)
    with BatchRunner(lib, cases) as b:
        b.step()
        _poison(cases[1], A.MIBM_F_VX, np.nan)
        cases[1].sync_from_host(lib, ALL)
        with pytest.raises(RuntimeError, match=r"\(10\)"):
            b.step()
    for c in cases:
        c.detach(lib)


def test_oracle_batch_stops_on_non_finite(oracle_lib):
    _batch_stops(oracle_lib)


@pytest.mark.gpu
def test_gpu_batch_stops_on_non_finite(gpu_lib):
    _batch_stops(gpu_lib)
