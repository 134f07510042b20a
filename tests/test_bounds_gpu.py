"""The bounds build (-DMIBM_BOUNDS): every checked index of the stencils, line
solves, narrow-band tagging, force scatter and cell indexing is tested
against its array; an index out of range skips the access and is counted on
the device instead of faulting.

* the check itself works: a planted out-of-range index in a kernel of its
  own (checked before the access) is counted;
* whole steps of both forms, with a free melting body, HIT forcing,
  per-step diagnostics and the staged line solves, touch no index out of
  range, and give the same bits as the normal build.
"""
from __future__ import annotations

import numpy as np
import pytest

from melt_ibm_gb300 import abi
from melt_ibm_gb300.case import Case
from tests.helpers import FIELDS_OUT, small_config

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="session")
def bounds_lib(gpu_lib):
    from melt_ibm_gb300 import build as mbuild
    lib = abi.Lib(mbuild.build(bounds=True))
    assert lib.mibm_bounds_check_() >= 0, "the bounds library was not built with -DMIBM_BOUNDS"
    return lib


def test_planted_index_is_caught(bounds_lib):
    assert bounds_lib.mibm_bounds_selftest_() == 0


def _run(case, lib, nsteps, precision):
    c = case.clone()
    c.attach(lib)
    c.bind(lib)
    lib.mibm_set_precision_(abi.ref_int(precision), abi.ref_int(2))
    lib.mibm_set_diagnostics_(abi.ref_int(1))
    lib.check("setup")
    c.run(lib, nsteps)
    c.sync_to_host(lib, -1)
    out = {k: c.interior(f).copy() for k, f in FIELDS_OUT.items()}
    out["xyzv"] = c.mesh_arrays[abi.MIBM_M_XYZV].copy()
    c.detach(lib)
    return out


@pytest.mark.parametrize("precision", [0, 1])
def test_steps_touch_no_index_out_of_range(bounds_lib, gpu_lib, precision):
    case = Case(small_config(n=32, level=2, imlsstr=1, dens_ratio=2.0, forcing=1, which_hit=1, c_hit=0.2))
    assert bounds_lib.mibm_bounds_check_() >= 0            # drain
    got = _run(case, bounds_lib, 3, precision)
    assert bounds_lib.mibm_bounds_check_() == 0
    ref = _run(case, gpu_lib, 3, precision)
    for k in got:
        assert np.array_equal(got[k], ref[k]), k
