"""mibm_pin_host_: page-locked host arrays change how the copies run, not
what they carry -- a run with host copies every step gives the same bits
pinned or not; release and re-pin work on a live context."""
from __future__ import annotations

import numpy as np
import pytest

from melt_ibm_gb300 import abi
from melt_ibm_gb300.case import Case
from tests.helpers import FIELDS_OUT, small_config

pytestmark = pytest.mark.gpu
A = abi
ALL = -1


def _run(gpu_lib, pin):
    c = Case(small_config(n=32, level=3))
    c.attach(gpu_lib)
    c.bind(gpu_lib)
    if pin:
        assert gpu_lib.mibm_pin_host_(A.ref_int(1)) == 0
    for nt in range(1, 4):
        c.sync_from_host(gpu_lib, ALL)
        c.step(gpu_lib, nt)
        c.sync_to_host(gpu_lib, ALL)
    if pin:
        assert gpu_lib.mibm_pin_host_(A.ref_int(0)) == 0
        assert gpu_lib.mibm_pin_host_(A.ref_int(1)) == 0      # pin again, then let destroy release
    out = ({k: c.interior(f).copy() for k, f in FIELDS_OUT.items()}, c.mesh_arrays[A.MIBM_M_XYZV].copy())
    c.detach(gpu_lib)
    return out


def test_pinned_copies_same_results(gpu_lib):
    (f0, x0), (f1, x1) = _run(gpu_lib, False), _run(gpu_lib, True)
    for k in FIELDS_OUT:
        assert np.array_equal(f0[k], f1[k]), k
    assert np.array_equal(x0, x1)
