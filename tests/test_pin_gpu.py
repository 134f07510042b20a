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


def test_host_uploads_each_step_graph_vs_direct(gpu_lib):
    """A host that uploads fields and mesh before every step (the e2e pattern):
    the step graph is kept across the uploads (the scatter-plan rebuild they
    request is read at replay), and its results equal direct launches."""
    import ctypes as C
    outs = []
    for graphs in (0, 1):
        c = Case(small_config(n=32, level=3, imlsstr=1, dens_ratio=2.0))
        c.attach(gpu_lib)
        c.bind(gpu_lib)
        gpu_lib.mibm_set_graphs_(C.byref(C.c_int(graphs)))
        for nt in range(1, 5):
            c.sync_from_host(gpu_lib, ALL)
            c.step(gpu_lib, nt)
            c.sync_to_host(gpu_lib, ALL)
        outs.append(({k: c.interior(f).copy() for k, f in FIELDS_OUT.items()}, c.mesh_arrays[A.MIBM_M_XYZV].copy()))
        c.detach(gpu_lib)
    (f0, x0), (f1, x1) = outs
    for k in FIELDS_OUT:
        assert np.array_equal(f0[k], f1[k]), k
    assert np.array_equal(x0, x1)
