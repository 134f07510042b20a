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


def _snap(c):
    return {k: c.interior(f).copy() for k, f in FIELDS_OUT.items()}, c.mesh_arrays[A.MIBM_M_XYZV].copy()


@pytest.mark.parametrize("pin", [0, 1])
def test_identical_upload_keeps_state(gpu_lib, pin):
    """Downloading everything and uploading it back unchanged between steps
    (the e2e pattern) gives the bits of a run without host copies: the
    uploaded mesh compares equal, so the geometry work the previous step
    enqueued stands."""
    outs = []
    for copies in (False, True):
        c = Case(small_config(n=32, level=3, imlsstr=1, dens_ratio=2.0))
        c.attach(gpu_lib)
        c.bind(gpu_lib)
        if pin:
            assert gpu_lib.mibm_pin_host_(A.ref_int(1)) == 0
        for nt in range(1, 5):
            if copies:
                c.sync_to_host(gpu_lib, ALL)
                c.sync_from_host(gpu_lib, ALL)
            c.step(gpu_lib, nt)
        c.sync_to_host(gpu_lib, ALL)
        outs.append(_snap(c))
        c.detach(gpu_lib)
    (f0, x0), (f1, x1) = outs
    for k in FIELDS_OUT:
        assert np.array_equal(f0[k], f1[k]), k
    assert np.array_equal(x0, x1)


@pytest.mark.parametrize("what", ["mesh", "vofp", "velocity"])
@pytest.mark.parametrize("moving", [False, True])
def test_changed_upload_matches_oracle(gpu_lib, oracle_lib, what, moving):
    """A host that changes the mesh, the volume fraction or the velocity
    between steps: the step after the upload sees the new values (a changed
    mesh or VOF redoes the geometry work enqueued by the previous step) and
    matches the oracle doing the same."""
    from tests.helpers import rel_l2
    kw = dict(imlsstr=1, dens_ratio=2.0) if moving else {}
    outs = []
    for lib in (oracle_lib, gpu_lib):
        c = Case(small_config(n=32, level=3, **kw))
        c.attach(lib)
        c.bind(lib)
        c.step(lib, 1)
        c.sync_to_host(lib, ALL)
        if what == "mesh":
            x = c.mesh_arrays[A.MIBM_M_XYZV]
            x[0] += 0.37 / c.dx1                      # the body moves by a third of a cell in x
            mask = 1 << (32 + A.MIBM_M_XYZV)
        elif what == "vofp":
            v = c.fields[A.MIBM_F_VOFP]
            v[v < 0.5] = 0.0                          # sharpened volume fraction
            c.fill_ghosts(A.MIBM_F_VOFP)
            mask = 1 << A.MIBM_F_VOFP
        else:
            c.fields[A.MIBM_F_VX][...] *= 0.5
            c.fill_ghosts(A.MIBM_F_VX)
            mask = 1 << A.MIBM_F_VX
        c.sync_from_host(lib, mask)
        c.step(lib, 2)
        c.sync_to_host(lib, ALL)
        outs.append(_snap(c))
        c.detach(lib)
    (fo, xo), (fg, xg) = outs
    for k in FIELDS_OUT:
        assert rel_l2(fg[k], fo[k]) <= 1e-10, k
    assert np.abs(xg - xo).max() <= 1e-11
