"""The remeshing hand-off on the GPU against the oracle (particle.f90:
119-160): the device trigger, the call of the host's remesher with the mesh
written to the registered arrays, the upload of the new topology (rebuilt
vertex->face lists, scatter plans, MLS weights), the primitive geometry and
update_tri_velocity -- then further steps on the new mesh.  The remesher is
the test stand-in of tests/helpers.py (a coarser icosphere in the same
arrays, the rest ghosts), installed on both libraries."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from melt_ibm_gb300 import abi
from melt_ibm_gb300.case import Case
from tests.helpers import FIELDS_OUT, CoarseningRemesher, pair, rel_l2, small_config

pytestmark = pytest.mark.gpu
A = abi
ALL = -1


def _run_pair(oracle_lib, gpu_lib, cfg, nsteps=2, precision=0):
    case = Case(cfg)
    case.set_S(A.MIBM_S_E_THRESH, 0.1)
    co, cg = pair(case, oracle_lib, gpu_lib)
    ro, rg = CoarseningRemesher(co, 2), CoarseningRemesher(cg, 2)
    ro.install(oracle_lib)
    rg.install(gpu_lib)
    if precision:
        cg.bind(gpu_lib)
        gpu_lib.mibm_set_precision_(C.byref(C.c_int(1)), C.byref(C.c_int(2)))
    co.run(oracle_lib, nsteps)
    cg.run(gpu_lib, nsteps)
    cg.sync_to_host(gpu_lib, ALL)
    return co, cg, ro, rg


@pytest.mark.parametrize("imlsstr", [0, 1])
def test_remesh_handoff_parity(oracle_lib, gpu_lib, imlsstr):
    co, cg, ro, rg = _run_pair(oracle_lib, gpu_lib, small_config(n=24, level=3, iremesh=1, imlsstr=imlsstr,
                                                                 dens_ratio=2.0))
    assert ro.calls == rg.calls == 1
    cg.bind(gpu_lib)
    assert gpu_lib.mibm_remesh_count_() == 1
    for name, fid in FIELDS_OUT.items():
        err = rel_l2(cg.interior(fid), co.interior(fid))
        assert err <= 1e-10, f"{name}: {err:.3e}"
    live_f = co.mesh_arrays[A.MIBM_M_GHOST_FACE] == 0
    live_e = co.mesh_arrays[A.MIBM_M_GHOST_EDGE] == 0
    live_v = co.mesh_arrays[A.MIBM_M_GHOST_VERT] == 0
    assert int(live_f.sum()) == 320
    for mid in (A.MIBM_M_GHOST_FACE, A.MIBM_M_GHOST_EDGE, A.MIBM_M_GHOST_VERT, A.MIBM_M_VERT_OF_FACE):
        assert np.array_equal(cg.mesh_arrays[mid], co.mesh_arrays[mid]), mid
    # a moving body's face velocities follow vel_CM and omega_c, which carry
    # the MLS noise of the loads (~1e-10 absolute): 1e-9 for them
    for mid, live in ((A.MIBM_M_XYZV, live_v), (A.MIBM_M_TRI_BAR, live_f), (A.MIBM_M_VEL_TRI, live_f)):
        a, b = cg.mesh_arrays[mid][:, live], co.mesh_arrays[mid][:, live]
        tol = 1e-9 if (imlsstr and mid == A.MIBM_M_VEL_TRI) else 1e-10
        assert np.abs(a - b).max() <= tol * max(1.0, np.abs(b).max()), mid
    for mid, live in ((A.MIBM_M_ELENGTHS, live_e), (A.MIBM_M_SKEWNESS, live_f)):
        a, b = cg.mesh_arrays[mid][live], co.mesh_arrays[mid][live]
        assert np.abs(a - b).max() <= 1e-10 * max(1.0, np.abs(b).max()), mid
    assert abs(cg.S(A.MIBM_S_VOLUME) - co.S(A.MIBM_S_VOLUME)) <= 1e-10 * co.S(A.MIBM_S_VOLUME)


def test_remesh_handoff_precision_form(oracle_lib, gpu_lib):
    co, cg, ro, rg = _run_pair(oracle_lib, gpu_lib, small_config(n=24, level=3, iremesh=1), precision=1)
    assert ro.calls == rg.calls == 1
    for name, fid in FIELDS_OUT.items():
        assert rel_l2(cg.interior(fid), co.interior(fid)) <= 1e-6, name


def test_remesh_trigger_without_remesher_stops(gpu_lib):
    c = Case(small_config(n=16, level=3, iremesh=1))
    c.set_S(A.MIBM_S_E_THRESH, 0.1)
    c.attach(gpu_lib)
    c.bind(gpu_lib)
    gpu_lib.tschem_()
    assert gpu_lib.mibm_last_status_() == A.MIBM_ESTATE
    assert b"remesh" in gpu_lib.mibm_last_message()
    c.detach(gpu_lib)


def test_library_remesher_parity(oracle_lib, gpu_lib):
    """A real remesh event with the library's remesher (remesh_coarsen +
    remesh_smooth as host code): a fixed, melting spheroid whose shortest
    edges (the lowest 1.5 %) sit below E_thresh from the start.  The GPU run
    uses the remesh callback mibm_remesh_builtin_; the oracle run hands its
    own arrays to the same host remesher (mibm_remesh_mesh).  The body does
    not move, so both hand the remesher the same mesh to round-off: the same
    topology comes back, the smoothed vertices agree to 1e-10 (the smoothing
    amplifies last-bit differences), and the fields agree at the plain-form
    tolerance after the steps that follow."""
    cfg = small_config(n=32, level=3, iremesh=1, rad_p=0.55, axes=(1.0, 0.75, 0.75), imlsstr=0)
    case = Case(cfg)
    x = case.mesh_arrays[A.MIBM_M_XYZV]
    e = case.mesh_arrays[A.MIBM_M_VERT_OF_EDGE] - 1
    el = np.sort(np.linalg.norm(x[:, e[0]] - x[:, e[1]], axis=0))
    case.set_S(A.MIBM_S_E_THRESH, float(el[int(0.015 * el.size)]))
    co, cg = pair(case, oracle_lib, gpu_lib)
    co.use_library_remesher(oracle_lib, remesher=gpu_lib)
    cg.use_library_remesher(gpu_lib)
    co.run(oracle_lib, 3)
    cg.run(gpu_lib, 3)
    cg.sync_to_host(gpu_lib, ALL)
    cg.bind(gpu_lib)
    n_gpu = gpu_lib.mibm_remesh_count_()
    stats = np.zeros(8)
    assert gpu_lib.mibm_remesh_stats_(stats.ctypes.data) == 0 and stats[0] + stats[1] >= 1
    co.bind(oracle_lib)
    assert n_gpu >= 1 and oracle_lib.mibm_remesh_count_() == n_gpu
    for mid in (A.MIBM_M_GHOST_FACE, A.MIBM_M_GHOST_EDGE, A.MIBM_M_GHOST_VERT, A.MIBM_M_VERT_OF_FACE,
                A.MIBM_M_EDGE_OF_FACE, A.MIBM_M_VERT_OF_EDGE):
        assert np.array_equal(cg.mesh_arrays[mid], co.mesh_arrays[mid]), mid
    live_v = co.mesh_arrays[A.MIBM_M_GHOST_VERT] == 0
    assert live_v.sum() < case.maxnv
    a, b = cg.mesh_arrays[A.MIBM_M_XYZV][:, live_v], co.mesh_arrays[A.MIBM_M_XYZV][:, live_v]
    assert np.abs(a - b).max() <= 1e-10
    for name, fid in FIELDS_OUT.items():
        err = rel_l2(cg.interior(fid), co.interior(fid))
        assert err <= 1e-10, f"{name}: {err:.3e}"
