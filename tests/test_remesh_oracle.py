"""The remeshing hand-off in the oracle (particle.f90:119-160): the trigger
(calculate_eLengths against E_thresh), the call of the host's remesher on the
registered arrays, the primitive geometry of the new mesh (edge lengths and
skewness included, triaux.f90:277-358) and update_tri_velocity.  The
remesher here is the test stand-in of tests/helpers.py (a coarser icosphere
in the same arrays, the rest ghosts)."""
from __future__ import annotations

import numpy as np

from melt_ibm_gb300 import abi
from melt_ibm_gb300.case import Case
from tests.helpers import CoarseningRemesher, small_config

A = abi


def test_remesh_handoff(oracle_lib):
    c = Case(small_config(n=24, level=3, iremesh=1))
    c.set_S(A.MIBM_S_E_THRESH, 0.1)          # level-3 edges (0.069-0.082) trigger, level-2 (0.14-0.16) do not
    r = CoarseningRemesher(c, 2)
    c.attach(oracle_lib)
    r.install(oracle_lib)
    c.run(oracle_lib, 2)
    assert r.calls == 1 and oracle_lib.mibm_remesh_count_() == 1
    M = c.mesh_arrays
    assert int((M[A.MIBM_M_GHOST_FACE] == 0).sum()) == 320
    x = M[A.MIBM_M_XYZV].T
    e = M[A.MIBM_M_VERT_OF_EDGE].T[:480] - 1
    el = np.linalg.norm(x[e[:, 0]] - x[e[:, 1]], axis=1)
    np.testing.assert_allclose(M[A.MIBM_M_ELENGTHS][:480], el, rtol=1e-14)
    eof = M[A.MIBM_M_EDGE_OF_FACE].T[:320] - 1
    perim = el[eof].sum(1)
    opt = np.sqrt(3.0) / 4.0 * (perim / 3.0) ** 2
    np.testing.assert_allclose(M[A.MIBM_M_SKEWNESS][:320], (opt - M[A.MIBM_M_SUR][:320]) / opt, atol=1e-13)
    # the coarse body is a level-2 icosphere of radius ~0.5
    assert abs(c.S(A.MIBM_S_VOLUME) / (4 / 3 * np.pi * 0.125) - 1) < 0.05
    # fixed body: update_tri_velocity keeps the live faces at rest
    assert np.all(M[A.MIBM_M_VEL_TRI][:, :320] == 0.0)


def test_remesh_trigger_without_remesher_stops(oracle_lib):
    c = Case(small_config(n=16, level=3, iremesh=1))
    c.set_S(A.MIBM_S_E_THRESH, 0.1)
    c.attach(oracle_lib)
    c.bind(oracle_lib)
    oracle_lib.tschem_()
    assert oracle_lib.mibm_last_status_() == A.MIBM_ESTATE
    assert b"remesh" in oracle_lib.mibm_last_message()


def test_no_trigger_no_call(oracle_lib):
    c = Case(small_config(n=16, level=3, iremesh=1))
    c.set_S(A.MIBM_S_E_THRESH, 0.01)
    r = CoarseningRemesher(c, 2)
    c.attach(oracle_lib)
    r.install(oracle_lib)
    c.run(oracle_lib, 1)
    assert r.calls == 0
