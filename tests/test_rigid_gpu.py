"""Parity of the moving body (imlsstr = 1) on the GPU against the oracle:
mls_structLoads (mls_structLoads.f90:1-1298), update_part_pos / newton_euler
/ update_xyz (RigidAuxRoutines.f90:1-306, 818-868), and full RK3 steps with
a freely moving, melting body in both forms.

Tolerances: the reference's probe MLS builds its 4x4 moment matrix in
absolute coordinates (condition number ~1e8), which turns any last-bit
difference of its inputs into ~1e-8 relative per face.  The drop-in
mls_structloads_ of the plain form evaluates that construction in the
oracle's operation order with the shared written-out exp: per-face values
agree bit for bit, and the loads differ only by the order of the sum over
faces (compared against the sum of the magnitudes they add up, 1e-12).
Inside the step of a moving body the geometry carries the fluid solver's
round-off after the first step, so the library uses the separable
construction there, and the loads agree with the oracle's to its noise
(1e-7 of their size in the step comparisons).  The Newton-Euler update
itself is a few hundred FP64 operations in the oracle's order: 1e-12.  Full
steps keep the plain-form bound of 1e-10 (rel L2) on u, v, w, T, p; the
rigid state of a moving body is bounded by that MLS noise (~1e-10 absolute
after a few steps whichever side computes it): 1e-9 of max(1, |x|).  The step
comparisons use the density ratio 2: at 1.5 the reference's loosely coupled
update is itself unstable and amplifies round-off by ~1.1 per substep.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from melt_ibm_gb300 import abi
from melt_ibm_gb300.case import Case
from tests.helpers import FIELDS_OUT, pair, randomize, rel_l2, set_substep, small_config

pytestmark = pytest.mark.gpu
A = abi
ALL = -1
LOADS = (A.MIBM_S_INT_PRN_DA, A.MIBM_S_INT_TAU_DA, A.MIBM_S_INT_R_X_PRN_DA, A.MIBM_S_INT_R_X_TAU_DA)
LOADS_M1 = (A.MIBM_S_INT_PRN_DA_M1, A.MIBM_S_INT_TAU_DA_M1, A.MIBM_S_INT_R_X_PRN_DA_M1, A.MIBM_S_INT_R_X_TAU_DA_M1)
RIGID = (A.MIBM_S_VEL_CM, A.MIBM_S_OMEGA_C, A.MIBM_S_POS_CM)


def _cfg(n=24, level=2, **kw):
    kw.setdefault("imelt", 1)
    kw.setdefault("dens_ratio", 2.0)
    return small_config(n=n, level=level, imlsstr=1, **kw)


def _load_scales(case):
    """Sum of the magnitudes each load adds up (pressure, viscous; force, torque)."""
    sur = case.mesh_arrays[A.MIBM_M_SUR].sum()
    pmax = np.abs(case.interior(A.MIBM_F_PR)).max()
    umax = max(np.abs(case.interior(f)).max() for f in (A.MIBM_F_VX, A.MIBM_F_VY, A.MIBM_F_VZ))
    grad = 4.0 * umax * case.dx1
    r = case.cfg.rad_p * 1.5
    return {A.MIBM_S_INT_PRN_DA: pmax * sur, A.MIBM_S_INT_TAU_DA: 4 * grad * sur / case.cfg.ren,
            A.MIBM_S_INT_R_X_PRN_DA: r * pmax * sur, A.MIBM_S_INT_R_X_TAU_DA: 4 * r * grad * sur / case.cfg.ren}


def test_structloads_parity(oracle_lib, gpu_lib):
    case = Case(_cfg(n=32, level=3))
    randomize(case, forcing=False)
    case.sc[A.MIBM_S_INT_PRN_DA, :3] = [0.5, -0.25, 0.125]      # moves to the _m1 slot
    case.sc[A.MIBM_S_FP, :3] = [1.0, 2.0, 3.0]
    co, cg = pair(case, oracle_lib, gpu_lib, initial_tag=False)
    for c, lib in ((co, oracle_lib), (cg, gpu_lib)):
        c.bind(lib)
        lib.mls_structloads_()
        lib.check("mls_structloads")
    scales = _load_scales(co)
    for sid in LOADS:
        err = np.abs(cg.sc[sid, :3] - co.sc[sid, :3]).max()
        assert err <= 1e-12 * scales[sid], (sid, err, co.sc[sid, :3])
        assert np.abs(co.sc[sid, :3]).max() > 1e-6 * scales[sid]           # a real signal
    for sid in LOADS_M1:
        assert np.array_equal(cg.sc[sid, :3], co.sc[sid, :3])
    np.testing.assert_allclose(cg.sc[A.MIBM_S_FP, :3], co.sc[A.MIBM_S_FP, :3],
                               atol=1e-12 * scales[A.MIBM_S_INT_PRN_DA])


@pytest.mark.parametrize("ns", [0, 1, 2])
def test_update_part_pos_parity(oracle_lib, gpu_lib, ns):
    case = Case(_cfg(n=16, level=2))
    set_substep(case, ns, dt=1e-2)
    rng = np.random.default_rng(11 + ns)
    for sid in LOADS + LOADS_M1:
        case.sc[sid, :3] = rng.standard_normal(3) * 0.3
    case.sc[A.MIBM_S_VEL_CM, :3] = rng.standard_normal(3) * 0.2
    case.sc[A.MIBM_S_OMEGA_C, :3] = rng.standard_normal(3) * 2.0
    Q = np.linalg.qr(rng.standard_normal((3, 3)))[0]
    I = Q @ np.diag([0.05, 0.07, 0.031]) @ Q.T
    case.sc[A.MIBM_S_INERT_TENSOR, :9] = I.ravel(order="F")
    co, cg = pair(case, oracle_lib, gpu_lib, initial_tag=False)
    for c, lib in ((co, oracle_lib), (cg, gpu_lib)):
        c.bind(lib)
        lib.update_part_pos_()
        lib.check("update_part_pos")
    cg.sync_to_host(gpu_lib, ALL)
    for sid, w in ((A.MIBM_S_VEL_CM, 3), (A.MIBM_S_OMEGA_C, 3), (A.MIBM_S_POS_CM, 3), (A.MIBM_S_QUAT, 4),
                   (A.MIBM_S_INERT_TENSOR, 9)):
        a, b = cg.sc[sid, :w], co.sc[sid, :w]
        assert np.abs(a - b).max() <= 1e-12 * max(1.0, np.abs(b).max()), (sid, a, b)
    for mid in (A.MIBM_M_XYZV, A.MIBM_M_TRI_BAR, A.MIBM_M_VEL_TRI):
        assert np.abs(cg.mesh_arrays[mid] - co.mesh_arrays[mid]).max() <= 1e-12, mid
    assert not np.allclose(co.sc[A.MIBM_S_QUAT, :4], 0.0)


def _steps(case, lib, nsteps, start=1):
    case.run(lib, nsteps, start=start)
    if "libmibm" in lib.path:
        case.sync_to_host(lib, ALL)


def _cmp_rigid(co, cg, tol):
    for sid in RIGID:
        a, b = cg.sc[sid, :3], co.sc[sid, :3]
        assert np.abs(a - b).max() <= tol * max(1.0, np.abs(b).max()), (sid, a, b)
    for sid in LOADS:
        a, b = cg.sc[sid, :3], co.sc[sid, :3]
        assert np.abs(a - b).max() <= 1e3 * tol * max(1.0, np.abs(b).max()), (sid, a, b)


@pytest.mark.parametrize("imelt", [1, 0])
def test_moving_body_step_parity(oracle_lib, gpu_lib, imelt):
    """Plain FP64 form, 1 and 4 steps: a melting (or solid) body sinking and
    turning under the fluid loads."""
    case = Case(_cfg(n=24, level=2, imelt=imelt))
    co, cg = pair(case, oracle_lib, gpu_lib)
    for nsteps, start in ((1, 1), (3, 2)):
        _steps(co, oracle_lib, nsteps, start)
        _steps(cg, gpu_lib, nsteps, start)
        for name, fid in FIELDS_OUT.items():
            err = rel_l2(cg.interior(fid), co.interior(fid))
            assert err <= 1e-10, f"{name} after {start + nsteps - 1} steps: {err:.3e}"
        _cmp_rigid(co, cg, 1e-9)
        # vertex positions follow vel_CM / omega_c, which agree to ~1e-10
        assert rel_l2(cg.mesh_arrays[A.MIBM_M_XYZV], co.mesh_arrays[A.MIBM_M_XYZV]) <= 1e-11
    # the body did move
    assert np.abs(co.sc[A.MIBM_S_VEL_CM, :3]).max() > 1e-4


def test_free_body_forced_ten_steps(oracle_lib, gpu_lib):
    """The free-body configuration's physics (free melting body, density
    ratio 2, linear forcing) at 24^3: rel L2 <= 1e-10 on u, v, w, T, p after
    1 and 10 steps, the rigid state alike."""
    case = Case(_cfg(n=24, level=2, dens_ratio=2.0, forcing=1, which_hit=3, c_hit=0.2, ren=200.0))
    co, cg = pair(case, oracle_lib, gpu_lib)
    for nsteps, start in ((1, 1), (9, 2)):
        _steps(co, oracle_lib, nsteps, start)
        _steps(cg, gpu_lib, nsteps, start)
        for name, fid in FIELDS_OUT.items():
            err = rel_l2(cg.interior(fid), co.interior(fid))
            assert err <= 1e-10, f"{name} after {start + nsteps - 1} steps: {err:.3e}"
        _cmp_rigid(co, cg, 1e-9)


def test_moving_body_precision_form(oracle_lib, gpu_lib):
    case = Case(_cfg(n=24, level=2))
    co, cg = pair(case, oracle_lib, gpu_lib)
    cg.bind(gpu_lib)
    gpu_lib.mibm_set_precision_(C.byref(C.c_int(1)), C.byref(C.c_int(2)))
    gpu_lib.check("precision")
    _steps(co, oracle_lib, 3)
    _steps(cg, gpu_lib, 3)
    for name, fid in FIELDS_OUT.items():
        err = rel_l2(cg.interior(fid), co.interior(fid))
        assert err <= 1e-6, f"{name}: {err:.3e}"
    for sid in RIGID:
        assert np.abs(cg.sc[sid, :3] - co.sc[sid, :3]).max() <= 1e-6 * max(1.0, np.abs(co.sc[sid, :3]).max())


@pytest.mark.parametrize("precision", [0, 1])
def test_moving_body_graph_replay_is_bitwise_identical(gpu_lib, precision):
    case = Case(_cfg(n=32, level=3))
    runs = []
    for graphs in (0, 1):
        c = case.clone()
        c.attach(gpu_lib)
        c.bind(gpu_lib)
        gpu_lib.mibm_set_graphs_(C.byref(C.c_int(graphs)))
        gpu_lib.mibm_set_precision_(C.byref(C.c_int(precision)), C.byref(C.c_int(2)))
        gpu_lib.check("setup")
        c.run(gpu_lib, 4)
        c.sync_to_host(gpu_lib, ALL)
        runs.append(({k: c.interior(f).copy() for k, f in FIELDS_OUT.items()},
                     c.mesh_arrays[A.MIBM_M_XYZV].copy(), c.sc.copy()))
        c.detach(gpu_lib)
    (f0, x0, s0), (f1, x1, s1) = runs
    for k in FIELDS_OUT:
        assert np.array_equal(f0[k], f1[k]), k
    assert np.array_equal(x0, x1)
    assert np.array_equal(s0, s1)
