"""Known-answer tests of the oracle's moving-body routines (the checker):
mls_structLoads (mls_structLoads.f90:1-1298) and update_part_pos /
newton_euler / update_xyz (RigidAuxRoutines.f90:1-306, 818-868).

Each test states a property of the reference's algorithm that holds in exact
arithmetic and checks the oracle against it to round-off:

* MLS with the linear basis reproduces linear fields, so for a pressure
  linear in x and y the probe value extrapolated back to the face is the
  face-centroid value, and the summed pressure force of a closed polyhedron
  is grad(p) * Volume (the face integral of a linear function is its centroid
  value times the area);
* for a velocity field linear in x and y the MLS gradients are the exact
  velocity gradient, so the viscous loads follow the reference's per-face
  formulas evaluated with that gradient;
* with no loads the translation is the buoyancy update along -z, and an
  isotropic inertia tensor makes the rotation a rigid turn by
  |omega| al dt about omega.

The z layers of the gradient cages repeat k1 (mls_structLoads.f90:459), so
exactness holds for fields without z-variation, as for wght_gradT.
"""
from __future__ import annotations

import numpy as np

from melt_ibm_gb300 import abi
from melt_ibm_gb300.case import Case
from tests.helpers import set_substep, small_config

A = abi


def _loads_case(oracle_lib, n=32, level=2, **kw):
    kw.setdefault("velocity", "rest")
    cfg = small_config(n=n, level=level, imelt=1, imlsstr=1, **kw)
    c = Case(cfg)
    return c


def _face_geometry(c):
    M = c.mesh_arrays
    return M[A.MIBM_M_TRI_BAR].T.copy(), M[A.MIBM_M_TRI_NOR].T.copy(), M[A.MIBM_M_SUR].copy()


def test_pressure_force_of_linear_pressure(oracle_lib):
    c = _loads_case(oracle_lib)
    a = np.array([0.37, -0.81, 0.0])
    X, Y, Z = np.meshgrid(c.xm, c.ym, c.zm, indexing="ij")
    P = c.fields[A.MIBM_F_PR]
    P[:c.n1m, :c.n2m, 1:c.n3m + 1] = 0.2 + a[0] * X + a[1] * Y
    c.fill_ghosts(A.MIBM_F_PR)
    c.attach(oracle_lib, initial_tag=False)
    oracle_lib.mls_structloads_()
    oracle_lib.check("mls_structloads")
    bar, nor, sur = _face_geometry(c)
    p_face = 0.2 + bar @ a
    prn = c.sc[A.MIBM_S_INT_PRN_DA, :3]
    expect = (p_face[:, None] * sur[:, None] * nor).sum(0)
    assert np.max(np.abs(prn - expect)) < 1e-8 * np.abs(a).max() * c.S(A.MIBM_S_VOLUME) + 1e-12
    # closed polyhedron: sum p(centroid) n A = grad(p) V
    assert np.max(np.abs(prn - a * c.S(A.MIBM_S_VOLUME))) < 1e-8
    rad = bar - c.sc[A.MIBM_S_POS_CM, :3]
    torque = (np.cross(rad, p_face[:, None] * nor) * sur[:, None]).sum(0)
    assert np.max(np.abs(c.sc[A.MIBM_S_INT_R_X_PRN_DA, :3] - torque)) < 1e-9
    # a fluid at rest has no viscous load
    assert np.max(np.abs(c.sc[A.MIBM_S_INT_TAU_DA, :3])) == 0.0
    # the running sums for output took the loads once
    assert np.array_equal(c.sc[A.MIBM_S_FP, :3], prn)


def test_viscous_loads_of_linear_velocity(oracle_lib):
    c = _loads_case(oracle_lib)
    G = np.array([[0.3, -0.5, 0.0], [0.7, -0.1, 0.0], [0.2, 0.4, 0.0]])   # du_i/dx_j, no z-variation
    F = c.fields
    Xc, Ym, Zm = np.meshgrid(c.xc, c.ym, c.zm, indexing="ij")
    Xm, Yc, _ = np.meshgrid(c.xm, c.yc, c.zm, indexing="ij")
    Xm2, Ym2, Zc = np.meshgrid(c.xm, c.ym, c.zc, indexing="ij")
    sl = (slice(0, c.n1m), slice(0, c.n2m), slice(1, c.n3m + 1))
    F[A.MIBM_F_VX][sl] = G[0, 0] * Xc + G[0, 1] * Ym
    F[A.MIBM_F_VY][sl] = G[1, 0] * Xm + G[1, 1] * Yc
    F[A.MIBM_F_VZ][sl] = G[2, 0] * Xm2 + G[2, 1] * Ym2
    for fid in (A.MIBM_F_VX, A.MIBM_F_VY, A.MIBM_F_VZ):
        c.fill_ghosts(fid)
    # loads of the previous substep move to the _m1 slots
    c.sc[A.MIBM_S_INT_TAU_DA, :3] = [1.0, 2.0, 3.0]
    c.attach(oracle_lib, initial_tag=False)
    oracle_lib.mls_structloads_()
    oracle_lib.check("mls_structloads")
    assert np.array_equal(c.sc[A.MIBM_S_INT_TAU_DA_M1, :3], [1.0, 2.0, 3.0])
    bar, nor, sur = _face_geometry(c)
    ren = c.S(A.MIBM_S_REN)
    S = G
    n1, n2, n3 = nor[:, 0], nor[:, 1], nor[:, 2]
    sr = sur / ren
    # (U, V) part then W part, mls_structLoads.f90:148-201
    t_uv = np.stack([sr * (2.0 * S[0, 0] * n1 + (S[0, 1] + S[1, 0]) * n2 + S[0, 2] * n3),
                     sr * ((S[1, 0] + S[0, 1]) * n1 + 2.0 * S[1, 1] * n2 + S[1, 2] * n3),
                     sr * (S[0, 2] * n1 + S[1, 2] * n2)], 1)
    t_w = np.stack([sr * (S[2, 0] * n3), sr * (S[2, 1] * n3),
                    sr * (S[2, 0] * n1 + S[2, 1] * n2 + 2.0 * S[2, 2] * n3)], 1)
    rad = bar - c.sc[A.MIBM_S_POS_CM, :3]
    tau = (t_uv + t_w).sum(0)
    rtau = (np.cross(rad, t_uv) + np.cross(rad, t_w)).sum(0)
    scale = np.abs(G).max() * sur.sum() / ren
    assert np.max(np.abs(c.sc[A.MIBM_S_INT_TAU_DA, :3] - tau)) < 1e-7 * scale
    assert np.max(np.abs(c.sc[A.MIBM_S_INT_R_X_TAU_DA, :3] - rtau)) < 1e-7 * scale
    # the viscous stress is symmetric, so the viscous force and torque on a
    # closed surface vanish with a constant gradient (up to the quadrature
    # of the torque)
    assert np.max(np.abs(tau)) < 1e-12 * scale * c.maxnf


def _rotation(axis, angle):
    k = axis / np.linalg.norm(axis)
    K = np.array([[0, -k[2], k[1]], [k[2], 0, -k[0]], [-k[1], k[0], 0]])
    return np.eye(3) + np.sin(angle) * K + (1 - np.cos(angle)) * (K @ K)


def test_newton_euler_buoyancy_and_rigid_turn(oracle_lib):
    c = _loads_case(oracle_lib, n=16, level=2, dens_ratio=2.0)
    set_substep(c, 1, dt=5e-3)
    I0 = 0.0523
    c.sc[A.MIBM_S_INERT_TENSOR, :9] = (I0 * np.eye(3)).ravel(order="F")
    vel1 = np.array([0.1, -0.05, 0.02])
    om1 = np.array([0.4, -0.3, 1.1])
    c.sc[A.MIBM_S_VEL_CM, :3] = vel1
    c.sc[A.MIBM_S_OMEGA_C, :3] = om1
    x_old = c.mesh_arrays[A.MIBM_M_XYZV].T.copy()
    bar_old = c.mesh_arrays[A.MIBM_M_TRI_BAR].T.copy()
    pos1 = c.sc[A.MIBM_S_POS_CM, :3].copy()
    c.attach(oracle_lib, initial_tag=False)
    oracle_lib.update_part_pos_()
    oracle_lib.check("update_part_pos")
    al, dt = c.S(A.MIBM_S_AL), c.S(A.MIBM_S_DT)
    vel = vel1 + al * dt * (1.0 - 1.0 / 2.0) * np.array([0.0, 0.0, -1.0])
    pos = pos1 + 0.5 * al * dt * (vel + vel1)
    assert np.max(np.abs(c.sc[A.MIBM_S_VEL_CM, :3] - vel)) < 1e-15
    assert np.max(np.abs(c.sc[A.MIBM_S_POS_CM, :3] - pos)) < 1e-14
    om = c.sc[A.MIBM_S_OMEGA_C, :3]
    assert np.max(np.abs(om - om1)) < 1e-13
    q = c.sc[A.MIBM_S_QUAT, :4]
    angle = np.linalg.norm(om1) * al * dt
    assert abs(np.linalg.norm(q) - 1.0) < 1e-15
    assert abs(q[0] - np.cos(0.5 * angle)) < 1e-14
    R = _rotation(om1, angle)
    x_new = c.mesh_arrays[A.MIBM_M_XYZV].T
    assert np.max(np.abs(x_new - (pos + (x_old - pos1) @ R.T))) < 1e-13
    vt = c.mesh_arrays[A.MIBM_M_VEL_TRI].T
    assert np.max(np.abs(vt - (vel + np.cross(om1, bar_old - pos1)))) < 1e-13
    # centroids follow the vertices
    f = c.mesh_arrays[A.MIBM_M_VERT_OF_FACE].T - 1
    assert np.max(np.abs(c.mesh_arrays[A.MIBM_M_TRI_BAR].T - x_new[f].mean(1))) < 1e-14


def test_newton_euler_angular_momentum(oracle_lib):
    """Anisotropic body, no loads: the iteration converges to I_rot omega =
    I omega_m1 with I_rot = AA I AA^T for the turn it implies."""
    c = _loads_case(oracle_lib, n=16, level=2)
    set_substep(c, 0, dt=2e-2)
    I = np.array([[0.05, 0.004, -0.002], [0.004, 0.08, 0.001], [-0.002, 0.001, 0.03]])
    c.sc[A.MIBM_S_INERT_TENSOR, :9] = I.ravel(order="F")
    om1 = np.array([2.0, -1.0, 3.0])
    c.sc[A.MIBM_S_OMEGA_C, :3] = om1
    c.attach(oracle_lib, initial_tag=False)
    oracle_lib.update_part_pos_()
    oracle_lib.check("update_part_pos")
    om = c.sc[A.MIBM_S_OMEGA_C, :3]
    I_rot = c.sc[A.MIBM_S_INERT_TENSOR, :9].reshape(3, 3, order="F")
    assert np.max(np.abs(I_rot @ om - I @ om1)) < 1e-14
    q = c.sc[A.MIBM_S_QUAT, :4]
    mid = 0.5 * (om + om1)
    angle = np.linalg.norm(mid) * c.S(A.MIBM_S_AL) * c.S(A.MIBM_S_DT)
    # the vertices turn by R = AA^T (update_xyz), while the tensor is
    # updated as AA I AA^T = R^T I R (RigidAuxRoutines.f90:287-288): the
    # reference's convention, kept
    R = _rotation(mid, angle)
    assert np.max(np.abs(I_rot - R.T @ I @ R)) < 1e-14
    assert abs(q[0] - np.cos(0.5 * angle)) < 1e-14
    assert not np.allclose(om, om1)
