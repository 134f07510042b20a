"""Test helpers: seeded cases, paired oracle/GPU runs, error norms."""
from __future__ import annotations

import ctypes as C

import numpy as np

from melt_ibm_gb300 import abi
from melt_ibm_gb300.case import Case, CaseConfig

FIELDS_OUT = {"vx": abi.MIBM_F_VX, "vy": abi.MIBM_F_VY, "vz": abi.MIBM_F_VZ,
              "temp": abi.MIBM_F_TEMP, "pr": abi.MIBM_F_PR}


def rel_l2(a: np.ndarray, b: np.ndarray) -> float:
    den = float(np.sqrt(np.sum(b * b)))
    num = float(np.sqrt(np.sum((a - b) ** 2)))
    return num / den if den > 0 else num


def small_config(n=16, level=2, **kw) -> CaseConfig:
    base = dict(n=n, mesh_level=level, rad_p=0.5 * (2 * np.pi) / 2 / np.pi * 1.0, v_on_ve=0.0, seed=3)
    base.update(kw)
    return CaseConfig(**base)


def randomize(case: Case, seed: int = 7, forcing: bool = True) -> None:
    """Fill the state a routine reads with seeded noise (test inputs only)."""
    rng = np.random.default_rng(seed)
    A = abi
    for fid in (A.MIBM_F_VX, A.MIBM_F_VY, A.MIBM_F_VZ):     # not divergence-free
        case.fields[fid][...] += 0.1 * rng.standard_normal(case.fields[fid].shape)
    for fid in (A.MIBM_F_PR, A.MIBM_F_RU1, A.MIBM_F_RU2, A.MIBM_F_RU3, A.MIBM_F_RUT,
                A.MIBM_F_DQ, A.MIBM_F_QCAP, A.MIBM_F_HTEMP):
        case.fields[fid][...] = rng.standard_normal(case.fields[fid].shape)
    case.fields[A.MIBM_F_DPH][...] = rng.standard_normal(case.fields[A.MIBM_F_DPH].shape)
    if forcing:
        for fid in (A.MIBM_F_FORCX, A.MIBM_F_FORCY, A.MIBM_F_FORCZ):
            case.fields[fid][...] = rng.standard_normal(case.fields[fid].shape)
        case.iv[A.MIBM_I_FORCING] = 1
    for fid in (A.MIBM_F_VOFX, A.MIBM_F_VOFY, A.MIBM_F_VOFZ, A.MIBM_F_VOFP):
        v = rng.uniform(0, 1, case.fields[fid].shape)
        v[rng.uniform(0, 1, v.shape) < 0.5] = 1.0
        case.fields[fid][...] = v
    for fid in (A.MIBM_F_VX, A.MIBM_F_VY, A.MIBM_F_VZ, A.MIBM_F_TEMP, A.MIBM_F_PR, A.MIBM_F_DPH,
                A.MIBM_F_VOFP, A.MIBM_F_VOFX, A.MIBM_F_VOFY, A.MIBM_F_VOFZ,
                A.MIBM_F_FORCX, A.MIBM_F_FORCY, A.MIBM_F_FORCZ):
        case.fill_ghosts(fid)
    case.set_S(A.MIBM_S_BETAGZ, 0.3)
    case.sc[A.MIBM_S_VEL_CM, :3] = [0.1, -0.2, 0.05]
    case.sc[A.MIBM_S_OMEGA_C, :3] = [0.3, 0.1, -0.4]
    case.sc[A.MIBM_S_POS_CM, :3] += [0.01, -0.02, 0.03]
    set_substep(case, 1)


def set_substep(case: Case, ns: int, dt: float = 4e-3) -> None:
    gam = [8 / 15, 5 / 12, 3 / 4]
    rom = [0.0, -17 / 60, -5 / 12]
    A = abi
    case.set_S(A.MIBM_S_DT, dt)
    case.set_S(A.MIBM_S_BETA, dt / case.S(A.MIBM_S_REN) * 0.5)
    case.set_S(A.MIBM_S_AL, gam[ns] + rom[ns])
    case.set_S(A.MIBM_S_GA, gam[ns])
    case.set_S(A.MIBM_S_RO, rom[ns])


def pair(case: Case, oracle_lib, gpu_lib, initial_tag: bool = True):
    """Two independent copies of `case`, one per library."""
    co, cg = case.clone(), case.clone()
    co.attach(oracle_lib, initial_tag=initial_tag)
    cg.attach(gpu_lib, initial_tag=initial_tag)
    return co, cg


def elength_range(mesh, scale):
    """Shortest and longest edge of `mesh` scaled by `scale`."""
    e = mesh.vert_of_edge - 1
    d = np.linalg.norm(mesh.xyz[e[:, 0]] - mesh.xyz[e[:, 1]], axis=1) * scale
    return float(d.min()), float(d.max())


class CoarseningRemesher:
    """A stand-in for the host's remesher in tests: it replaces the live mesh
    by an icosphere of a coarser level, scaled to the body's mean radius and
    centred on its vertex mean, in the same (larger) arrays -- the unused
    vertices, edges and faces become ghosts, as after the reference's edge
    collapses.  The melt velocities are reset.  A topology change as drastic
    as a remesh can make, with a known result."""

    def __init__(self, case, level):
        from melt_ibm_gb300.mesh import icosphere
        self.case, self.mesh, self.calls = case, icosphere(level), 0
        self.fn = abi.REMESH_FN(self._call)

    def _call(self, user):
        A, M, m = abi, self.case.mesh_arrays, self.mesh
        live = M[A.MIBM_M_GHOST_VERT] == 0
        x = M[A.MIBM_M_XYZV][:, live].T
        centre = x.mean(0)
        radius = float(np.linalg.norm(x - centre, axis=1).mean())
        nv, ne, nf = m.nv, m.ne, m.nf
        M[A.MIBM_M_XYZV][:, :nv] = (m.xyz * radius + centre).T
        M[A.MIBM_M_VERT_OF_FACE][:, :nf] = m.vert_of_face.T
        M[A.MIBM_M_VERT_OF_FACE][:, nf:] = 1
        M[A.MIBM_M_EDGE_OF_FACE][:, :nf] = m.edge_of_face.T
        M[A.MIBM_M_EDGE_OF_FACE][:, nf:] = 1
        M[A.MIBM_M_VERT_OF_EDGE][:, :ne] = m.vert_of_edge.T
        M[A.MIBM_M_VERT_OF_EDGE][:, ne:] = 1
        for mid, n in ((A.MIBM_M_GHOST_VERT, nv), (A.MIBM_M_GHOST_EDGE, ne), (A.MIBM_M_GHOST_FACE, nf)):
            M[mid][:n] = 0
            M[mid][n:] = 1
        M[A.MIBM_M_VMELT][...] = 0.0
        M[A.MIBM_M_VMELT_M1][...] = 0.0
        self.calls += 1
        return 0

    def install(self, lib):
        self.case.bind(lib)
        lib.mibm_set_remesh_callback_(C.cast(self.fn, C.c_void_p), None)
