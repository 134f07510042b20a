"""Continuation files: write a case's restart set and read it back.

Mirrors the reference's restart path, file for file and dataset for dataset:

* ``continua_grid.dat`` -- ``n1 n2 n3 time`` as text (mpi_routines.f90:1429-
  1435; read by inirea.f90:19-26).  n1, n2, n3 count grid points (cells + 1).
* ``continua_vx``, ``_vy``, ``_vz``, ``_pr``, ``_temp`` -- datasets ``Vx``,
  ``Vy``, ``Vz``, ``pr``, ``Temp`` of shape (n1, n2, n3m): the owned planes
  k = 1..n3m with the padding column and row (mpi_write_continua
  mpi_routines.f90:1223-1420; mpi_read_continua :1528-1620).
* ``continua_master`` -- ``Re``, ``Pr`` and the coordinates ``X_cordin`` (xc),
  ``Y_cordin`` (yc), ``Z_cordin`` (zm) (mpi_routines.f90:1441-1520).
* ``continua_bhat`` -- ``bhat_re``, ``bhat_im`` of shape (3, nm, nm, nm)
  (WriteRandForcCoef hit.f90:256-305; hdf_read_bhat :307-356).
* ``particles`` -- the rigid-body state and the surface mesh under the
  reference's dataset names (continua_particle create_geo.f90:280-407;
  import_particles :135-278), each with its trailing Nparticle = 1 axis.

HDF5 is not available to this package, so each ``.h5`` file of the reference
is a ``.npz`` archive of the same name holding the same datasets (same
names, shapes and element types, Fortran order).

Some datasets are additions, needed for a continued run to take exactly
the steps of the uninterrupted one (the reference restarts approximately: it
reseeds the forcing stream and restarts the Newton-Euler history):
``rng`` in ``continua_bhat`` (the position of the forcing increments' stream,
``mibm_hit_rng_``) and, in ``particles``, the surface velocity ``vel_tri``
(the forcing's target velocity of the first substep, which the reference
restarts at zero), the previous-substep loads ``int_*_dA_m1`` and the
accumulated loads ``Fp``, ``Ftau``, ``torq_p``, ``torq_tau``.  Without them
(a set written by the reference) the reader keeps the case's own values.

Reading follows inirea.f90: the same grid reads the five fields directly;
a different grid (at most twice the old points per direction, else the
reference aborts, inirea.f90:36-41) reads vx, vy, vz and temp into an old
array whose top plane is zeroed (inirea.f90:62-68) and regrids them with the
library's ``interp_`` (interp.f90), temperature with the vz staggering as
inirea.f90:121 passes it; the pressure is not read on that path.
"""
from __future__ import annotations

import os
from dataclasses import dataclass

import numpy as np

from . import abi
from .case import Case

A = abi

#: reference file stem -> (dataset name, field id, interp staggering)
FIELD_FILES = {
    "continua_vx": ("Vx", A.MIBM_F_VX, 1),
    "continua_vy": ("Vy", A.MIBM_F_VY, 2),
    "continua_vz": ("Vz", A.MIBM_F_VZ, 3),
    "continua_pr": ("pr", A.MIBM_F_PR, 4),
    "continua_temp": ("Temp", A.MIBM_F_TEMP, 3),     # inirea.f90:121 passes 3
}

#: particles dataset -> (scalar id, shape without the Nparticle axis)
PARTICLE_SCALARS = {
    "pos_CM": (A.MIBM_S_POS_CM, (3,)),
    "vel_CM": (A.MIBM_S_VEL_CM, (3,)),
    "omega_c": (A.MIBM_S_OMEGA_C, (3,)),
    "quat": (A.MIBM_S_QUAT, (4,)),
    "int_prn_dA": (A.MIBM_S_INT_PRN_DA, (3,)),
    "int_tau_dA": (A.MIBM_S_INT_TAU_DA, (3,)),
    "int_r_x_prn_dA": (A.MIBM_S_INT_R_X_PRN_DA, (3,)),
    "int_r_x_tau_dA": (A.MIBM_S_INT_R_X_TAU_DA, (3,)),
    "InertTensor": (A.MIBM_S_INERT_TENSOR, (3, 3)),
    "volume": (A.MIBM_S_VOLUME, ()),
    "total_area": (A.MIBM_S_SURFACE, ()),
}
#: additions for an exact continuation (not in the reference's particles.h5)
PARTICLE_SCALARS_EXACT = {
    "int_prn_dA_m1": (A.MIBM_S_INT_PRN_DA_M1, (3,)),
    "int_tau_dA_m1": (A.MIBM_S_INT_TAU_DA_M1, (3,)),
    "int_r_x_prn_dA_m1": (A.MIBM_S_INT_R_X_PRN_DA_M1, (3,)),
    "int_r_x_tau_dA_m1": (A.MIBM_S_INT_R_X_TAU_DA_M1, (3,)),
    "Fp": (A.MIBM_S_FP, (3,)),
    "Ftau": (A.MIBM_S_FTAU, (3,)),
    "torq_p": (A.MIBM_S_TORQ_P, (3,)),
    "torq_tau": (A.MIBM_S_TORQ_TAU, (3,)),
}
#: particles dataset -> mesh array id (create_geo.f90:337-400)
PARTICLE_MESH = {
    "vert_of_edge": A.MIBM_M_VERT_OF_EDGE,
    "isGhostEdge": A.MIBM_M_GHOST_EDGE,
    "eLengths": A.MIBM_M_ELENGTHS,
    "vert_of_face": A.MIBM_M_VERT_OF_FACE,
    "edge_of_face": A.MIBM_M_EDGE_OF_FACE,
    "isGhostFace": A.MIBM_M_GHOST_FACE,
    "tri_bar": A.MIBM_M_TRI_BAR,
    "tri_nor": A.MIBM_M_TRI_NOR,
    "Atri": A.MIBM_M_SUR,
    "skewness": A.MIBM_M_SKEWNESS,
    "isGhostVert": A.MIBM_M_GHOST_VERT,
    "xyzv": A.MIBM_M_XYZV,
    "vert_nor": A.MIBM_M_VERT_NOR,
    "Avert": A.MIBM_M_AVERT,
}
#: addition for an exact continuation
PARTICLE_MESH_EXACT = {"vel_tri": A.MIBM_M_VEL_TRI}


@dataclass
class ForcingState:
    """bhat (complex, (3, nm, nm, nm)) and the increments' stream position."""
    bhat: np.ndarray
    rng: int

    def apply(self, case: Case, lib: abi.Lib) -> None:
        """Install into the case's context on ``lib`` (after ``attach``)."""
        case.bind(lib)
        buf = np.empty(2 * self.bhat.size)
        flat = self.bhat.ravel(order="F")
        buf[0::2], buf[1::2] = flat.real, flat.imag
        lib.mibm_hit_bhat_(buf.ctypes.data, abi.ref_int(1))
        state = np.array([self.rng], dtype=np.uint64)
        lib.mibm_hit_rng_(state.ctypes.data, abi.ref_int(1))
        lib.check("continuation forcing state")


def _path(directory: str, stem: str) -> str:
    return os.path.join(directory, stem + ".npz")


def write_continuation(case: Case, lib: abi.Lib, directory: str) -> None:
    """Write the restart set of ``case`` (attached to ``lib``) into ``directory``.

    The device state is copied to the registered host arrays first (the
    reference writes from its host arrays at the end of the run, quit /
    gcurv.f90:245-251)."""
    os.makedirs(directory, exist_ok=True)
    case.sync_to_host(lib, -1)
    n1, n2, n3 = case.n1m + 1, case.n2m + 1, case.n3m + 1
    with open(os.path.join(directory, "continua_grid.dat"), "w") as f:
        f.write(f" {n1:12d} {n2:12d} {n3:12d} {case.S(A.MIBM_S_TIME)!r}\n")
    for stem, (name, fid, _) in FIELD_FILES.items():
        a = case.fields[fid]
        k0 = 1 if a.shape[2] == case.n3m + 2 else 0
        np.savez(_path(directory, stem), **{name: np.asfortranarray(a[:n1, :n2, k0:k0 + case.n3m])})
    np.savez(_path(directory, "continua_master"), Re=np.array([case.S(A.MIBM_S_REN)]),
             Pr=np.array([case.S(A.MIBM_S_PEC) / case.S(A.MIBM_S_REN)]),
             X_cordin=np.append(case.xc, case.xlen), Y_cordin=np.append(case.yc, case.ylen),
             Z_cordin=case.zm.copy())
    case.bind(lib)
    nm = int(lib.mibm_hit_modes_())
    buf = np.zeros(6 * nm ** 3)
    lib.mibm_hit_bhat_(buf.ctypes.data, abi.ref_int(0))
    state = np.zeros(1, dtype=np.uint64)
    lib.mibm_hit_rng_(state.ctypes.data, abi.ref_int(0))
    lib.check("continuation forcing state")
    bh = (buf[0::2] + 1j * buf[1::2]).reshape((3, nm, nm, nm), order="F")
    np.savez(_path(directory, "continua_bhat"), bhat_re=np.asfortranarray(bh.real),
             bhat_im=np.asfortranarray(bh.imag), rng=state)
    part = {}
    for name, (sid, shape) in {**PARTICLE_SCALARS, **PARTICLE_SCALARS_EXACT}.items():
        size = int(np.prod(shape)) if shape else 1
        v = case.sc[sid, :size].reshape(shape + (1,), order="F") if shape else case.sc[sid, :1].copy()
        part[name] = np.asfortranarray(v)
    for name, mid in {**PARTICLE_MESH, **PARTICLE_MESH_EXACT}.items():
        m = case.mesh_arrays[mid]
        part[name] = np.asfortranarray(m.reshape(m.shape + (1,), order="F"))
    np.savez(_path(directory, "particles"), **part)


def read_grid(directory: str) -> tuple[int, int, int, float]:
    """(n1, n2, n3, time) of continua_grid.dat (inirea.f90:19-26)."""
    with open(os.path.join(directory, "continua_grid.dat")) as f:
        tok = f.read().split()
    return int(tok[0]), int(tok[1]), int(tok[2]), float(tok[3])


def read_continuation(case: Case, directory: str, lib: abi.Lib | None = None) -> ForcingState:
    """Load the restart set in ``directory`` into the host arrays of ``case``
    (not yet attached), as inirea.f90 + import_particles + hdf_read_bhat do.

    A different grid is regridded through ``lib.interp_`` (a temporary
    context of ``case`` on ``lib``), so ``lib`` is needed then.  Returns the
    forcing state; install it with ``ForcingState.apply`` after ``attach``."""
    if case.ctx:
        raise ValueError("read_continuation loads host arrays before Case.attach")
    n1o, n2o, n3o, time = read_grid(directory)
    n1, n2, n3 = case.n1m + 1, case.n2m + 1, case.n3m + 1
    case.set_S(A.MIBM_S_TIME, time)
    same = (n1o, n2o, n3o) == (n1, n2, n3)
    if same:                                                    # inirea.f90:131-137
        for stem, (name, fid, _) in FIELD_FILES.items():
            with np.load(_path(directory, stem)) as z:
                data = z[name]
            if data.shape != (n1, n2, case.n3m):
                raise ValueError(f"{stem}: dataset {name} has shape {data.shape}")
            case.fields[fid][:n1, :n2, 1:case.n3m + 1] = data
            case.fill_ghosts(fid)
    else:
        if n1 > 2 * n1o or n2 > 2 * n2o or n3 > 2 * n3o:      # inirea.f90:36-41
            raise ValueError("new grid resolution can not be more than twice the old resolution")
        if lib is None:
            raise ValueError("a different grid is regridded by interp_: pass the library")
        case.attach(lib, initial_tag=False)
        try:
            for stem, (name, fid, intvar) in FIELD_FILES.items():
                if fid == A.MIBM_F_PR:
                    continue                                     # not read when regridding
                with np.load(_path(directory, stem)) as z:
                    data = z[name]
                old = np.zeros((n1o, n2o, n3o + 1), order="F")   # planes 0..n3o
                old[:, :, 1:n3o] = data                          # mpi_read_continua planes 1..n3o-1
                old[:, :, n3o] = 0.0                             # inirea.f90:62-68
                new = np.zeros((n1, n2, case.n3m), order="F")
                ints = [abi.ref_int(v) for v in (n1o, n2o, n3o, intvar, 1, n3o - 1)]
                case.bind(lib)
                lib.interp_(old.ctypes.data, new.ctypes.data, *ints)
                lib.check("interp")
                case.fields[fid][:n1, :n2, 1:case.n3m + 1] = new
                case.fill_ghosts(fid)
        finally:
            case.detach(lib)
    with np.load(_path(directory, "particles")) as z:
        for name, (sid, shape) in {**PARTICLE_SCALARS, **PARTICLE_SCALARS_EXACT}.items():
            if name not in z:
                continue                               # a reference-written set lacks the additions
            v = np.asarray(z[name], dtype=np.float64).ravel(order="F")
            case.sc[sid, :v.size] = v
        for name, mid in {**PARTICLE_MESH, **PARTICLE_MESH_EXACT}.items():
            if name not in z:
                continue
            m = case.mesh_arrays[mid]
            v = z[name]
            if v.size != m.size:
                raise ValueError(f"particles: {name} has {v.size} entries, the case's mesh {m.size}")
            m[...] = v.reshape(m.shape, order="F")
    h, cv = case.S(A.MIBM_S_H_EULERIAN), case.S(A.MIBM_S_CELVOL)
    case.mesh_arrays[A.MIBM_M_CFAC][...] = (case.mesh_arrays[A.MIBM_M_SUR] * h) / cv   # initmls.f90:25
    with np.load(_path(directory, "continua_bhat")) as z:
        bhat = np.asfortranarray(z["bhat_re"] + 1j * z["bhat_im"])
        rng = int(z["rng"][0]) if "rng" in z else int(case.iv[A.MIBM_I_HIT_SEED])
    return ForcingState(bhat=bhat, rng=rng)
