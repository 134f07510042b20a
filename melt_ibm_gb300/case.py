"""Host-side case: the Fortran module state that the C-ABI borrows.

A :class:`Case` owns numpy arrays laid out exactly like the reference's
Fortran allocations (column-major, ghost planes, padding column/row;
init.f90:15-83, allotri.f90:1-88) plus the scalars of ``param`` /
``mls_param``.  :meth:`Case.attach` registers them with a library that
exports the mibm C-ABI, which is what a thin ``bind(C)`` Fortran shim does
for the reference host program.  :meth:`Case.step` replays one iteration of
the reference time loop (gcurv.f90:147-172): ``cfl`` -> ``get_dt`` ->
``tschem``.

Set-up follows the reference's initialisation: ``cordin`` (grid),
``tri_geo`` -> ``setup_particles`` / ``init_geomCoords`` / geometry
(tri_geo.f90:19-38, create_geo.f90:1-104), ``init_mlsForce`` (initmls.f90),
initial full tagging (tagCells with initial_tag, gcurv.f90:61-63), and an
initial condition (seeded random-phase velocity, tanh temperature around the
body as in inqpr.f90:18-28).
"""
from __future__ import annotations

import copy
from dataclasses import dataclass, field

import numpy as np

from . import abi
from .fields import random_velocity, tanh_temperature
from .mesh import Mesh, icosphere

GHOSTED = {abi.MIBM_F_VX, abi.MIBM_F_VY, abi.MIBM_F_VZ, abi.MIBM_F_TEMP, abi.MIBM_F_PR,
           abi.MIBM_F_FORCX, abi.MIBM_F_FORCY, abi.MIBM_F_FORCZ,
           abi.MIBM_F_VOFX, abi.MIBM_F_VOFY, abi.MIBM_F_VOFZ, abi.MIBM_F_VOFP,
           abi.MIBM_F_FORXC, abi.MIBM_F_FORYC, abi.MIBM_F_FORZC, abi.MIBM_F_FORTEMP}
VECTOR_SCALARS = {abi.MIBM_S_POS_CM, abi.MIBM_S_VEL_CM, abi.MIBM_S_OMEGA_C, abi.MIBM_S_QUAT,
                  abi.MIBM_S_INERT_TENSOR, abi.MIBM_S_INT_PRN_DA, abi.MIBM_S_INT_TAU_DA,
                  abi.MIBM_S_INT_R_X_PRN_DA, abi.MIBM_S_INT_R_X_TAU_DA, abi.MIBM_S_INT_PRN_DA_M1,
                  abi.MIBM_S_INT_TAU_DA_M1, abi.MIBM_S_INT_R_X_PRN_DA_M1, abi.MIBM_S_INT_R_X_TAU_DA_M1,
                  abi.MIBM_S_FP, abi.MIBM_S_FTAU, abi.MIBM_S_TORQ_P, abi.MIBM_S_TORQ_TAU}
#: doubles per registered scalar slot (InertTensor(3,3) is the widest)
SCALAR_WIDTH = 9


def field_shape(fid: int, n1m: int, n2m: int, n3m: int) -> tuple[int, int, int]:
    n1, n2 = n1m + 1, n2m + 1
    if fid == abi.MIBM_F_DPH:
        return (n1, n2 + 1, n3m + 2)
    if fid in GHOSTED:
        return (n1, n2, n3m + 2)
    return (n1, n2, n3m)


def mesh_spec(mid: int, nv: int, ne: int, nf: int):
    """Fortran shape and dtype of each registered mesh array."""
    d, i = np.float64, np.int32
    spec = {
        abi.MIBM_M_XYZV: ((3, nv), d), abi.MIBM_M_VERT_OF_FACE: ((3, nf), i),
        abi.MIBM_M_TRI_BAR: ((3, nf), d), abi.MIBM_M_TRI_NOR: ((3, nf), d),
        abi.MIBM_M_VERT_NOR: ((3, nv), d), abi.MIBM_M_SUR: ((nf,), d),
        abi.MIBM_M_AVERT: ((nv,), d), abi.MIBM_M_VEL_TRI: ((3, nf), d),
        abi.MIBM_M_CFAC: ((nf,), d), abi.MIBM_M_GHOST_FACE: ((nf,), i),
        abi.MIBM_M_GHOST_VERT: ((nv,), i), abi.MIBM_M_PIND: ((6, nf), i),
        abi.MIBM_M_PTXAB_Q1: ((27, nf), d), abi.MIBM_M_PTXAB_Q2: ((27, nf), d),
        abi.MIBM_M_PTXAB_Q3: ((27, nf), d), abi.MIBM_M_PTXAB_TEMP: ((27, nf), d),
        abi.MIBM_M_QW_O: ((nf,), d), abi.MIBM_M_QW_I: ((nf,), d),
        abi.MIBM_M_QW_OVERT: ((nv,), d), abi.MIBM_M_QW_IVERT: ((nv,), d),
        abi.MIBM_M_VMELT: ((3, nv), d), abi.MIBM_M_VMELT_M1: ((3, nv), d),
        abi.MIBM_M_VERT_OF_EDGE: ((2, ne), i), abi.MIBM_M_EDGE_OF_FACE: ((3, nf), i),
        abi.MIBM_M_GHOST_EDGE: ((ne,), i), abi.MIBM_M_ELENGTHS: ((ne,), d),
        abi.MIBM_M_SKEWNESS: ((nf,), d),
    }
    return spec[mid]


def inertia_tensor(p1: np.ndarray, p2: np.ndarray, p3: np.ndarray, dens_ratio: float) -> np.ndarray:
    """Inertia tensor about the centroid of the closed mesh with faces
    (p1, p2, p3), scaled by the density ratio: the signed-tetrahedron sums of
    calc_rigidBody_params (RigidAuxRoutines.f90:653-780, Kallay 2006), used
    at set-up as create_geo.f90:42 does."""
    v = np.einsum("ij,ij->i", p1, np.cross(p2, p3))
    s4 = p1 + p2 + p3
    vol = v.sum()
    com = (v[:, None] * s4).sum(0) / (4.0 * vol)
    vol = vol / 6.0
    mono = lambda a, b: (v * (p1[:, a] * p1[:, b] + p2[:, a] * p2[:, b] + p3[:, a] * p3[:, b]
                              + s4[:, a] * s4[:, b])).sum() / 120.0 - vol * com[a] * com[b]
    xx, yy, zz = mono(0, 0), mono(1, 1), mono(2, 2)
    ixy, ixz, iyz = mono(0, 1), mono(0, 2), mono(1, 2)
    return dens_ratio * np.array([[yy + zz, -ixy, -ixz], [-ixy, zz + xx, -iyz], [-ixz, -iyz, xx + yy]])


@dataclass
class CaseConfig:
    """Physical and numerical parameters (bou.in, part.in, HITForcing.in)."""
    n: int = 64
    n3: int | None = None
    length: float = 2.0 * np.pi
    ren: float = 100.0            # 1/nu
    prandtl: float = 1.0
    betagz: float = 0.0
    tmelt: float = 0.0
    tliq: float = 1.0
    tsol: float = 0.0
    latheat: float = 1.0          # Stefan number St = cp (Tliq - Tmelt) / L
    cpliquid: float = 1.0
    dt: float = 1e-2
    dtmax: float = 1e-2
    cflfix: float = 0.5
    idtv: int = 1
    imlsfor: int = 1
    imlsstr: int = 0
    imelt: int = 1
    iremesh: int = 0
    tagtype: int = 1
    forcing: int = 0
    which_hit: int = 1            # 1 Eswaran-Pope, 2 ABC (HITForcing.in); 3 = linear forcing (extension)
    tl: float = 0.5               # HITForcing.in: TL, EPSSTAR, KF/KMIN, C
    epsstar: float = 0.05
    kf_on_kmin: float = 2.3
    c_hit: float = 0.1
    hit_seed: int = 0
    dens_ratio: float = 1.0
    mesh_level: int = 3
    rad_p: float = 0.5
    axes: tuple = (1.0, 1.0, 1.0)  # anisotropic scaling of the unit mesh
    perc_ethresh: float = 0.7
    v_on_ve: float = 27.0
    seed: int = 0
    kmax: int = 8
    velocity: str = "random"       # "random" | "rest"
    mesh: Mesh | None = None

    @property
    def nz(self) -> int:
        return self.n if self.n3 is None else self.n3


CONFIG0 = dict(n=64, ren=100.0, prandtl=1.0, latheat=1.0, cpliquid=1.0, mesh_level=3, rad_p=0.5,
               imelt=1, imlsstr=0, seed=0)


class Case:
    """Fortran-layout state of one melting case."""

    def __init__(self, cfg: CaseConfig):
        self.cfg = cfg
        n, nz = cfg.n, cfg.nz
        self.n1m = self.n2m = n
        self.n3m = nz
        self.xlen = self.ylen = self.zlen = cfg.length
        self.fields = {fid: np.zeros(field_shape(fid, n, n, nz), dtype=np.float64, order="F")
                       for fid in range(abi.MIBM_NFIELDS)}
        for fid in (abi.MIBM_F_VOFX, abi.MIBM_F_VOFY, abi.MIBM_F_VOFZ, abi.MIBM_F_VOFP):
            self.fields[fid][...] = 1.0                       # init.f90:30-33
        self.sc = np.zeros((abi.MIBM_NSCALARS, SCALAR_WIDTH), dtype=np.float64)
        self.iv = np.zeros(abi.MIBM_NINTS, dtype=np.int32)
        self.mesh_arrays: dict[int, np.ndarray] = {}
        self._grid()
        self._params()
        self._geometry()
        self._initial_condition()
        self.ctx: dict[str, int] = {}

    # ---------------------------------------------------------------- grid
    def _grid(self):
        n1m, n2m, n3m = self.n1m, self.n2m, self.n3m
        self.dx1, self.dx2, self.dx3 = n1m / self.xlen, n2m / self.ylen, n3m / self.zlen
        i = np.arange(1, n1m + 1)
        self.xc = self.xlen * ((i - 1) / n1m)
        self.xm = (self.xlen * ((i - 1) / n1m) + self.xlen * (i / n1m)) * 0.5
        j = np.arange(1, n2m + 1)
        self.yc = self.ylen * ((j - 1) / n2m)
        self.ym = (self.ylen * ((j - 1) / n2m) + self.ylen * (j / n2m)) * 0.5
        k = np.arange(1, n3m + 1)
        self.zc = self.zlen * ((k - 1) / n3m)
        self.zm = (self.zlen * ((k - 1) / n3m) + self.zlen * (k / n3m)) * 0.5

    def S(self, sid: int) -> float:
        return float(self.sc[sid, 0])

    def set_S(self, sid: int, v: float) -> None:
        self.sc[sid, 0] = v

    def _params(self):
        c, A = self.cfg, abi
        self.set_S(A.MIBM_S_DT, c.dt)
        self.set_S(A.MIBM_S_DTMAX, c.dtmax)
        self.set_S(A.MIBM_S_CFLFIX, c.cflfix)
        self.set_S(A.MIBM_S_REN, c.ren)
        self.set_S(A.MIBM_S_PEC, c.ren * c.prandtl)           # papero.f90:365
        self.set_S(A.MIBM_S_BETAGZ, c.betagz)
        self.set_S(A.MIBM_S_TMELT, c.tmelt)
        self.set_S(A.MIBM_S_TLIQ, c.tliq)
        self.set_S(A.MIBM_S_TSOL, c.tsol)
        self.set_S(A.MIBM_S_LATHEAT, c.latheat)
        self.set_S(A.MIBM_S_CPLIQUID, c.cpliquid)
        self.set_S(A.MIBM_S_WCON, 0.3)                          # initmls.f90:12
        self.set_S(A.MIBM_S_WSCL, 1.5)                          # initmls.f90:13
        self.set_S(A.MIBM_S_DENS_RATIO, c.dens_ratio)
        self.set_S(A.MIBM_S_TL, c.tl)
        self.set_S(A.MIBM_S_EPSSTAR, c.epsstar)
        self.set_S(A.MIBM_S_KF_ON_KMIN, c.kf_on_kmin)
        self.set_S(A.MIBM_S_C_HIT, c.c_hit)
        h = (1.0 / self.dx1 + 1.0 / self.dx2 + 1.0 / self.dx3) / 3.0
        celvol = 1.0 / (self.dx1 * self.dx2 * self.dx3)
        self.set_S(A.MIBM_S_H_EULERIAN, h)
        self.set_S(A.MIBM_S_CELVOL, celvol)
        self.set_S(A.MIBM_S_E_THRESH, c.perc_ethresh * h)
        self.set_S(A.MIBM_S_V_THRESH, c.v_on_ve * celvol)
        iv = self.iv
        iv[A.MIBM_I_IMLSFOR], iv[A.MIBM_I_IMLSSTR], iv[A.MIBM_I_IMELT] = c.imlsfor, c.imlsstr, c.imelt
        iv[A.MIBM_I_IREMESH], iv[A.MIBM_I_TAGTYPE], iv[A.MIBM_I_FORCING] = c.iremesh, c.tagtype, c.forcing
        iv[A.MIBM_I_IDTV], iv[A.MIBM_I_NSST] = c.idtv, 3
        iv[A.MIBM_I_WHICH_HIT], iv[A.MIBM_I_HIT_SEED] = c.which_hit, c.hit_seed
        stationary = not (c.imlsfor == 1 and (c.imlsstr == 1 or c.imelt == 1))   # papero.f90:353-358
        iv[A.MIBM_I_STATIONARY] = 1 if stationary else 0

    # ------------------------------------------------------------ geometry
    def _geometry(self):
        c, A = self.cfg, abi
        mesh = c.mesh if c.mesh is not None else icosphere(c.mesh_level)
        nv, ne, nf = mesh.nv, mesh.ne, mesh.nf
        self.maxnv, self.maxne, self.maxnf = nv, ne, nf
        for mid in range(A.MIBM_NMESH):
            shape, dt = mesh_spec(mid, nv, ne, nf)
            self.mesh_arrays[mid] = np.zeros(shape, dtype=dt, order="F")
        M = self.mesh_arrays
        xyz0 = mesh.xyz * np.asarray(c.axes)[None, :] * c.rad_p      # create_geo.f90:22
        pos = np.array([0.5 * self.xlen, 0.5 * self.ylen, 0.5 * self.zlen])  # create_geo.f90:51-53
        M[A.MIBM_M_XYZV][...] = (xyz0 + pos[None, :]).T               # create_geo.f90:125-130
        M[A.MIBM_M_VERT_OF_FACE][...] = mesh.vert_of_face.T
        M[A.MIBM_M_VERT_OF_EDGE][...] = mesh.vert_of_edge.T
        M[A.MIBM_M_EDGE_OF_FACE][...] = mesh.edge_of_face.T
        self.sc[A.MIBM_S_POS_CM, :3] = pos
        self._geometry_refresh(initial=True)
        h, cv = self.S(A.MIBM_S_H_EULERIAN), self.S(A.MIBM_S_CELVOL)
        M[A.MIBM_M_CFAC][...] = (M[A.MIBM_M_SUR] * h) / cv            # initmls.f90:25

    def _geometry_refresh(self, initial=False):
        """Areas, normals, centroids, vertex areas/normals (triaux.f90:53-323)."""
        A, M = abi, self.mesh_arrays
        x = M[A.MIBM_M_XYZV].T
        f = M[A.MIBM_M_VERT_OF_FACE].T - 1
        p1, p2, p3 = x[f[:, 0]], x[f[:, 1]], x[f[:, 2]]
        d12 = np.sqrt(((p1 - p2) ** 2).sum(1))
        d23 = np.sqrt(((p2 - p3) ** 2).sum(1))
        d31 = np.sqrt(((p3 - p1) ** 2).sum(1))
        sp = (d12 + d23 + d31) / 2.0
        sur = np.sqrt(sp * (sp - d12) * (sp - d23) * (sp - d31))
        M[A.MIBM_M_SUR][...] = sur
        nrm = np.cross(p2 - p1, p3 - p1)
        nrm = nrm / np.sqrt((nrm ** 2).sum(1))[:, None]
        M[A.MIBM_M_TRI_NOR][...] = nrm.T
        M[A.MIBM_M_TRI_BAR][...] = ((p1 + p2 + p3) / 3.0).T
        av = np.zeros(self.maxnv)
        vn = np.zeros((self.maxnv, 3))
        for q in range(3):
            np.add.at(av, f[:, q], sur / 3.0)
            np.add.at(vn, f[:, q], sur[:, None] * nrm)
        M[A.MIBM_M_AVERT][...] = av
        M[A.MIBM_M_VERT_NOR][...] = (vn / np.sqrt((vn ** 2).sum(1))[:, None]).T
        vol = (x[f[:, 0], 0] * (x[f[:, 1], 1] * x[f[:, 2], 2] - x[f[:, 1], 2] * x[f[:, 2], 1])
               + x[f[:, 1], 0] * (x[f[:, 2], 1] * x[f[:, 0], 2] - x[f[:, 2], 2] * x[f[:, 0], 1])
               + x[f[:, 2], 0] * (x[f[:, 0], 1] * x[f[:, 1], 2] - x[f[:, 0], 2] * x[f[:, 1], 1]))
        self.set_S(A.MIBM_S_VOLUME, vol.sum() / 6.0)
        self.set_S(A.MIBM_S_SURFACE, sur.sum())
        self.sc[A.MIBM_S_INERT_TENSOR, :9] = inertia_tensor(p1, p2, p3, self.cfg.dens_ratio).ravel(order="F")
        e = M[A.MIBM_M_VERT_OF_EDGE].T - 1
        M[A.MIBM_M_ELENGTHS][...] = np.sqrt(((x[e[:, 0]] - x[e[:, 1]]) ** 2).sum(1))

    # --------------------------------------------------- initial condition
    def _initial_condition(self):
        c, A, F = self.cfg, abi, self.fields
        n1m, n2m, n3m = self.n1m, self.n2m, self.n3m
        if c.velocity == "random":
            if n1m != n3m:
                raise ValueError("random velocity needs a cube")
            u, v, w = random_velocity(n1m, self.xlen, c.seed, c.kmax)
            F[A.MIBM_F_VX][:n1m, :n2m, 1:n3m + 1] = u
            F[A.MIBM_F_VY][:n1m, :n2m, 1:n3m + 1] = v
            F[A.MIBM_F_VZ][:n1m, :n2m, 1:n3m + 1] = w
        pos = self.sc[A.MIBM_S_POS_CM, :3]
        T = tanh_temperature(self.xm, self.ym, self.zm, pos, c.rad_p, c.tliq, c.tsol, self.dx1, c.axes)
        F[A.MIBM_F_TEMP][...] = c.tsol
        F[A.MIBM_F_TEMP][:n1m, :n2m, 1:n3m + 1] = T
        for fid in (A.MIBM_F_VX, A.MIBM_F_VY, A.MIBM_F_VZ, A.MIBM_F_TEMP, A.MIBM_F_PR):
            self.fill_ghosts(fid)

    def fill_ghosts(self, fid: int) -> None:
        a = self.fields[fid]
        a[:, :, 0] = a[:, :, self.n3m]
        a[:, :, self.n3m + 1] = a[:, :, 1]

    def interior(self, fid: int) -> np.ndarray:
        """Owned cells (1:n1m, 1:n2m, 1:n3m) as a 0-based [i,j,k] view."""
        a = self.fields[fid]
        k0 = 1 if a.shape[2] == self.n3m + 2 else 0
        return a[:self.n1m, :self.n2m, k0:k0 + self.n3m]

    def clone(self) -> "Case":
        other = copy.copy(self)
        other.fields = {k: v.copy(order="F") for k, v in self.fields.items()}
        other.mesh_arrays = {k: v.copy(order="F") for k, v in self.mesh_arrays.items()}
        other.sc = self.sc.copy()
        other.iv = self.iv.copy()
        other.ctx = {}
        return other

    # ----------------------------------------------------------- C-ABI use
    def attach(self, lib: abi.Lib, initial_tag: bool = True) -> int:
        """Register every array and scalar with ``lib`` and initialise it."""
        A = abi
        cid = lib.mibm_context_create_()
        lib.check("context_create")
        lib.mibm_set_grid_(A.ref_int(self.n1m), A.ref_int(self.n2m), A.ref_int(self.n3m),
                           A.ref_double(self.xlen), A.ref_double(self.ylen), A.ref_double(self.zlen))
        lib.check("set_grid")
        lib.mibm_set_mesh_sizes_(A.ref_int(self.maxnv), A.ref_int(self.maxne), A.ref_int(self.maxnf))
        for fid, arr in self.fields.items():
            lib.mibm_register_field_(A.ref_int(fid), arr.ctypes.data)
        for mid, arr in self.mesh_arrays.items():
            lib.mibm_register_mesh_(A.ref_int(mid), arr.ctypes.data)
        for sid in range(A.MIBM_NSCALARS):
            lib.mibm_register_scalar_(A.ref_int(sid), self.sc[sid].ctypes.data)
        for iid in range(A.MIBM_NINTS):
            lib.mibm_register_int_(A.ref_int(iid), self.iv[iid:iid + 1].ctypes.data)
        lib.check("register")
        lib.mibm_init_()
        lib.check("init")
        self.ctx[lib.path] = cid
        if initial_tag and self.cfg.imlsfor == 1:
            lib.tagcells_initial_()
            lib.check("tagcells_initial")
        return cid

    def bind(self, lib: abi.Lib) -> None:
        lib.mibm_context_bind_(abi.ref_int(self.ctx[lib.path]))

    def detach(self, lib: abi.Lib) -> None:
        if lib.path in self.ctx:
            lib.mibm_context_destroy_(abi.ref_int(self.ctx.pop(lib.path)))

    def step(self, lib: abi.Lib, ntime: int) -> None:
        """One iteration of the reference time loop, gcurv.f90:151-172."""
        A = abi
        self.bind(lib)
        self.iv[A.MIBM_I_NTIME] = ntime
        lib.cfl_()
        lib.check("cfl")
        if self.iv[A.MIBM_I_IDTV] == 1:
            if ntime != 1:
                self.set_S(A.MIBM_S_DT, self.S(A.MIBM_S_DTMAX))
            lib.get_dt_()
        if self.iv[A.MIBM_I_FORCING] == 1:        # gcurv.f90:164-170
            which = self.iv[A.MIBM_I_WHICH_HIT]
            if which == 1:
                lib.calchitrandomforce_()
            elif which == 2:
                lib.calcabc_hitforce_()
            elif which == 3:
                lib.mibm_linear_hit_force_()
            lib.check("forcing")
        lib.tschem_()
        lib.check("tschem")
        self.set_S(A.MIBM_S_TIME, self.S(A.MIBM_S_TIME) + self.S(A.MIBM_S_DT))

    def run(self, lib: abi.Lib, nsteps: int, start: int = 1) -> None:
        for nt in range(start, start + nsteps):
            self.step(lib, nt)

    def use_library_remesher(self, lib: abi.Lib, remesher: abi.Lib | None = None) -> None:
        """Set the library's remesher (QEM coarsening + volume-conserving
        smoothing, the reference's remesh_coarsen / remesh_smooth) as this
        case's remesh callback in `lib`.  With `remesher` None (or `lib`
        itself) that is `mibm_remesh_builtin_`; otherwise `remesher` is a
        libmibm.so whose host function `mibm_remesh_mesh` is called on this
        case's registered arrays (another library exporting the same ABI
        gets the same remesher), with face_of_edge kept here between calls."""
        A = abi
        self.bind(lib)
        if remesher is None or remesher.path == lib.path:
            fn = abi.C.cast(lib.dll.mibm_remesh_builtin_, abi.C.c_void_p)
            lib.mibm_set_remesh_callback_(fn, None)
            return
        M = self.mesh_arrays
        foe = np.zeros((2, self.maxne), dtype=np.int32, order="F")
        stats = np.zeros(8)

        def call(user):
            P = lambda mid: M[mid].ctypes.data
            return int(remesher.mibm_remesh_mesh(
                self.maxnv, self.maxne, self.maxnf, P(A.MIBM_M_XYZV), P(A.MIBM_M_TRI_NOR), P(A.MIBM_M_VMELT),
                P(A.MIBM_M_ELENGTHS), P(A.MIBM_M_VERT_OF_FACE), P(A.MIBM_M_EDGE_OF_FACE), P(A.MIBM_M_VERT_OF_EDGE),
                foe.ctypes.data, P(A.MIBM_M_GHOST_FACE), P(A.MIBM_M_GHOST_EDGE), P(A.MIBM_M_GHOST_VERT),
                self.S(A.MIBM_S_E_THRESH), stats.ctypes.data))

        self._remesh_trampoline = (abi.REMESH_FN(call), foe, stats)     # kept alive with the case
        lib.mibm_set_remesh_callback_(abi.C.cast(self._remesh_trampoline[0], abi.C.c_void_p), None)

    def sync_to_host(self, lib: abi.Lib, mask: int = -1) -> None:
        self.bind(lib)
        lib.mibm_sync_to_host_(abi.ref_ll(mask))
        lib.check("sync_to_host")

    def sync_from_host(self, lib: abi.Lib, mask: int = -1) -> None:
        self.bind(lib)
        lib.mibm_sync_from_host_(abi.ref_ll(mask))
        lib.check("sync_from_host")
