"""Test helpers: seeded cases, paired oracle/GPU runs, error norms."""
from __future__ import annotations

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
