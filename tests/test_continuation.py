"""Continuation files (mpi_write_continua mpi_routines.f90:1223-1522,
continua_particle create_geo.f90:280-407, WriteRandForcCoef hit.f90:256-305)
and the restart path (inirea.f90, import_particles, hdf_read_bhat).

A run of 2 + 2 steps with a continuation written and read in between must
equal a run of 4 steps bit for bit, in both libraries, for a free melting
body and for the stochastic and ABC forcings; across the libraries the
continued runs agree to the steps' parity.  A restart on a finer grid goes
through interp_ as inirea.f90 does.
"""
from __future__ import annotations

import os

import numpy as np
import pytest

from melt_ibm_gb300 import abi as A
from melt_ibm_gb300.case import Case
from melt_ibm_gb300.continuation import (FIELD_FILES, PARTICLE_MESH, PARTICLE_SCALARS, read_continuation,
                                         read_grid, write_continuation)
from tests.helpers import FIELDS_OUT, rel_l2, small_config

CONFIGS = {
    "free_melting": dict(imlsstr=1, dens_ratio=2.0),
    "stochastic_forcing": dict(imlsstr=1, dens_ratio=2.0, forcing=1, which_hit=1),
    "abc_forcing": dict(forcing=1, which_hit=2),
}


def _fields(case):
    return {k: case.interior(f).copy() for k, f in FIELDS_OUT.items()}


def _continued(lib, cfg, directory, steps=(2, 2), reader_lib=None, precision=None):
    """Run steps[0], write, read into a fresh case (on reader_lib), run steps[1]."""
    import ctypes as C
    a = Case(cfg)
    a.attach(lib)
    if precision is not None:
        a.bind(lib)
        lib.mibm_set_precision_(C.byref(C.c_int(precision)), C.byref(C.c_int(2)))
    a.run(lib, steps[0])
    write_continuation(a, lib, directory)
    a.detach(lib)
    rl = reader_lib or lib
    b = Case(cfg)
    fs = read_continuation(b, directory)
    b.attach(rl)
    fs.apply(b, rl)
    if precision is not None:
        b.bind(rl)
        rl.mibm_set_precision_(C.byref(C.c_int(precision)), C.byref(C.c_int(2)))
    b.run(rl, steps[1], start=steps[0] + 1)
    b.sync_to_host(rl, -1)
    out = _fields(b), b.mesh_arrays[A.MIBM_M_XYZV].copy()
    b.detach(rl)
    return out


def _straight(lib, cfg, nsteps=4, precision=None):
    import ctypes as C
    r = Case(cfg)
    r.attach(lib)
    if precision is not None:
        r.bind(lib)
        lib.mibm_set_precision_(C.byref(C.c_int(precision)), C.byref(C.c_int(2)))
    r.run(lib, nsteps)
    r.sync_to_host(lib, -1)
    out = _fields(r), r.mesh_arrays[A.MIBM_M_XYZV].copy()
    r.detach(lib)
    return out


@pytest.mark.parametrize("name", list(CONFIGS))
def test_oracle_continuation_is_exact(oracle_lib, tmp_path, name):
    cfg = small_config(n=16, level=2, **CONFIGS[name])
    f_ref, x_ref = _straight(oracle_lib, cfg)
    f_c, x_c = _continued(oracle_lib, cfg, str(tmp_path))
    for k in FIELDS_OUT:
        assert np.array_equal(f_c[k], f_ref[k]), k
    assert np.array_equal(x_c, x_ref)


def test_files_follow_the_reference_layout(oracle_lib, tmp_path):
    cfg = small_config(n=16, level=2, imlsstr=1, dens_ratio=2.0, forcing=1, which_hit=1)
    c = Case(cfg)
    c.attach(oracle_lib)
    c.run(oracle_lib, 1)
    write_continuation(c, oracle_lib, str(tmp_path))
    n1, n2, n3, t = read_grid(str(tmp_path))
    assert (n1, n2, n3) == (17, 17, 17) and t == c.S(A.MIBM_S_TIME) and t > 0
    for stem, (name, fid, _) in FIELD_FILES.items():
        with np.load(os.path.join(tmp_path, stem + ".npz")) as z:
            assert list(z.keys()) == [name]
            assert z[name].shape == (17, 17, 16) and z[name].dtype == np.float64
            assert np.array_equal(z[name][:16, :16, :], c.interior(fid))
    with np.load(os.path.join(tmp_path, "particles.npz")) as z:
        for name in PARTICLE_SCALARS:
            assert name in z
        assert z["pos_CM"].shape == (3, 1) and z["InertTensor"].shape == (3, 3, 1)
        for name, mid in PARTICLE_MESH.items():
            assert z[name].shape == c.mesh_arrays[mid].shape + (1,), name
            assert z[name].dtype == c.mesh_arrays[mid].dtype, name
    with np.load(os.path.join(tmp_path, "continua_bhat.npz")) as z:
        nm = int(oracle_lib.mibm_hit_modes_())
        assert z["bhat_re"].shape == (3, nm, nm, nm) and np.any(z["bhat_re"] != 0)
    with np.load(os.path.join(tmp_path, "continua_master.npz")) as z:
        assert z["Re"][0] == c.S(A.MIBM_S_REN) and z["X_cordin"].shape == (17,) and z["Z_cordin"].shape == (16,)
    c.detach(oracle_lib)


def test_reference_written_set_restarts(oracle_lib, tmp_path):
    """A set without this library's additions (what the reference writes)
    reads: fields, mesh and rigid state load, the rest keeps the case's values."""
    cfg = small_config(n=16, level=2, imlsstr=1, dens_ratio=2.0)
    a = Case(cfg)
    a.attach(oracle_lib)
    a.run(oracle_lib, 2)
    write_continuation(a, oracle_lib, str(tmp_path))
    p = os.path.join(tmp_path, "particles.npz")
    with np.load(p) as z:
        keep = {k: z[k] for k in z if k in PARTICLE_SCALARS or k in PARTICLE_MESH}
    np.savez(p, **keep)
    b = Case(cfg)
    read_continuation(b, str(tmp_path))
    for k, f in FIELDS_OUT.items():
        assert np.array_equal(b.interior(f), a.interior(f)), k
    assert np.array_equal(b.mesh_arrays[A.MIBM_M_XYZV], a.mesh_arrays[A.MIBM_M_XYZV])
    assert np.array_equal(b.mesh_arrays[A.MIBM_M_VEL_TRI], 0.0 * b.mesh_arrays[A.MIBM_M_VEL_TRI])
    b.attach(oracle_lib)
    b.run(oracle_lib, 1, start=3)
    assert all(np.isfinite(b.interior(f)).all() for f in FIELDS_OUT.values())
    a.detach(oracle_lib)
    b.detach(oracle_lib)


def test_finer_grid_limit(oracle_lib, tmp_path):
    a = Case(small_config(n=8, level=1))
    a.attach(oracle_lib)
    write_continuation(a, oracle_lib, str(tmp_path))
    a.detach(oracle_lib)
    with pytest.raises(ValueError, match="twice"):
        read_continuation(Case(small_config(n=24, level=1)), str(tmp_path), oracle_lib)


def test_oracle_regrid_restart(oracle_lib, tmp_path):
    """16^3 -> 24^3 through interp_: the new velocity keeps the old one's
    large scales (rms within a few percent) and stays nearly solenoidal."""
    a = Case(small_config(n=16, level=2, imlsstr=1, dens_ratio=2.0))
    a.attach(oracle_lib)
    a.run(oracle_lib, 1)
    write_continuation(a, oracle_lib, str(tmp_path))
    b = Case(small_config(n=24, level=2, imlsstr=1, dens_ratio=2.0))
    read_continuation(b, str(tmp_path), oracle_lib)
    assert b.S(A.MIBM_S_TIME) == a.S(A.MIBM_S_TIME)
    ua, ub = a.interior(A.MIBM_F_VX), b.interior(A.MIBM_F_VX)
    mid = slice(3, 12)      # away from the zeroed top plane of the old array
    assert abs(np.sqrt(np.mean(ub[:, :, 5:18] ** 2)) / np.sqrt(np.mean(ua[:, :, mid] ** 2)) - 1) < 0.1
    assert np.array_equal(b.interior(A.MIBM_F_PR), 0.0 * b.interior(A.MIBM_F_PR))   # not read
    b.attach(oracle_lib)
    b.run(oracle_lib, 1, start=2)
    assert all(np.isfinite(b.interior(f)).all() for f in FIELDS_OUT.values())
    a.detach(oracle_lib)
    b.detach(oracle_lib)


# ------------------------------------------------------------------ GPU
@pytest.mark.gpu
@pytest.mark.parametrize("name", list(CONFIGS))
def test_gpu_continuation_is_exact(gpu_lib, tmp_path, name):
    cfg = small_config(n=24, level=2, **CONFIGS[name])
    f_ref, x_ref = _straight(gpu_lib, cfg)
    f_c, x_c = _continued(gpu_lib, cfg, str(tmp_path))
    for k in FIELDS_OUT:
        assert np.array_equal(f_c[k], f_ref[k]), k
    assert np.array_equal(x_c, x_ref)


@pytest.mark.gpu
def test_gpu_precision_form_continuation(gpu_lib, tmp_path):
    cfg = small_config(n=24, level=2, imlsstr=1, dens_ratio=2.0)
    f_ref, _ = _straight(gpu_lib, cfg, precision=1)
    f_c, _ = _continued(gpu_lib, cfg, str(tmp_path), precision=1)
    for k in FIELDS_OUT:
        assert rel_l2(f_c[k], f_ref[k]) <= 1e-6, k


@pytest.mark.gpu
def test_gpu_written_oracle_continued(gpu_lib, oracle_lib, tmp_path):
    """A set written by the GPU library continues on the oracle: the result
    matches the GPU's own continued run to the steps' parity."""
    cfg = small_config(n=24, level=2, imlsstr=1, dens_ratio=2.0, forcing=1, which_hit=1)
    f_g, x_g = _continued(gpu_lib, cfg, str(tmp_path / "g"))
    f_o, x_o = _continued(gpu_lib, cfg, str(tmp_path / "o"), reader_lib=oracle_lib)
    for k in FIELDS_OUT:
        assert rel_l2(f_g[k], f_o[k]) <= 1e-10, k
    assert np.abs(x_g - x_o).max() <= 1e-11


@pytest.mark.gpu
def test_gpu_regrid_restart_parity(gpu_lib, oracle_lib, tmp_path):
    a = Case(small_config(n=16, level=2, imlsstr=1, dens_ratio=2.0))
    a.attach(oracle_lib)
    a.run(oracle_lib, 1)
    write_continuation(a, oracle_lib, str(tmp_path))
    a.detach(oracle_lib)
    out = []
    for lib in (oracle_lib, gpu_lib):
        b = Case(small_config(n=24, level=2, imlsstr=1, dens_ratio=2.0))
        read_continuation(b, str(tmp_path), lib)
        b.attach(lib)
        b.run(lib, 2, start=2)
        b.sync_to_host(lib, -1)
        out.append(_fields(b))
        b.detach(lib)
    for k in FIELDS_OUT:
        assert rel_l2(out[1][k], out[0][k]) <= 1e-10, k
