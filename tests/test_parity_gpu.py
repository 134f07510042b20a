"""Parity of libmibm.so (GB300) against the CPU oracle, through the C-ABI.

Per-routine tests drive each drop-in symbol on seeded random inputs and
compare the arrays the routine writes.  Step tests run the reference time
loop (cfl -> get_dt -> tschem) on config-0 physics and require relative L2
<= 1e-10 on u, v, w, T, p after 1 and 10 steps (the plain-form tolerance),
post-projection divergence <= 1e-12, and bitwise run-to-run determinism.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from melt_ibm_gb300 import abi
from melt_ibm_gb300.case import Case, CaseConfig, CONFIG0
from melt_ibm_gb300.fields import discrete_divergence_max
from tests.helpers import FIELDS_OUT, pair, randomize, rel_l2, set_substep, small_config

pytestmark = pytest.mark.gpu
A = abi
TOL_ROUTINE = 1e-12     # one routine on identical inputs (FMA / summation order only)
TOL_STEP = 1e-10        # plain FP64 form: tolerance after 1 and 10 steps
ALL = -1


def _run(case: Case, lib, routine: str, *args):
    case.bind(lib)
    getattr(lib, routine)(*args)
    lib.check(routine)
    case.sync_to_host(lib, ALL)


def _cmp_fields(co, cg, fids, tol=TOL_ROUTINE):
    for fid in fids:
        a, b = cg.interior(fid), co.interior(fid)
        err = rel_l2(a, b)
        assert err <= tol, f"field {fid}: rel L2 {err:.3e}"


STENCIL_ROUTINES = {
    "hdnl1_": [A.MIBM_F_DQ], "hdnl2_": [A.MIBM_F_DPH], "hdnl3_": [A.MIBM_F_QCAP], "hdnlte_": [A.MIBM_F_HTEMP],
    "invtr1_": [A.MIBM_F_VX, A.MIBM_F_RU1, A.MIBM_F_RHS], "invtr2_": [A.MIBM_F_VY, A.MIBM_F_RU2, A.MIBM_F_RHS],
    "invtr3_": [A.MIBM_F_VZ, A.MIBM_F_RU3, A.MIBM_F_RHS], "invtrte_": [A.MIBM_F_TEMP, A.MIBM_F_RUT, A.MIBM_F_RHS],
    "divg_": [A.MIBM_F_DPH], "updvp_": [A.MIBM_F_VX, A.MIBM_F_VY, A.MIBM_F_VZ], "prcalc_": [A.MIBM_F_PR],
}


@pytest.mark.parametrize("n", [16, 24])
@pytest.mark.parametrize("routine", list(STENCIL_ROUTINES))
def test_stencil_routine_parity(oracle_lib, gpu_lib, routine, n):
    case = Case(small_config(n=n))
    randomize(case)
    co, cg = pair(case, oracle_lib, gpu_lib, initial_tag=False)
    co.bind(oracle_lib)
    getattr(oracle_lib, routine)()
    _run(cg, gpu_lib, routine)
    _cmp_fields(co, cg, STENCIL_ROUTINES[routine])


@pytest.mark.parametrize("n, n3", [(16, None), (24, None), (48, None), (192, 8), (32, 256), (24, 18),
                                   (128, None), (256, None)])
def test_phcalc_parity(oracle_lib, gpu_lib, n, n3):
    """Poisson solve; the z lines are chunked below 16384 (kx, ky) lines
    (32 x 32 x 256: 16 chunks of 16, the largest block; 128^3: 8320 lines)
    and swept one per thread from there on (192 x 192 x 8: 18624 lines;
    256^3: 33024) or where no chunk length divides the line (24 x 24 x 18).
    128^3 and 256^3 run the compile-time x/y transforms of those lengths, the
    instances the 128^3 and 256^3 configurations use."""
    small = n3 is None and n <= 48
    case = Case(small_config(n=n, n3=n3, velocity="random" if small else "rest"))
    randomize(case)
    co, cg = pair(case, oracle_lib, gpu_lib, initial_tag=False)
    for c, lib in ((co, oracle_lib), (cg, gpu_lib)):
        c.bind(lib)
        lib.divg_()
        lib.phcalc_()
        lib.check("phcalc")
    cg.sync_to_host(gpu_lib, ALL)
    _cmp_fields(co, cg, [A.MIBM_F_DPH])


@pytest.mark.parametrize("which", ["solxi_", "solxj_", "solxk_"])
@pytest.mark.parametrize("betadx", [0.004, 0.9, 40.0])
def test_line_solve_parity(oracle_lib, gpu_lib, which, betadx):
    case = Case(small_config(n=16))
    randomize(case)
    case.fields[A.MIBM_F_RHS][...] = np.random.default_rng(5).standard_normal(case.fields[A.MIBM_F_RHS].shape)
    co, cg = pair(case, oracle_lib, gpu_lib, initial_tag=False)
    for c, lib in ((co, oracle_lib), (cg, gpu_lib)):
        c.bind(lib)
        bd = C.byref(C.c_double(betadx))
        if which == "solxk_":
            vx = c.fields[A.MIBM_F_VX]
            q = vx.ctypes.data + vx.shape[0] * vx.shape[1] * 8      # vx(1,1,kstart)
            lib.solxk_(C.c_void_p(q), bd)
        else:
            getattr(lib, which)(bd)
        lib.check(which)
    cg.sync_to_host(gpu_lib, ALL)
    _cmp_fields(co, cg, [A.MIBM_F_RHS, A.MIBM_F_VX])


def _lag_pair(oracle_lib, gpu_lib, n=24, level=2, **kw):
    case = Case(small_config(n=n, level=level, **kw))
    co, cg = pair(case, oracle_lib, gpu_lib, initial_tag=True)
    return co, cg


def test_initial_tagging_parity(oracle_lib, gpu_lib):
    co, cg = _lag_pair(oracle_lib, gpu_lib, n=32, level=3)
    cg.sync_to_host(gpu_lib, ALL)
    for fid in (A.MIBM_F_VOFP, A.MIBM_F_VOFX, A.MIBM_F_VOFY, A.MIBM_F_VOFZ, A.MIBM_F_SDF):
        assert np.max(np.abs(cg.interior(fid) - co.interior(fid))) <= 1e-13, fid


def test_mls_weight_and_indices_parity(oracle_lib, gpu_lib):
    co, cg = _lag_pair(oracle_lib, gpu_lib)
    for c, lib in ((co, oracle_lib), (cg, gpu_lib)):
        c.bind(lib)
        lib.findcentroidindices_()
        lib.mlsweight_()
        lib.check("mlsweight")
    cg.sync_to_host(gpu_lib, ALL)
    assert np.array_equal(cg.mesh_arrays[A.MIBM_M_PIND], co.mesh_arrays[A.MIBM_M_PIND])
    # the reference's construction in the oracle's operation order, with the
    # shared written-out exp: the same bits up to the last place
    for mid in (A.MIBM_M_PTXAB_Q1, A.MIBM_M_PTXAB_Q2, A.MIBM_M_PTXAB_Q3, A.MIBM_M_PTXAB_TEMP):
        assert rel_l2(cg.mesh_arrays[mid], co.mesh_arrays[mid]) <= 1e-15, mid


def test_mls_force_parity(oracle_lib, gpu_lib):
    co, cg = _lag_pair(oracle_lib, gpu_lib)
    for c, lib in ((co, oracle_lib), (cg, gpu_lib)):
        c.bind(lib)
        lib.findcentroidindices_()
        lib.mlsweight_()
        lib.mlsforce_()
        lib.velforce_()
        lib.tempforce_()
        lib.check("force")
    cg.sync_to_host(gpu_lib, ALL)
    _cmp_fields(co, cg, [A.MIBM_F_VX, A.MIBM_F_VY, A.MIBM_F_VZ, A.MIBM_F_TEMP], tol=1e-13)
    _cmp_fields(co, cg, [A.MIBM_F_FORXC, A.MIBM_F_FORYC, A.MIBM_F_FORZC, A.MIBM_F_FORTEMP], tol=1e-13)


def test_heat_flux_and_stefan_parity(oracle_lib, gpu_lib):
    co, cg = _lag_pair(oracle_lib, gpu_lib)
    for c, lib in ((co, oracle_lib), (cg, gpu_lib)):
        c.bind(lib)
        set_substep(c, 0, dt=0.01)
        lib.findprobeindices_()
        lib.mls_heatflux_()
        lib.apply_stefancondition_()
        lib.check("heat")
    cg.sync_to_host(gpu_lib, ALL)
    assert np.array_equal(cg.mesh_arrays[A.MIBM_M_PIND], co.mesh_arrays[A.MIBM_M_PIND])
    # The reference's MLS basis [1, x, y, z] in absolute coordinates
    # (mls_heatFlux.f90:267-270) gives 4x4 moment matrices with condition
    # numbers ~1e8: a last-bit difference of any input would show as 1e-9
    # here.  The plain form evaluates that construction in the oracle's
    # operation order with the shared exp: the same bits.
    for mid in (A.MIBM_M_QW_O, A.MIBM_M_QW_I, A.MIBM_M_QW_OVERT, A.MIBM_M_QW_IVERT):
        assert rel_l2(cg.mesh_arrays[mid], co.mesh_arrays[mid]) <= 1e-15, mid
    assert rel_l2(cg.mesh_arrays[A.MIBM_M_XYZV], co.mesh_arrays[A.MIBM_M_XYZV]) <= 1e-14


def test_narrow_band_parity_after_motion(oracle_lib, gpu_lib):
    co, cg = _lag_pair(oracle_lib, gpu_lib, n=32, level=3)
    for c, lib in ((co, oracle_lib), (cg, gpu_lib)):
        c.bind(lib)
        x = c.mesh_arrays[A.MIBM_M_XYZV]
        x *= 1.0
        c.mesh_arrays[A.MIBM_M_TRI_BAR][0, :] += 0.013     # shift the centroids only
        c.sync_from_host(lib, ALL)
        lib.tagcells_()
        lib.check("tagcells")
    cg.sync_to_host(gpu_lib, ALL)
    for fid in (A.MIBM_F_VOFP, A.MIBM_F_VOFX, A.MIBM_F_VOFY, A.MIBM_F_VOFZ, A.MIBM_F_SDF):
        assert np.max(np.abs(cg.interior(fid) - co.interior(fid))) <= 1e-12, fid


def test_cfl_and_dt_parity(oracle_lib, gpu_lib):
    case = Case(small_config(n=16))
    co, cg = pair(case, oracle_lib, gpu_lib, initial_tag=False)
    for c, lib in ((co, oracle_lib), (cg, gpu_lib)):
        c.bind(lib)
        lib.cfl_()
        lib.get_dt_()
    assert cg.S(A.MIBM_S_CFLM) == pytest.approx(co.S(A.MIBM_S_CFLM), rel=1e-15)
    assert cg.S(A.MIBM_S_DT) == pytest.approx(co.S(A.MIBM_S_DT), rel=1e-15)


def _steps(case, lib, nsteps):
    case.run(lib, nsteps)
    if lib.mibm_device_count_() > 0 and "libmibm" in lib.path:
        case.sync_to_host(lib, ALL)


@pytest.mark.parametrize("imelt", [1, 0])
def test_step_parity_small(oracle_lib, gpu_lib, imelt):
    case = Case(small_config(n=24, level=2, imelt=imelt))
    co, cg = pair(case, oracle_lib, gpu_lib)
    _steps(co, oracle_lib, 3)
    _steps(cg, gpu_lib, 3)
    for name, fid in FIELDS_OUT.items():
        assert rel_l2(cg.interior(fid), co.interior(fid)) <= TOL_STEP, name


@pytest.fixture(scope="module")
def config0_runs(oracle_lib, gpu_lib):
    """Config 0: 64^3, level-3 icosphere r=0.5, nu=kappa=0.01, St=1, 10 steps."""
    case = Case(CaseConfig(**CONFIG0))
    co, cg = pair(case, oracle_lib, gpu_lib)
    out = {}
    for nsteps, start in ((1, 1), (9, 2)):
        co.run(oracle_lib, nsteps, start=start)
        cg.run(gpu_lib, nsteps, start=start)
        cg.sync_to_host(gpu_lib, ALL)
        out[start + nsteps - 1] = ({k: co.interior(f).copy() for k, f in FIELDS_OUT.items()},
                                   {k: cg.interior(f).copy() for k, f in FIELDS_OUT.items()},
                                   co.S(A.MIBM_S_VOLUME), cg.S(A.MIBM_S_VOLUME))
    return out, cg


@pytest.mark.parametrize("after", [1, 10])
def test_config0_parity(config0_runs, after):
    out, _ = config0_runs
    ref, got, vo, vg = out[after]
    for k in FIELDS_OUT:
        err = rel_l2(got[k], ref[k])
        assert err <= TOL_STEP, f"{k} after {after} steps: rel L2 {err:.3e}"
    assert abs(vg - vo) <= 1e-10 * abs(vo)


def test_config0_divergence(config0_runs):
    out, cg = config0_runs
    got = out[10][1]
    assert discrete_divergence_max(got["vx"], got["vy"], got["vz"], cg.xlen, cg.ylen, cg.zlen) <= 1e-12


def test_gpu_determinism(gpu_lib):
    case = Case(small_config(n=32, level=3))
    runs = []
    for _ in range(2):
        c = case.clone()
        c.attach(gpu_lib)
        c.run(gpu_lib, 2)
        c.sync_to_host(gpu_lib, ALL)
        runs.append({k: c.interior(f).copy() for k, f in FIELDS_OUT.items()})
        c.detach(gpu_lib)
    for k in FIELDS_OUT:
        assert np.array_equal(runs[0][k], runs[1][k]), k


@pytest.mark.parametrize("precision", [0, 1])
def test_step_graph_replay_is_bitwise_identical(gpu_lib, precision):
    """From the second step on tschem_ replays a captured CUDA graph; the
    result must equal launching every kernel directly, bit for bit."""
    case = Case(small_config(n=32, level=3))
    runs = []
    for graphs in (0, 1):
        c = case.clone()
        c.attach(gpu_lib)
        c.bind(gpu_lib)
        gpu_lib.mibm_set_graphs_(C.byref(C.c_int(graphs)))
        gpu_lib.mibm_set_precision_(C.byref(C.c_int(precision)), C.byref(C.c_int(2)))
        gpu_lib.check("setup")
        launches0 = gpu_lib.mibm_launch_count_()
        c.run(gpu_lib, 4)
        c.sync_to_host(gpu_lib, ALL)
        runs.append(({k: c.interior(f).copy() for k, f in FIELDS_OUT.items()},
                     c.mesh_arrays[A.MIBM_M_XYZV].copy(), c.S(A.MIBM_S_VOLUME),
                     gpu_lib.mibm_launch_count_() - launches0))
        c.detach(gpu_lib)
    (f0, x0, v0, n0), (f1, x1, v1, n1) = runs
    for k in FIELDS_OUT:
        assert np.array_equal(f0[k], f1[k]), k
    assert np.array_equal(x0, x1) and v0 == v1
    assert n0 == n1            # the graph's kernels are counted at every replay
