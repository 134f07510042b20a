"""Batched form: every case of a batch gets exactly the result of stepping
it alone (uneven grids, both forms, forcing), and the GPU batch matches the
oracle's."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from melt_ibm_gb300 import abi
from melt_ibm_gb300.batch import BatchRunner
from melt_ibm_gb300.case import Case
from tests.helpers import FIELDS_OUT, rel_l2, small_config

pytestmark = pytest.mark.gpu
ALL = -1


def _cases():
    return [Case(small_config(n=16, level=2, seed=1)),
            Case(small_config(n=24, level=2, seed=2, latheat=2.0)),
            Case(small_config(n=32, level=3, seed=3, forcing=1, which_hit=1, hit_seed=4)),
            Case(small_config(n=24, level=2, seed=5, imelt=0))]


def _attach(case, lib, precision):
    c = case.clone()
    c.attach(lib)
    c.bind(lib)
    lib.mibm_set_precision_(C.byref(C.c_int(precision)), C.byref(C.c_int(2)))
    return c


def _state(c, lib):
    c.sync_to_host(lib, ALL)
    return ({k: c.interior(f).copy() for k, f in FIELDS_OUT.items()}, c.mesh_arrays[abi.MIBM_M_XYZV].copy(),
            c.S(abi.MIBM_S_DT), c.S(abi.MIBM_S_TIME))


@pytest.mark.parametrize("precision", [0, 1])
def test_batch_equals_cases_stepped_alone(gpu_lib, precision):
    nsteps = 4
    alone = []
    for case in _cases():
        c = _attach(case, gpu_lib, precision)
        c.run(gpu_lib, nsteps)
        alone.append(_state(c, gpu_lib))
        c.detach(gpu_lib)
    batch_cases = [_attach(case, gpu_lib, precision) for case in _cases()]
    with BatchRunner(gpu_lib, batch_cases) as b:
        b.run(nsteps)
    for q, c in enumerate(batch_cases):
        f, x, dt, t = _state(c, gpu_lib)
        fa, xa, dta, ta = alone[q]
        for k in FIELDS_OUT:
            assert np.array_equal(f[k], fa[k]), (q, k)
        assert np.array_equal(x, xa) and dt == dta and t == ta, q
        c.detach(gpu_lib)


def test_batch_matches_oracle(oracle_lib, gpu_lib):
    nsteps = 3
    res = {}
    for lib in (oracle_lib, gpu_lib):
        cs = [_attach(case, lib, 0) for case in _cases()]
        with BatchRunner(lib, cs) as b:
            b.run(nsteps)
        res[lib.path] = [_state(c, lib) if lib is gpu_lib else
                         ({k: c.interior(f).copy() for k, f in FIELDS_OUT.items()}, None, c.S(abi.MIBM_S_DT), None)
                         for c in cs]
        for c in cs:
            c.detach(lib)
    for (fo, _, dto, _), (fg, _, dtg, _) in zip(res[oracle_lib.path], res[gpu_lib.path]):
        for k in FIELDS_OUT:
            assert rel_l2(fg[k], fo[k]) <= 1e-10, k
        assert dtg == pytest.approx(dto, rel=1e-12)


def test_autotune_keeps_state_and_parity(oracle_lib, gpu_lib, tmp_path):
    case = Case(small_config(n=32, level=3, seed=7))
    cg = case.clone()
    cg.attach(gpu_lib)
    before, *_ = _state(cg, gpu_lib)
    cg.bind(gpu_lib)
    assert gpu_lib.mibm_autotune_() == 0
    shapes = np.zeros(4, dtype=np.int32)
    gpu_lib.mibm_autotune_get_(shapes.ctypes.data)
    assert all(32 % m == 0 for m in shapes[:3]) and shapes[3] in (2, 4, 8)
    after, *_ = _state(cg, gpu_lib)
    for k in FIELDS_OUT:
        assert np.array_equal(before[k], after[k]), k        # tuning ran on scratch data
    path = str(tmp_path / "tune.txt").encode()
    assert gpu_lib.mibm_autotune_save_(path) == 0 and gpu_lib.mibm_autotune_load_(path) == 0
    co = case.clone()
    co.attach(oracle_lib)
    co.run(oracle_lib, 3)
    cg.run(gpu_lib, 3)
    got, *_ = _state(cg, gpu_lib)
    for k, f in FIELDS_OUT.items():
        assert rel_l2(got[k], co.interior(f)) <= 1e-10, k
    cg.detach(gpu_lib)
    co.detach(oracle_lib)


def test_autotuned_batch_equals_cases_alone(gpu_lib):
    nsteps = 3
    cases = _cases()
    alone = []
    for case in cases:
        c = _attach(case, gpu_lib, 1)
        assert gpu_lib.mibm_autotune_() == 0
        c.run(gpu_lib, nsteps)
        alone.append(_state(c, gpu_lib))
        c.detach(gpu_lib)
    bc = [_attach(case, gpu_lib, 1) for case in cases]
    with BatchRunner(gpu_lib, bc, autotune=True) as b:
        b.run(nsteps)
    for q, c in enumerate(bc):
        f, x, dt, t = _state(c, gpu_lib)
        for k in FIELDS_OUT:
            assert np.array_equal(f[k], alone[q][0][k]), (q, k)
        c.detach(gpu_lib)
