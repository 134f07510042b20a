"""HIT forcing (hit.f90) on the GPU against the oracle.

Eswaran-Pope forcing: the mode amplitudes bhat (host O-U update, the
library's documented random stream) must be bitwise equal, the forcing
fields (device DFT sums, summed in a different order) equal to round-off;
ABC and the linear-forcing extension likewise; and a forced RK3 run matches
the oracle at the plain-form tolerance.
"""
from __future__ import annotations

import numpy as np
import pytest

from melt_ibm_gb300 import abi
from melt_ibm_gb300.case import Case
from tests.helpers import FIELDS_OUT, pair, randomize, rel_l2, small_config

pytestmark = pytest.mark.gpu
FORC = (abi.MIBM_F_FORCX, abi.MIBM_F_FORCY, abi.MIBM_F_FORCZ)
ALL = -1


def _bhat(c, lib):
    c.bind(lib)
    nm = lib.mibm_hit_modes_()
    b = np.zeros(2 * 3 * nm ** 3)
    lib.mibm_hit_bhat_(b.ctypes.data, abi.ref_int(0))
    lib.check("bhat")
    return b


@pytest.mark.parametrize("calls", [1, 4])
def test_eswaran_pope_forcing_parity(oracle_lib, gpu_lib, calls):
    case = Case(small_config(n=24, level=2, forcing=1, which_hit=1, hit_seed=5))
    co, cg = pair(case, oracle_lib, gpu_lib, initial_tag=False)
    for c, lib in ((co, oracle_lib), (cg, gpu_lib)):
        c.bind(lib)
        for _ in range(calls):
            lib.calchitrandomforce_()
        lib.check("hit")
    cg.sync_to_host(gpu_lib, ALL)
    assert np.array_equal(_bhat(co, oracle_lib), _bhat(cg, gpu_lib))
    for fid in FORC:
        ref = co.interior(fid)
        assert np.max(np.abs(cg.interior(fid) - ref)) <= 1e-13 * max(1.0, np.max(np.abs(ref))), fid


def test_bhat_round_trip(gpu_lib):
    case = Case(small_config(n=16, level=2, forcing=1, which_hit=1, hit_seed=9))
    c = case.clone()
    c.attach(gpu_lib, initial_tag=False)
    c.bind(gpu_lib)
    gpu_lib.calchitrandomforce_()
    b = _bhat(c, gpu_lib)
    assert np.any(b != 0.0)
    b2 = 2.0 * b                       # keep the array alive across the call
    gpu_lib.mibm_hit_bhat_(b2.ctypes.data, abi.ref_int(1))
    assert np.array_equal(_bhat(c, gpu_lib), b2)
    c.detach(gpu_lib)


@pytest.mark.parametrize("which", [2, 3])
def test_abc_and_linear_forcing_parity(oracle_lib, gpu_lib, which):
    case = Case(small_config(n=24, level=2, forcing=1, which_hit=which, c_hit=0.2))
    randomize(case)
    co, cg = pair(case, oracle_lib, gpu_lib, initial_tag=False)
    for c, lib in ((co, oracle_lib), (cg, gpu_lib)):
        c.bind(lib)
        (lib.calcabc_hitforce_ if which == 2 else lib.mibm_linear_hit_force_)()
        lib.check("forcing")
    cg.sync_to_host(gpu_lib, ALL)
    for fid in FORC:
        ref = co.interior(fid)
        assert np.max(np.abs(cg.interior(fid) - ref)) <= 1e-14 * max(1.0, np.max(np.abs(ref))), fid


@pytest.mark.parametrize("which", [1, 3])
def test_forced_steps_parity(oracle_lib, gpu_lib, which):
    case = Case(small_config(n=24, level=2, forcing=1, which_hit=which, hit_seed=3, epsstar=0.5, c_hit=0.05))
    co, cg = pair(case, oracle_lib, gpu_lib)
    co.run(oracle_lib, 3)
    cg.run(gpu_lib, 3)
    cg.sync_to_host(gpu_lib, ALL)
    for name, fid in FIELDS_OUT.items():
        assert rel_l2(cg.interior(fid), co.interior(fid)) <= 1e-10, name
    for fid in FORC:
        assert np.max(np.abs(co.interior(fid))) > 0.0
