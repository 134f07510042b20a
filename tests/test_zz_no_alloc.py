"""The allocation-free x-line solve against the existing solxi_.

mibm_solxi_noalloc serves callers that own every byte of device memory
(a CUDA Fortran / OpenACC host passing its own device arrays, or a process
whose HBM is reserved by a case pool) and so cannot let the library call
cudaMalloc.  The test gives it a device buffer it did not allocate and
checks that two calls in a row reproduce solxi_ on the same data, then that
an oversize line is refused without a launch.  This file is collected last
so that a run stopping at the first failure has already run every other test.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from melt_ibm_gb300 import abi
from melt_ibm_gb300.case import Case
from tests.helpers import randomize, rel_l2, small_config

pytestmark = pytest.mark.gpu


def _reference(lib, case, rhs0, betadx):
    """solxi_ on the registered RHS field of a context (the existing path)."""
    case.fields[abi.MIBM_F_RHS][...] = rhs0
    case.sync_from_host(lib, 1 << abi.MIBM_F_RHS)
    case.bind(lib)
    lib.solxi_(C.byref(C.c_double(betadx)))
    lib.check("solxi_")
    case.sync_to_host(lib, 1 << abi.MIBM_F_RHS)
    return case.interior(abi.MIBM_F_RHS).copy()


def test_noalloc_solve_matches_solxi(gpu_lib):
    torch = pytest.importorskip("torch")
    n = 24
    case = Case(small_config(n=n))
    randomize(case)
    rng = np.random.default_rng(17)
    rhs0 = rng.standard_normal(case.fields[abi.MIBM_F_RHS].shape)
    case.attach(gpu_lib, initial_tag=False)
    betas = (0.37, 6.5)
    refs = [_reference(gpu_lib, case, rhs0, b) for b in betas]
    case.detach(gpu_lib)

    # a device buffer owned by the caller, compact layout [k][j][i], pitch n
    interior = np.asfortranarray(rhs0)[:n, :n, :n]
    compact = np.ascontiguousarray(interior.transpose(2, 1, 0))
    dev = torch.cuda.current_device()
    stream = torch.cuda.current_stream()
    outs = []
    for b in betas:                                   # two calls in a row
        buf = torch.from_numpy(compact.copy()).to(f"cuda:{dev}")
        st = gpu_lib.mibm_solxi_noalloc(C.c_void_p(buf.data_ptr()), n, n, n, n, b,
                                        C.c_void_p(stream.cuda_stream))
        assert st == abi.MIBM_OK
        torch.cuda.synchronize()
        outs.append(buf.cpu().numpy().transpose(2, 1, 0))
    for got, ref in zip(outs, refs):
        assert rel_l2(got, ref) <= 1e-12

    big = torch.zeros(8, device=f"cuda:{dev}", dtype=torch.float64)
    st = gpu_lib.mibm_solxi_noalloc(C.c_void_p(big.data_ptr()), 1024, 1, 1, 1024, 0.5,
                                    C.c_void_p(stream.cuda_stream))
    assert st == abi.MIBM_EINVAL
    assert torch.count_nonzero(big).item() == 0
