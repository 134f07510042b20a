"""The allocation-free x-line solve against the existing solxi_.

mibm_solxi_noalloc serves callers that own every byte of device memory
(a CUDA Fortran / OpenACC host passing its own device arrays, or a process
whose HBM is reserved by a case pool) and so cannot let the library call
cudaMalloc.  The test gives it a device buffer it did not allocate and
checks that two calls in a row reproduce solxi_ on the same data, then that
an oversize line is refused without a launch.  Two more shapes go through the
paths that the small case does not reach, checked against the oracle's
solxi_: the longest line allowed (512 cells, whose shared-memory tile needs
the opt-in above 48 KB) and a row pitch wider than the line with more than
one block of rows (the padding between rows must come back untouched).
This file is collected last so that a run stopping at the first failure has
already run every other test.
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


@pytest.mark.parametrize("n1m, n2m, n3m, pitch", [(512, 2, 2, 512), (200, 40, 3, 208)])
def test_noalloc_solve_matches_oracle_at_limits(oracle_lib, gpu_lib, n1m, n2m, n3m, pitch):
    """Lines are independent, so the first n2m rows and n3m planes of the
    oracle's solve of an n1m x n1m x max(n3m, 4) case are the expected result
    of the n2m-row, n3m-plane call."""
    torch = pytest.importorskip("torch")
    case = Case(small_config(n=n1m, n3=max(n3m, 4), velocity="rest"))
    rng = np.random.default_rng(23 + n1m)
    rhs0 = rng.standard_normal(case.fields[abi.MIBM_F_RHS].shape)
    case.fields[abi.MIBM_F_RHS][...] = rhs0
    case.attach(oracle_lib, initial_tag=False)
    expect = {}
    for b in (0.37, 6.5):
        case.fields[abi.MIBM_F_RHS][...] = rhs0
        case.bind(oracle_lib)
        oracle_lib.solxi_(C.byref(C.c_double(b)))
        oracle_lib.check("solxi_")
        expect[b] = case.interior(abi.MIBM_F_RHS)[:, :n2m, :n3m].copy()
    case.detach(oracle_lib)

    # caller-owned buffer [k][j][pitch]: the row padding holds its own values
    buf_h = rng.standard_normal((n3m, n2m, pitch))
    buf_h[:, :, :n1m] = rhs0[:n1m, :n2m, :n3m].transpose(2, 1, 0)
    dev = torch.cuda.current_device()
    stream = torch.cuda.current_stream()
    for b in (0.37, 6.5):                              # two calls in a row
        buf = torch.from_numpy(buf_h.copy()).to(f"cuda:{dev}")
        st = gpu_lib.mibm_solxi_noalloc(C.c_void_p(buf.data_ptr()), n1m, n2m, n3m, pitch, b,
                                        C.c_void_p(stream.cuda_stream))
        assert st == abi.MIBM_OK
        torch.cuda.synchronize()
        out = buf.cpu().numpy()
        got = out[:, :, :n1m].transpose(2, 1, 0)
        assert rel_l2(got, expect[b]) <= 1e-12, (n1m, b)
        assert np.array_equal(out[:, :, n1m:], buf_h[:, :, n1m:])
