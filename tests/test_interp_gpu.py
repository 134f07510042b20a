"""Restart regrid interp_ (interp.f90) on the GPU against the oracle."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from melt_ibm_gb300.case import Case
from tests.helpers import small_config

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("intvar", [1, 2, 3, 4])
@pytest.mark.parametrize("old", [(17, 17, 13), (33, 25, 29)])
def test_interp_parity(oracle_lib, gpu_lib, intvar, old):
    n1o, n2o, n3o = old
    case = Case(small_config(n=24, level=2))
    rng = np.random.default_rng(intvar)
    arr = rng.standard_normal((n3o + 2, n2o, n1o))         # (kstarto-1:kendo+1, n2o, n1o), x fastest
    results = []
    for lib in (oracle_lib, gpu_lib):
        c = case.clone()
        c.attach(lib, initial_tag=False)
        c.bind(lib)
        a = np.ascontiguousarray(arr.copy())
        out = np.zeros((c.n3m, c.n2m + 1, c.n1m + 1))
        ints = [C.c_int(v) for v in (n1o, n2o, n3o, intvar, 1, n3o)]
        lib.interp_(a.ctypes.data, out.ctypes.data, *[C.byref(v) for v in ints])
        lib.check("interp")
        results.append((a, out))
        c.detach(lib)
    (ao, no), (ag, ng) = results
    assert np.array_equal(ao, ag)            # the reference's in-place edits of the old array
    assert np.max(np.abs(ng - no)) <= 1e-14 * max(1.0, np.max(np.abs(no)))
    assert np.any(no != 0.0)
