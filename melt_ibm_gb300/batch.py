"""Batched form: many independent cases advanced together through the C-ABI.

Each case is a `Case` attached to the library (its own context: any grid
size, FP64 or precision form, its own mesh and parameters).  `BatchRunner`
hands their context ids to `mibm_batch_create_` and advances all of them by
one iteration of the reference time loop per `step` (cfl, get_dt, forcing,
tschem for every case; gcurv.f90:151-172), with their device work
overlapped (see include/mibm.h).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import abi
from .case import Case


class BatchRunner:
    def __init__(self, lib: abi.Lib, cases: list[Case], autotune: bool = False):
        self.lib = lib
        self.cases = list(cases)
        if autotune:                  # shapes per (grid, form); repeated shapes hit the cache
            for c in self.cases:
                c.bind(lib)
                st = int(lib.mibm_autotune_())
                if st != 0:
                    raise RuntimeError(f"mibm_autotune_ failed ({st}): {lib.mibm_last_message().decode()}")
        ids = np.array([c.ctx[lib.path] for c in self.cases], dtype=np.int32)
        self._ids = ids
        self.handle = int(lib.mibm_batch_create_(ids.ctypes.data, abi.ref_int(len(ids))))
        if self.handle <= 0:
            raise RuntimeError(f"mibm_batch_create_ failed: {lib.mibm_last_message().decode()}")
        self.ntime = 1

    def step(self) -> None:
        st = int(self.lib.mibm_batch_step_(abi.ref_int(self.handle), abi.ref_int(self.ntime)))
        if st != 0:
            raise RuntimeError(f"mibm_batch_step_ failed ({st}): {self.lib.mibm_last_message().decode()}")
        self.ntime += 1

    def run(self, nsteps: int) -> None:
        for _ in range(nsteps):
            self.step()

    def close(self) -> None:
        if self.handle > 0:
            self.lib.mibm_batch_destroy_(abi.ref_int(self.handle))
            self.handle = 0

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
