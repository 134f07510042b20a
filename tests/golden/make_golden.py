"""Regenerate tests/golden/*.json from the CPU oracle.

The reference publishes no golden vectors; these fixtures pin the oracle's
own output for a seeded 16^3 case (2 RK3 steps, config-0 physics on a
level-2 icosphere) so that the oracle built on another host (the Arm GPU
box) is checked against the one that produced the fixtures.
Run:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from melt_ibm_gb300 import abi  # noqa: E402
from melt_ibm_gb300.case import Case  # noqa: E402
import oracle  # noqa: E402
from tests.helpers import small_config  # noqa: E402


def main():
    lib = abi.Lib(oracle.build())
    c = Case(small_config(n=16, level=2))
    c.attach(lib)
    c.run(lib, 2)
    out = {}
    for name, fid in (("vx", abi.MIBM_F_VX), ("vy", abi.MIBM_F_VY), ("vz", abi.MIBM_F_VZ),
                      ("temp", abi.MIBM_F_TEMP), ("pr", abi.MIBM_F_PR)):
        a = c.interior(fid)
        out[name] = {"sum": float(np.sum(a)), "l2": float(np.sqrt(np.sum(a * a)))}
    out["dt"] = c.S(abi.MIBM_S_DT)
    out["volume"] = c.S(abi.MIBM_S_VOLUME)
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "oracle_c16_2steps.json")
    json.dump(out, open(path, "w"), indent=1)
    print(path)


if __name__ == "__main__":
    main()
