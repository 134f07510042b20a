"""Regenerate tests/golden/unitSphere_N3.npz from the reference's own mesh.

The reference ships its surface meshes as GTS files; the plain configuration
uses gts/unitSphere_N3.gts (642 vertices, 1920 edges, 1280 faces, read by
partaux.f90:160-268).  This script reads that file with the package's GTS
reader (the reference's edge-walk face ordering, set_connectivity) and stores
the arrays, so that tests on machines without the reference checkout run the
configuration on the reference's mesh.
Run:  python tests/golden/make_mesh_fixture.py [reference checkout]
"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from melt_ibm_gb300.mesh import read_gts  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "unitSphere_N3.npz")


def main(ref: str) -> None:
    m = read_gts(os.path.join(ref, "gts", "unitSphere_N3.gts"))
    np.savez_compressed(OUT, xyz=m.xyz, vert_of_face=m.vert_of_face, vert_of_edge=m.vert_of_edge,
                        edge_of_face=m.edge_of_face)
    print(f"wrote {OUT}: {m.nv} vertices, {m.ne} edges, {m.nf} faces")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
