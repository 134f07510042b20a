"""The reference's own mesh as a fixture (tests/golden/unitSphere_N3.npz,
written by tests/golden/make_mesh_fixture.py from gts/unitSphere_N3.gts).

The fixture must hold the counts of the reference file (642 vertices, 1920
edges, 1280 faces, partaux.f90:160-268), vertices on the unit sphere,
outward faces after the edge-walk ordering, and the same edge lengths as the
generated icosphere of the same level.  Where the reference checkout is
present, reading the file again must give the fixture bit for bit.
"""
from __future__ import annotations

import os

import numpy as np
import pytest

from melt_ibm_gb300.mesh import Mesh, icosphere, read_gts

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURE = os.path.join(HERE, "golden", "unitSphere_N3.npz")
REFERENCE_GTS = os.path.join(os.sep, "root", "reference", "gts", "unitSphere_N3.gts")


def reference_n3() -> Mesh:
    d = np.load(FIXTURE)
    return Mesh(xyz=d["xyz"], vert_of_face=d["vert_of_face"], vert_of_edge=d["vert_of_edge"],
                edge_of_face=d["edge_of_face"])


def test_fixture_is_the_level3_icosphere():
    m = reference_n3()
    assert (m.nv, m.ne, m.nf) == (642, 1920, 1280)
    r = np.linalg.norm(m.xyz, axis=1)
    assert np.abs(r - 1.0).max() < 1e-7
    f = m.vert_of_face - 1
    p1, p2, p3 = m.xyz[f[:, 0]], m.xyz[f[:, 1]], m.xyz[f[:, 2]]
    assert np.all(np.einsum("ij,ij->i", np.cross(p2 - p1, p3 - p1), p1 + p2 + p3) > 0)   # outward
    # every face's three edges join its three vertices
    e = m.vert_of_edge[m.edge_of_face - 1]
    for q in range(m.nf):
        assert set(e[q].ravel()) == set(m.vert_of_face[q])
    g = icosphere(3)
    le = np.sort(np.linalg.norm(m.xyz[m.vert_of_edge[:, 0] - 1] - m.xyz[m.vert_of_edge[:, 1] - 1], axis=1))
    lg = np.sort(np.linalg.norm(g.xyz[g.vert_of_edge[:, 0] - 1] - g.xyz[g.vert_of_edge[:, 1] - 1], axis=1))
    assert np.abs(le - lg).max() < 1e-7


@pytest.mark.skipif(not os.path.exists(REFERENCE_GTS), reason="reference checkout not present")
def test_fixture_equals_reference_file():
    m, r = reference_n3(), read_gts(REFERENCE_GTS)
    for a, b in ((m.xyz, r.xyz), (m.vert_of_face, r.vert_of_face), (m.vert_of_edge, r.vert_of_edge),
                 (m.edge_of_face, r.edge_of_face)):
        assert np.array_equal(a, b)
