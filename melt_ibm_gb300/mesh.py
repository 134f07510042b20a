"""Triangulated surface input for the immersed boundary.

The reference reads a GTS file (header ``nv ne nf``, then vertices, edges as
vertex pairs, faces as edge triples) and rebuilds the face -> vertex table
from the edge table (partaux.f90:160-268, ``set_connectivity``).  This module
provides

* :func:`icosphere` -- a unit icosphere built from an icosahedron subdivided
  ``level`` times (10*4**n+2 vertices, 30*4**n edges, 20*4**n faces), the
  family the reference ships as ``gts/unitSphere_N{level}.gts``;
* :func:`read_gts` -- a reader for the reference's GTS format that applies the
  same ``set_connectivity`` edge-walk to order each face's vertices.

Both return a :class:`Mesh` with 1-based connectivity, the convention of the
Fortran arrays registered through the C-ABI.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


@dataclass
class Mesh:
    xyz: np.ndarray            # (nv, 3) float64
    vert_of_face: np.ndarray   # (nf, 3) int32, 1-based
    vert_of_edge: np.ndarray   # (ne, 2) int32, 1-based
    edge_of_face: np.ndarray   # (nf, 3) int32, 1-based

    @property
    def nv(self) -> int:
        return self.xyz.shape[0]

    @property
    def nf(self) -> int:
        return self.vert_of_face.shape[0]

    @property
    def ne(self) -> int:
        return self.vert_of_edge.shape[0]


def _edges_from_faces(faces0: np.ndarray):
    """Edge table and face->edge table from 0-based faces."""
    edge_id: dict[tuple[int, int], int] = {}
    voe = []
    eof = np.zeros_like(faces0)
    for f, (a, b, c) in enumerate(faces0):
        for q, (u, v) in enumerate(((a, b), (b, c), (c, a))):
            key = (min(u, v), max(u, v))
            if key not in edge_id:
                edge_id[key] = len(voe)
                voe.append(key)
            eof[f, q] = edge_id[key]
    return np.asarray(voe, dtype=np.int64), eof


def icosphere(level: int) -> Mesh:
    """Unit icosphere, outward-oriented faces (right-hand rule)."""
    t = (1.0 + 5.0 ** 0.5) / 2.0
    verts = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0),
             (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
             (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    verts = [np.asarray(v, dtype=np.float64) / np.linalg.norm(v) for v in verts]
    faces = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11),
             (1, 5, 9), (5, 11, 4), (11, 10, 2), (10, 7, 6), (7, 1, 8),
             (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9),
             (4, 9, 5), (2, 4, 11), (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    for _ in range(level):
        cache: dict[tuple[int, int], int] = {}

        def mid(a: int, b: int) -> int:
            key = (min(a, b), max(a, b))
            if key not in cache:
                m = verts[a] + verts[b]
                verts.append(m / np.linalg.norm(m))
                cache[key] = len(verts) - 1
            return cache[key]

        nxt = []
        for a, b, c in faces:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            nxt += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        faces = nxt
    xyz = np.asarray(verts, dtype=np.float64)
    f0 = np.asarray(faces, dtype=np.int64)
    # orient outward: (v2-v1)x(v3-v1) . centroid > 0
    e1 = xyz[f0[:, 1]] - xyz[f0[:, 0]]
    e2 = xyz[f0[:, 2]] - xyz[f0[:, 0]]
    flip = np.einsum("ij,ij->i", np.cross(e1, e2), xyz[f0].mean(axis=1)) < 0
    f0[flip] = f0[flip][:, ::-1]
    voe, eof = _edges_from_faces(f0)
    return Mesh(xyz=xyz, vert_of_face=(f0 + 1).astype(np.int32),
                vert_of_edge=(voe + 1).astype(np.int32),
                edge_of_face=(eof + 1).astype(np.int32))


def _set_connectivity(voe1: np.ndarray, eof1: np.ndarray) -> np.ndarray:
    """Face vertex order from the edge table (partaux.f90:192-219)."""
    nf = eof1.shape[0]
    vof = np.zeros((nf, 3), dtype=np.int32)
    for i in range(nf):
        e1, e2 = eof1[i, 0] - 1, eof1[i, 1] - 1
        a1, b1 = voe1[e1]
        a2, b2 = voe1[e2]
        if b1 == a2:
            v = (a1, b1, b2)
        elif b1 == b2:
            v = (a1, b1, a2)
        elif a1 == a2:
            v = (b1, a1, b2)
        else:
            v = (b1, a1, a2)
        vof[i] = v
    return vof


def read_gts(path: str) -> Mesh:
    """Read a GTS surface as the reference does (partaux.f90:160-219)."""
    with open(path) as fh:
        nv, ne, nf = (int(x) for x in fh.readline().split()[:3])
        xyz = np.array([[float(x) for x in fh.readline().split()[:3]] for _ in range(nv)])
        voe = np.array([[int(x) for x in fh.readline().split()[:2]] for _ in range(ne)], dtype=np.int32)
        eof = np.array([[int(x) for x in fh.readline().split()[:3]] for _ in range(nf)], dtype=np.int32)
    return Mesh(xyz=xyz, vert_of_face=_set_connectivity(voe, eof), vert_of_edge=voe, edge_of_face=eof)


def write_gts(mesh: Mesh, path: str) -> None:
    """Write a mesh in the GTS layout the reference reads."""
    with open(path, "w") as fh:
        fh.write(f"{mesh.nv} {mesh.ne} {mesh.nf}\n")
        for p in mesh.xyz:
            fh.write(f"{p[0]!r} {p[1]!r} {p[2]!r}\n")
        for e in mesh.vert_of_edge:
            fh.write(f"{e[0]} {e[1]}\n")
        for f in mesh.edge_of_face:
            fh.write(f"{f[0]} {f[1]} {f[2]}\n")
