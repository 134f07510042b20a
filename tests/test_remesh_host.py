"""The library's remesher (remesh.cu: remesh_coarsen.f90 + remesh_smooth.f90,
host code) on jittered spheres, through mibm_remesh_mesh.  No GPU: the
remesher is host code of libmibm.so.

Checked, as the reference checks its own remeshing (remesh_coarsen.f90:89-
96, 196-202; particle.f90:205-213) and beyond: the call succeeds when a few
percent of the edges are below the threshold (what the per-substep trigger
hands it); the Euler characteristic stays 2; every live edge has two live
faces that contain it and its vertices, every live face three live edges
whose faces list it; the surface stays closed and consistently oriented,
with tri_nor along each face's winding; the volume is conserved to 1e-14
(absolute, the reference's abort threshold); the result is the same bits on
a second run; face_of_edge, kept by the caller, carries over to a further
call; and a mass collapse that the reference's single-relaxation volume
restore cannot absorb returns the residual code 3 instead of a broken mesh.
"""
from __future__ import annotations

import numpy as np
import pytest

from melt_ibm_gb300.mesh import icosphere


def _mesh(level, r, seed):
    m = icosphere(level)
    rng = np.random.default_rng(seed)
    x = (m.xyz * r).T.copy(order="F")
    x *= (1.0 + 0.02 * rng.standard_normal(m.nv))[None, :]
    x += 0.002 * rng.standard_normal(x.shape)
    vof = m.vert_of_face.T.copy(order="F")
    f = vof - 1
    p1, p2, p3 = x[:, f[0]], x[:, f[1]], x[:, f[2]]
    n = np.cross((p2 - p1).T, (p3 - p1).T).T
    n /= np.linalg.norm(n, axis=0)
    return dict(x=x, nor=np.asfortranarray(n), vm=np.asfortranarray(rng.standard_normal((3, m.nv))),
                el=np.zeros(m.ne), vof=vof, eof=m.edge_of_face.T.copy(order="F"),
                voe=m.vert_of_edge.T.copy(order="F"), foe=np.zeros((2, m.ne), np.int32, order="F"),
                gf=np.zeros(m.nf, np.int32), ge=np.zeros(m.ne, np.int32), gv=np.zeros(m.nv, np.int32)), m


def _edge_lengths(A):
    e = A["voe"] - 1
    return np.linalg.norm(A["x"][:, e[0]] - A["x"][:, e[1]], axis=0)


def _volume(A):
    f = A["vof"][:, A["gf"] == 0] - 1
    x = A["x"]
    p1, p2, p3 = x[:, f[0]], x[:, f[1]], x[:, f[2]]
    return float(np.einsum("ij,ij->j", p1, np.cross(p2.T, p3.T).T).sum() / 6.0)


def _remesh(lib, A, m, th):
    st = np.zeros(8)
    P = lambda a: a.ctypes.data
    rc = lib.mibm_remesh_mesh(m.nv, m.ne, m.nf, P(A["x"]), P(A["nor"]), P(A["vm"]), P(A["el"]), P(A["vof"]),
                              P(A["eof"]), P(A["voe"]), P(A["foe"]), P(A["gf"]), P(A["ge"]), P(A["gv"]), th, P(st))
    return rc, st


def check_mesh(A):
    """Closed, consistently oriented, consistent connectivity and normals."""
    gf, ge, gv = A["gf"], A["ge"], A["gv"]
    vof, eof, voe, foe = A["vof"], A["eof"], A["voe"], A["foe"]
    live_e, live_f = np.nonzero(ge == 0)[0], np.nonzero(gf == 0)[0]
    assert (gv == 0).sum() - len(live_e) + len(live_f) == 2
    for e in live_e:
        assert not gv[voe[0, e] - 1] and not gv[voe[1, e] - 1]
        for f in foe[:, e]:
            assert f > 0 and not gf[f - 1] and (e + 1) in eof[:, f - 1]
            assert set(voe[:, e]) <= set(vof[:, f - 1])
    directed = set()
    for f in live_f:
        for e in eof[:, f]:
            assert not ge[e - 1] and (f + 1) in foe[:, e - 1]
        a, b, c = vof[:, f]
        assert not (gv[a - 1] or gv[b - 1] or gv[c - 1])
        for u, w in ((a, b), (b, c), (c, a)):
            assert (u, w) not in directed
            directed.add((u, w))
    assert all((w, u) in directed for u, w in directed)
    x = A["x"]
    f = vof[:, live_f] - 1
    g = np.cross((x[:, f[1]] - x[:, f[0]]).T, (x[:, f[2]] - x[:, f[0]]).T)
    assert np.all(np.einsum("ij,ji->i", g, A["nor"][:, live_f]) > 0)


@pytest.mark.parametrize("level, r, q, seed", [(3, 0.5, 0.002, 0), (3, 0.5, 0.01, 1), (4, 0.4, 0.01, 0),
                                               (4, 0.4, 0.03, 1)])
def test_remesh_coarsens_and_conserves_volume(mibm_lib, level, r, q, seed):
    A, m = _mesh(level, r, seed)
    th = float(np.sort(_edge_lengths(A))[int(q * m.ne)])
    v0 = _volume(A)
    B = {k: v.copy(order="F") for k, v in A.items()}
    rc, st = _remesh(mibm_lib, A, m, th)
    assert rc == 0
    assert st[0] + st[1] > 0                                   # edges collapsed / vertices deleted
    check_mesh(A)
    assert abs(_volume(A) - v0) <= 1e-14
    assert abs(st[5] - st[3]) <= 1e-14                        # vol_smooth - vol_melt
    assert (A["ge"] == 0).sum() < m.ne                         # the mesh is coarser
    rc2, st2 = _remesh(mibm_lib, B, m, th)                    # same bits again
    assert rc2 == 0 and np.array_equal(st, st2)
    for k in A:
        assert np.array_equal(A[k], B[k]), k


def test_face_of_edge_carries_over_to_a_further_call(mibm_lib):
    A, m = _mesh(4, 0.4, 3)
    el = np.sort(_edge_lengths(A))
    assert _remesh(mibm_lib, A, m, float(el[int(0.005 * m.ne)]))[0] == 0
    assert A["foe"][:, A["ge"] == 0].min() > 0
    # the body shrinks a little (melting); the next call starts from the kept face_of_edge
    A["x"] *= 0.985
    live = A["ge"] == 0
    th = float(np.sort(_edge_lengths(A)[live])[int(0.005 * live.sum())])
    v0 = _volume(A)
    rc, st = _remesh(mibm_lib, A, m, th)
    assert rc == 0 and st[0] + st[1] > 0
    check_mesh(A)
    assert abs(_volume(A) - v0) <= 1e-14


def test_mass_collapse_reports_the_residual_abort(mibm_lib):
    A, m = _mesh(3, 0.5, 0)
    th = float(np.sort(_edge_lengths(A))[int(0.03 * m.ne)])
    rc, st = _remesh(mibm_lib, A, m, th)
    assert rc == 3 and abs(st[5] - st[3]) > 1e-14
    assert (A["gv"] == 0).sum() - (A["ge"] == 0).sum() + (A["gf"] == 0).sum() == 2
