// remesh.cu -- the reference's remesher, host code: quadric-error-metric edge
// collapses (remesh_coarsen.f90:2-258 with its helpers :260-760) and
// volume-conserving edge relaxation (remesh_smooth.f90:3-474, Kuprat et al.
// 2001, algorithm 4, as reframed by Rohair et al. 2016), called from
// particle.f90:119-160 when an edge is shorter than E_thresh.
//
// This is host code of the library, as the remesher is host code of the
// reference: sequential, branchy topology edits that run a handful of times
// per simulation.  Two entry points:
//   mibm_remesh_mesh      plain arrays (the reference's Fortran layouts and
//                         1-based indices) and a caller-owned face_of_edge;
//   mibm_remesh_builtin_  the remesh callback form (mibm_set_remesh_callback_)
//                         on the bound context's registered host arrays,
//                         with face_of_edge kept per context id.
// Every operation follows the reference's loops in their order (IEEE double,
// compiled without contraction), so a run that hands the same mesh to it
// gets the same mesh back.
//
// The reference's limits are kept: an edge collapse does not check the link
// condition, so collapsing an edge whose ends share a third neighbour leaves
// a vertex of valence 2, on which the next neighbour walk stops the run
// (remesh_smooth.f90:419-425; code 5 here); and the whole volume lost by
// coarsening is restored by the first edge relaxation, with a sign taken
// from the local smoothing move, so a call that coarsens a large part of the
// surface at once can miss the 1e-14 volume residual (code 3, the
// reference's abort of particle.f90:205-213).
//
// Where the reference leaves a value undefined, this restatement fixes it:
// the list of faces whose normals are refreshed starts empty (the
// reference's local `flagged_faces` is uninitialised before the first
// vertex deletion, remesh_coarsen.f90:85-86), and vol_melt is the volume of
// the mesh handed over, evaluated here (the reference's is that of the mesh
// after the Stefan update, particle.f90:92, the same mesh for a body that
// does not move).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <vector>

#include "common.cuh"

namespace mibm {

namespace {

constexpr int kRing = 30;          // neighbour buffers (remesh_coarsen.f90:18-19)

// return codes (the reference's aborts and stops)
enum RemeshStatus {
  kRemeshOk = 0,
  kRemeshTopology = 1,     // Euler characteristic != 2 (remesh_coarsen.f90:89-96)
  kRemeshTetrahedron = 2,  // reduced to a tetrahedron (:196-202)
  kRemeshResidual = 3,     // |vol_melt - vol_smooth| > 1e-14 (particle.f90:205-213)
  kRemeshQem = 4,          // singular QEM system (remesh_coarsen.f90:334-337)
  kRemeshWalk = 5,         // neighbour walk failed / buffer exceeded (remesh_smooth.f90:399-425, 465-473)
  kRemeshArgs = 6,
};

struct Mesh {
  int nv, ne, nf;
  double* xyz;        // (3, nv)
  double* tri_nor;    // (3, nf)
  double* vmelt;      // (3, nv)
  double* elen;       // (ne)
  int* vof;           // (3, nf)
  int* eof;           // (3, nf)
  int* voe;           // (2, ne)
  int* foe;           // (2, ne)
  int* gf;            // (nf) ghost flags
  int* ge;            // (ne)
  int* gv;            // (nv)
  double& X(int d, int v) { return xyz[(d - 1) + 3 * (size_t)(v - 1)]; }
  double& N(int d, int f) { return tri_nor[(d - 1) + 3 * (size_t)(f - 1)]; }
  double& VM(int d, int v) { return vmelt[(d - 1) + 3 * (size_t)(v - 1)]; }
  int& VOF(int q, int f) { return vof[(q - 1) + 3 * (size_t)(f - 1)]; }
  int& EOF_(int q, int f) { return eof[(q - 1) + 3 * (size_t)(f - 1)]; }
  int& VOE(int q, int e) { return voe[(q - 1) + 2 * (size_t)(e - 1)]; }
  int& FOE(int q, int e) { return foe[(q - 1) + 2 * (size_t)(e - 1)]; }
  bool GF(int f) const { return gf[f - 1] != 0; }
  bool GE(int e) const { return ge[e - 1] != 0; }
  bool GV(int v) const { return gv[v - 1] != 0; }
};

struct Walk {
  int status = kRemeshOk;
};

void cross(double r[3], const double x[3], const double y[3]) {   // triaux.f90:385-393
  r[0] = x[1] * y[2] - y[1] * x[2];
  r[1] = x[2] * y[0] - y[2] * x[0];
  r[2] = x[0] * y[1] - y[0] * x[1];
}

double norm2_3(const double a[3]) { return std::sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]); }

// face_of_edge as partaux.f90:221-245 builds it: faces in ascending order,
// first free slot
void build_face_of_edge(Mesh& m) {
  for (int e = 1; e <= m.ne; ++e) m.FOE(1, e) = m.FOE(2, e) = 0;
  for (int i = 1; i <= m.nf; ++i) {
    if (m.GF(i)) continue;
    for (int q = 1; q <= 3; ++q) {
      const int e = m.EOF_(q, i);
      if (m.FOE(1, e) == 0) m.FOE(1, e) = i;
      else if (m.FOE(2, e) == 0) m.FOE(2, e) = i;
    }
  }
}

// A kept face_of_edge is used as it is if it still describes the mesh: every
// live edge lists two live faces that contain it, and every live face is
// listed by its three edges (else it is rebuilt, e.g. on a first call or
// after the host replaced the mesh).
bool face_of_edge_consistent(Mesh& m) {
  for (int e = 1; e <= m.ne; ++e) {
    if (m.GE(e)) continue;
    for (int q = 1; q <= 2; ++q) {
      const int f = m.FOE(q, e);
      if (f < 1 || f > m.nf || m.GF(f)) return false;
      if (m.EOF_(1, f) != e && m.EOF_(2, f) != e && m.EOF_(3, f) != e) return false;
    }
    if (m.FOE(1, e) == m.FOE(2, e)) return false;
  }
  for (int f = 1; f <= m.nf; ++f) {
    if (m.GF(f)) continue;
    for (int q = 1; q <= 3; ++q) {
      const int e = m.EOF_(q, f);
      if (e < 1 || e > m.ne || m.GE(e) || (m.FOE(1, e) != f && m.FOE(2, e) != f)) return false;
    }
  }
  return true;
}

// calculate_volume, triaux.f90:53-79
double calculate_volume(Mesh& m) {
  double Volume = 0.0;
  for (int i = 1; i <= m.nf; ++i) {
    if (m.GF(i)) continue;
    const int v1 = m.VOF(1, i), v2 = m.VOF(2, i), v3 = m.VOF(3, i);
    const double vol = m.X(1, v1) * (m.X(2, v2) * m.X(3, v3) - m.X(3, v2) * m.X(2, v3)) +
                       m.X(1, v2) * (m.X(2, v3) * m.X(3, v1) - m.X(3, v3) * m.X(2, v1)) +
                       m.X(1, v3) * (m.X(2, v1) * m.X(3, v2) - m.X(3, v1) * m.X(2, v2));
    Volume = Volume + vol;
  }
  return Volume / 6.0;
}

// calculate_eLengths, triaux.f90:277-305; returns rm_flag
bool calculate_elengths(Mesh& m, double thresh) {
  bool rm = false;
  for (int i = 1; i <= m.ne; ++i) {
    if (m.GE(i)) continue;
    const int v1 = m.VOE(1, i), v2 = m.VOE(2, i);
    const double a = m.X(1, v1) - m.X(1, v2), b = m.X(2, v1) - m.X(2, v2), c = m.X(3, v1) - m.X(3, v2);
    m.elen[i - 1] = std::sqrt(a * a + b * b + c * c);
    if (m.elen[i - 1] < thresh) rm = true;
  }
  return rm;
}

int euler_number(const Mesh& m) {
  int v = 0, e = 0, f = 0;
  for (int i = 0; i < m.nv; ++i) v += m.gv[i] == 0;
  for (int i = 0; i < m.ne; ++i) e += m.ge[i] == 0;
  for (int i = 0; i < m.nf; ++i) f += m.gf[i] == 0;
  return v - e + f;
}

int live_faces(const Mesh& m) {
  int f = 0;
  for (int i = 0; i < m.nf; ++i) f += m.gf[i] == 0;
  return f;
}

// get_next_edge_of_v (remesh_coarsen.f90:423-450) / get_next_edge
// (remesh_smooth.f90:443-474): the last edge of currentFace, other than
// prevEdge, that joins v
int next_edge_of_v(Mesh& m, int v, int currentFace, int prevEdge, Walk& w) {
  int next = -1;
  for (int i = 1; i <= 3; ++i) {
    const int e = m.EOF_(i, currentFace);
    if (e != prevEdge && (m.VOE(1, e) == v || m.VOE(2, e) == v)) next = e;
  }
  if (next < 0) w.status = kRemeshWalk;
  return next;
}

// the face of prevEdge that is not prevFace
int other_face(Mesh& m, int prevEdge, int prevFace) {
  return m.FOE(1, prevEdge) != prevFace ? m.FOE(1, prevEdge) : m.FOE(2, prevEdge);
}

// get_vertNeighbours, remesh_smooth.f90:349-441
int vert_neighbours(Mesh& m, int v, int e, bool reverse, int nb[kRing], Walk& w) {
  for (int q = 0; q < kRing; ++q) nb[q] = 0;
  const int F1 = m.FOE(1, e);
  int prevFace = F1, currentEdge = 0, prevEdge = e;
  int num = 1;
  nb[0] = m.VOE(1, e) == v ? m.VOE(2, e) : m.VOE(1, e);
  while (currentEdge != e) {
    const int currentFace = other_face(m, prevEdge, prevFace);
    if (currentFace == F1) break;
    ++num;
    if (num > kRing) { w.status = kRemeshWalk; return num; }
    currentEdge = next_edge_of_v(m, v, currentFace, prevEdge, w);
    if (w.status != kRemeshOk) return num;
    nb[num - 1] = m.VOE(1, currentEdge) == v ? m.VOE(2, currentEdge) : m.VOE(1, currentEdge);
    prevFace = currentFace;
    prevEdge = currentEdge;
  }
  if (num < 3) { w.status = kRemeshWalk; return num; }
  if (reverse)   // v_neighbours(2:num) = v_neighbours(num:2:-1)
    for (int a = 1, b = num - 1; a < b; ++a, --b) std::swap(nb[a], nb[b]);
  return num;
}

// get_edge_face_1ring, remesh_coarsen.f90:515-579
void edge_face_1ring(Mesh& m, int v, int e, int en[kRing], int fn[kRing], int& cnt_en, int& cnt_f, Walk& w) {
  for (int q = 0; q < kRing; ++q) en[q] = fn[q] = 0;
  cnt_en = 1;
  en[0] = e;
  const int F1 = m.FOE(1, e);
  int prevFace = F1, currentEdge = 0, prevEdge = e;
  cnt_f = 1;
  fn[0] = F1;
  while (currentEdge != e) {
    const int currentFace = other_face(m, prevEdge, prevFace);
    if (currentFace == F1) break;
    if (cnt_f >= kRing || cnt_en >= kRing) { w.status = kRemeshWalk; return; }
    fn[cnt_f++] = currentFace;
    currentEdge = next_edge_of_v(m, v, currentFace, prevEdge, w);
    if (w.status != kRemeshOk) return;
    en[cnt_en++] = currentEdge;
    prevFace = currentFace;
    prevEdge = currentEdge;
  }
}

// flag_neighbours_1ring, remesh_coarsen.f90:454-513: un-anchor the 1-ring of
// v, flag its edges for smoothing and list its faces
void flag_neighbours_1ring(Mesh& m, std::vector<char>& anchor, std::vector<char>& flagged_edge,
                           int flagged_faces[kRing], int v, int e, Walk& w) {
  anchor[v - 1] = 0;
  flagged_edge[e - 1] = 1;
  for (int q = 0; q < kRing; ++q) flagged_faces[q] = 0;
  const int F1 = m.FOE(1, e);
  int prevFace = F1, currentEdge = 0, prevEdge = e;
  int cnt_f = 1;
  flagged_faces[0] = F1;
  while (currentEdge != e) {
    const int currentFace = other_face(m, prevEdge, prevFace);
    if (currentFace == F1) break;
    if (cnt_f >= kRing) { w.status = kRemeshWalk; return; }
    flagged_faces[cnt_f++] = currentFace;
    currentEdge = next_edge_of_v(m, v, currentFace, prevEdge, w);
    if (w.status != kRemeshOk) return;
    anchor[m.VOE(1, currentEdge) - 1] = 0;
    anchor[m.VOE(2, currentEdge) - 1] = 0;
    flagged_edge[currentEdge - 1] = 1;
    prevFace = currentFace;
    prevEdge = currentEdge;
  }
}

// update_1ring_normals, remesh_coarsen.f90:581-633: recompute the normals of
// the listed live faces; a normal that turned over flips the face's winding
// and keeps its old orientation
void update_1ring_normals(Mesh& m, const int flagged_faces[kRing]) {
  for (int cnt = 0; cnt < kRing && flagged_faces[cnt] != 0; ++cnt) {
    const int i = flagged_faces[cnt];
    if (m.GF(i)) continue;
    const double old[3] = {m.N(1, i), m.N(2, i), m.N(3, i)};
    const int v1 = m.VOF(1, i), v2 = m.VOF(2, i), v3 = m.VOF(3, i);
    double ve1[3], ve2[3];
    for (int d = 1; d <= 3; ++d) {
      ve1[d - 1] = m.X(d, v2) - m.X(d, v1);
      ve2[d - 1] = m.X(d, v3) - m.X(d, v1);
    }
    double n[3];
    n[0] = ve1[1] * ve2[2] - ve1[2] * ve2[1];
    n[1] = ve1[2] * ve2[0] - ve1[0] * ve2[2];
    n[2] = ve1[0] * ve2[1] - ve1[1] * ve2[0];
    const double s = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
    for (int d = 0; d < 3; ++d) n[d] = n[d] / s;
    double sgn = n[0] * old[0] + n[1] * old[1] + n[2] * old[2];
    if (sgn < 0.0) std::swap(m.VOF(1, i), m.VOF(3, i));    // vert_of_face(3:1:-1, i)
    sgn = std::copysign(1.0, sgn);
    for (int d = 1; d <= 3; ++d) m.N(d, i) = n[d - 1] * sgn;
  }
}

// calc_errorQuadric_of_v, remesh_coarsen.f90:260-316: Q += p p^T over the
// faces around v (Garland & Heckbert 1997, eq. 2), p = [n, -n.x_v] / |.|
void error_quadric(Mesh& m, double Q[16], int v, int e, Walk& w) {
  auto add = [&](int f) {
    double p[4] = {m.N(1, f), m.N(2, f), m.N(3, f), 0.0};
    p[3] = -(m.N(1, f) * m.X(1, v) + m.N(2, f) * m.X(2, v) + m.N(3, f) * m.X(3, v));
    const double s = std::sqrt(p[0] * p[0] + p[1] * p[1] + p[2] * p[2] + p[3] * p[3]);
    for (int q = 0; q < 4; ++q) p[q] = p[q] / s;
    for (int c = 0; c < 4; ++c)             // DGEMM('N','T',4,4,1,1,p,4,p,4,1,Q,4)
      for (int r = 0; r < 4; ++r) Q[r + 4 * c] = Q[r + 4 * c] + p[r] * p[c];
  };
  const int F1 = m.FOE(1, e);
  int prevFace = F1, currentEdge = 0, prevEdge = e;
  add(F1);
  while (currentEdge != e) {
    const int currentFace = other_face(m, prevEdge, prevFace);
    if (currentFace == F1) break;
    add(currentFace);
    currentEdge = next_edge_of_v(m, v, currentFace, prevEdge, w);
    if (w.status != kRemeshOk) return;
    prevFace = currentFace;
    prevEdge = currentEdge;
  }
}

// solve_QEM_system, remesh_coarsen.f90:318-341: (Q1 + Q2) with its last row
// replaced by [0 0 0 1], solved against [0 0 0 1] by LU with partial
// pivoting (dgesv); the first three entries are the new position
bool solve_qem(const double Q1[16], const double Q2[16], double out[3]) {
  double a[16], b[4] = {0.0, 0.0, 0.0, 1.0};
  for (int q = 0; q < 16; ++q) a[q] = Q1[q] + Q2[q];
  for (int c = 0; c < 4; ++c) a[3 + 4 * c] = c == 3 ? 1.0 : 0.0;
  int piv[4];
  for (int j = 0; j < 4; ++j) {            // dgetrf (unblocked), first maximal pivot
    int p = j;
    double amax = std::fabs(a[j + 4 * j]);
    for (int i = j + 1; i < 4; ++i)
      if (std::fabs(a[i + 4 * j]) > amax) { amax = std::fabs(a[i + 4 * j]); p = i; }
    piv[j] = p;
    if (a[p + 4 * j] == 0.0) return false;
    if (p != j)
      for (int c = 0; c < 4; ++c) std::swap(a[j + 4 * c], a[p + 4 * c]);
    const double r = 1.0 / a[j + 4 * j];
    for (int i = j + 1; i < 4; ++i) a[i + 4 * j] *= r;
    for (int c = j + 1; c < 4; ++c) {
      const double t = a[j + 4 * c];
      if (t != 0.0)
        for (int i = j + 1; i < 4; ++i) a[i + 4 * c] -= t * a[i + 4 * j];
    }
  }
  for (int j = 0; j < 4; ++j)              // dgetrs: row interchanges, L (unit), U
    if (piv[j] != j) std::swap(b[j], b[piv[j]]);
  for (int j = 0; j < 4; ++j)
    if (b[j] != 0.0)
      for (int i = j + 1; i < 4; ++i) b[i] -= b[j] * a[i + 4 * j];
  for (int j = 3; j >= 0; --j)
    if (b[j] != 0.0) {
      b[j] = b[j] / a[j + 4 * j];
      for (int i = 0; i < j; ++i) b[i] -= b[j] * a[i + 4 * j];
    }
  out[0] = b[0]; out[1] = b[1]; out[2] = b[2];
  return true;
}

// get_ghost_and_retained_edges, remesh_coarsen.f90:344-366
void ghost_and_retained(Mesh& m, int f, int e, int& ghost, int& retained) {
  int buf[3] = {0, 0, 0}, cnt = 0;
  for (int i = 1; i <= 3; ++i)
    if (m.EOF_(i, f) != e) buf[cnt++] = m.EOF_(i, f);
  ghost = buf[0];
  retained = buf[1];
}

// update_face_connectivity + update_edge_connectivity, remesh_coarsen.f90:368-421
void update_connectivity_collapse(Mesh& m, int v1, int v2, int e1, int e2, int re1, int re2, int F1, int F2) {
  for (int i = 0; i < 3 * m.nf; ++i) if (m.vof[i] == v2) m.vof[i] = v1;
  for (int i = 0; i < 3 * m.nf; ++i) if (m.eof[i] == e1) m.eof[i] = re1;
  for (int i = 0; i < 3 * m.nf; ++i) if (m.eof[i] == e2) m.eof[i] = re2;
  for (int i = 0; i < 2 * m.ne; ++i) if (m.voe[i] == v2) m.voe[i] = v1;
  auto merge = [&](int eg, int er, int F) {
    const int fb[4] = {m.FOE(1, eg), m.FOE(2, eg), m.FOE(1, er), m.FOE(2, er)};
    int cnt = 1;
    for (int i = 0; i < 4; ++i)
      if (fb[i] != F && cnt <= 2) m.FOE(cnt++, er) = fb[i];
  };
  merge(e1, re1, F1);
  merge(e2, re2, F2);
}

// update_connectivity_vert_deletion, remesh_coarsen.f90:637-760: the
// valence-3 vertex v1 goes with the edge e; of its faces fL (kept), fR, f3
// (ghosted) and edges e1, e2 (ghosted); fL becomes {v2, v3, v4}
int vert_deletion(Mesh& m, int v1, int v2, int e, const int en[kRing], const int fn[kRing], const int vn[kRing],
                  int cnt_en, int cnt_fn, int cnt_vn) {
  int local_e[2] = {0, 0}, incr = 0;
  for (int i = 0; i < cnt_en; ++i) {
    if (en[i] == e) continue;
    if (incr < 2) local_e[incr] = en[i];
    ++incr;
  }
  const int e1 = local_e[0], e2 = local_e[1];
  int local_v[2] = {0, 0};
  incr = 0;
  for (int i = 0; i < cnt_vn; ++i) {
    if (vn[i] == v2) continue;
    if (incr < 2) local_v[incr] = vn[i];
    ++incr;
  }
  const int fL = m.FOE(1, e), fR = m.FOE(2, e);
  int f3 = 0;
  for (int i = 0; i < cnt_fn; ++i) {
    if (fn[i] == fL || fn[i] == fR) continue;
    f3 = fn[i];
  }
  int e3 = 0, e4 = 0, e5 = 0;
  for (int i = 1; i <= 3; ++i) {
    const int a = m.EOF_(i, fL), b = m.EOF_(i, fR), c = m.EOF_(i, f3);
    if (a != e && a != e1 && a != e2) e3 = a;
    if (b != e && b != e1 && b != e2) e4 = b;
    if (c != e1 && c != e2) e5 = c;
  }
  for (int i = 1; i <= 2; ++i) {
    if (m.FOE(i, e3) == fR || m.FOE(i, e3) == f3) m.FOE(i, e3) = fL;
    if (m.FOE(i, e4) == fR || m.FOE(i, e4) == f3) m.FOE(i, e4) = fL;
    if (m.FOE(i, e5) == fR || m.FOE(i, e5) == f3) m.FOE(i, e5) = fL;
  }
  incr = 0;
  for (int i = 1; i <= 3; ++i) {
    if (m.VOF(i, fL) == v2) continue;
    if (incr < 2) m.VOF(i, fL) = local_v[incr];
    ++incr;
  }
  incr = 0;
  const int le[2] = {e4, e5};
  for (int i = 1; i <= 3; ++i) {
    if (m.EOF_(i, fL) == e3) continue;
    if (incr < 2) m.EOF_(i, fL) = le[incr];
    ++incr;
  }
  m.gv[v1 - 1] = 1;
  m.ge[e - 1] = 1; m.ge[e1 - 1] = 1; m.ge[e2 - 1] = 1;
  m.gf[fR - 1] = 1; m.gf[f3 - 1] = 1;
  return fL;
}

struct Stats {
  double n_ecol = 0, n_vdel = 0, n_erel = 0, vol_melt = 0, vol_coarse = 0, vol_smooth = 0, drift = 0, refresh = 0;
};

// remesh_coarsen, remesh_coarsen.f90:2-258
int coarsen(Mesh& m, double e_thresh, std::vector<char>& anchor, std::vector<char>& flagged_edge, Stats& st) {
  Walk w;
  bool rm = calculate_elengths(m, e_thresh);
  int flagged_faces[kRing];
  for (int q = 0; q < kRing; ++q) flagged_faces[q] = 0;
  int sweep = 0;
  const int max_sweep = 5;
  while (rm && sweep < max_sweep) {
    for (int e = 1; e <= m.ne; ++e) {
      if (m.GE(e) || !(m.elen[e - 1] <= e_thresh)) continue;
      const int v1 = m.VOE(1, e), v2 = m.VOE(2, e);
      int v1_n[kRing], v2_n[kRing];
      const int v1val = vert_neighbours(m, v1, e, true, v1_n, w);
      if (w.status != kRemeshOk) return w.status;
      const int v2val = vert_neighbours(m, v2, e, false, v2_n, w);
      if (w.status != kRemeshOk) return w.status;
      if (v1val == 3 || v2val == 3) {
        // vertex deletion of the valence-3 end (v1 first)
        const int vd = v1val == 3 ? v1 : v2, vk = v1val == 3 ? v2 : v1;
        const int* vn = v1val == 3 ? v1_n : v2_n;
        const int vval = v1val == 3 ? v1val : v2val;
        int en[kRing], fn[kRing], cnt_en = 0, cnt_f = 0;
        edge_face_1ring(m, vd, e, en, fn, cnt_en, cnt_f, w);
        if (w.status != kRemeshOk) return w.status;
        const int F1 = vert_deletion(m, vd, vk, e, en, fn, vn, cnt_en, cnt_f, vval);
        flagged_faces[0] = F1;
        update_1ring_normals(m, flagged_faces);
        st.n_vdel += 1;
        if (euler_number(m) != 2) return kRemeshTopology;
      } else {
        // edge collapse to the QEM-optimal position
        double Q1[16], Q2[16];
        for (int q = 0; q < 16; ++q) Q1[q] = Q2[q] = 0.0;
        error_quadric(m, Q1, v1, e, w);
        if (w.status != kRemeshOk) return w.status;
        error_quadric(m, Q2, v2, e, w);
        if (w.status != kRemeshOk) return w.status;
        double xnew[3];
        if (!solve_qem(Q1, Q2, xnew)) return kRemeshQem;
        for (int d = 1; d <= 3; ++d) m.X(d, v1) = xnew[d - 1];
        for (int d = 1; d <= 3; ++d) m.VM(d, v1) = 0.5 * (m.VM(d, v1) + m.VM(d, v2));
        const int F1 = m.FOE(1, e), F2 = m.FOE(2, e);
        int e1, re1, e2, re2;
        ghost_and_retained(m, F1, e, e1, re1);
        ghost_and_retained(m, F2, e, e2, re2);
        m.gf[F1 - 1] = 1; m.gf[F2 - 1] = 1;
        m.gv[v2 - 1] = 1;
        m.ge[e - 1] = 1; m.ge[e1 - 1] = 1; m.ge[e2 - 1] = 1;
        update_connectivity_collapse(m, v1, v2, e1, e2, re1, re2, F1, F2);
        flag_neighbours_1ring(m, anchor, flagged_edge, flagged_faces, v1, re1, w);
        if (w.status != kRemeshOk) return w.status;
        rm = calculate_elengths(m, e_thresh);
        update_1ring_normals(m, flagged_faces);
        if (euler_number(m) != 2) return kRemeshTopology;
        if (live_faces(m) <= 4) return kRemeshTetrahedron;
        st.n_ecol += 1;
      }
    }
    ++sweep;
  }
  return kRemeshOk;
}

// One edge relaxation of remesh_smooth.f90:96-205 on edge i; returns false on
// a failed neighbour walk
bool relax_edge(Mesh& m, int i, bool vol_corrected, double target_dv, double& drift, Walk& w) {
  const double omega = 1.0, small = 1.e-15;
  const int v1 = m.VOE(1, i), v2 = m.VOE(2, i);
  double A1[3] = {0, 0, 0}, A2[3] = {0, 0, 0}, vec[3] = {0, 0, 0};
  int v1_n[kRing], v2_n[kRing];
  const int v1val = vert_neighbours(m, v1, i, true, v1_n, w);
  if (w.status != kRemeshOk) return false;
  const int v2val = vert_neighbours(m, v2, i, false, v2_n, w);
  if (w.status != kRemeshOk) return false;
  double ej[3], ejp1[3], buf[3];
  for (int j = 1; j <= v1val; ++j) {
    const int jp1 = 1 + (j % v1val);
    for (int d = 1; d <= 3; ++d) {
      ej[d - 1] = m.X(d, v1_n[j - 1]) - m.X(d, v1);
      ejp1[d - 1] = m.X(d, v1_n[jp1 - 1]) - m.X(d, v1);
    }
    cross(buf, ej, ejp1);
    for (int d = 0; d < 3; ++d) A1[d] = A1[d] + buf[d];
  }
  for (int j = 1; j <= v2val; ++j) {
    const int jp1 = 1 + (j % v2val);
    for (int d = 1; d <= 3; ++d) {
      ej[d - 1] = m.X(d, v2_n[j - 1]) - m.X(d, v2);
      ejp1[d - 1] = m.X(d, v2_n[jp1 - 1]) - m.X(d, v2);
    }
    cross(buf, ej, ejp1);
    for (int d = 0; d < 3; ++d) A2[d] = A2[d] + buf[d];
    if (j == v2val) for (int d = 0; d < 3; ++d) vec[d] = vec[d] + ej[d];
    else if (j == 2) for (int d = 0; d < 3; ++d) vec[d] = vec[d] - ej[d];
  }
  double x1s[3], x2s[3], dx1s[3], dx2s[3];
  for (int d = 1; d <= 3; ++d) {
    double s2 = 0.0, s1 = 0.0;
    for (int q = 2; q <= v2val; ++q) s2 = s2 + m.X(d, v2_n[q - 1]);
    for (int q = 2; q <= v1val; ++q) s1 = s1 + m.X(d, v1_n[q - 1]);
    x1s[d - 1] = (s2 + (double)v2val * s1) / ((double)(v1val * v2val) - 1.0);
    x2s[d - 1] = (x1s[d - 1] + s2) / (double)v2val;
    dx1s[d - 1] = omega * (x1s[d - 1] - m.X(d, v1));
    dx2s[d - 1] = omega * (x2s[d - 1] - m.X(d, v2));
  }
  const double dd[3] = {dx1s[0] - dx2s[0], dx1s[1] - dx2s[1], dx1s[2] - dx2s[2]};
  cross(buf, vec, dd);
  double A[3], nhat[3];
  for (int d = 0; d < 3; ++d) A[d] = A1[d] + A2[d] + buf[d];
  const double nA = norm2_3(A);
  for (int d = 0; d < 3; ++d) nhat[d] = A[d] / (nA + small);
  cross(buf, vec, dx1s);
  double h = -((dx1s[0] * A1[0] + dx1s[1] * A1[1] + dx1s[2] * A1[2]) +
               (dx2s[0] * A2[0] + dx2s[1] * A2[1] + dx2s[2] * A2[2]) +
               (dx2s[0] * buf[0] + dx2s[1] * buf[1] + dx2s[2] * buf[2]));
  if (!vol_corrected) h = h + std::copysign(1.0, h) * target_dv * 6.0;
  h = h / (nA + small);
  double d1[3], d2[3];
  for (int d = 0; d < 3; ++d) { d1[d] = dx1s[d] + h * nhat[d]; d2[d] = dx2s[d] + h * nhat[d]; }
  drift = std::max(drift, std::max(norm2_3(d1), norm2_3(d2)));
  for (int d = 1; d <= 3; ++d) {
    m.X(d, v1) = m.X(d, v1) + dx1s[d - 1] + h * nhat[d - 1];
    m.X(d, v2) = m.X(d, v2) + dx2s[d - 1] + h * nhat[d - 1];
  }
  return true;
}

// remesh_smooth, remesh_smooth.f90:3-347
int smooth(Mesh& m, double vol_old, double target_dv, std::vector<char>& flagged_edge, Stats& st) {
  Walk w;
  bool vol_corrected = false;
  double drift = 1.0e-18;
  const int num_iter = 10;
  for (int cnt = 1; cnt <= num_iter; ++cnt)
    for (int i = 1; i <= m.ne; ++i) {
      if (!flagged_edge[i - 1] || m.GE(i)) continue;
      st.n_erel += 1;
      if (!relax_edge(m, i, vol_corrected, target_dv, drift, w)) return w.status;
      if (!vol_corrected) {
        const double vol_check = calculate_volume(m);
        if (std::fabs(vol_check - vol_old) < 1.e-14) vol_corrected = true;
        else st.refresh += 1;
      }
    }
  if (std::fabs(calculate_volume(m) - vol_old) > 1.e-14) vol_corrected = false;
  if (!vol_corrected)
    for (int i = 1; i <= m.ne; ++i) {
      if (m.GE(i)) continue;
      st.n_erel += 1;
      if (!relax_edge(m, i, vol_corrected, target_dv, drift, w)) return w.status;
      const double vol_check = calculate_volume(m);
      if (std::fabs(vol_check - vol_old) < 1.e-14) vol_corrected = true;
      else st.refresh += 1;
      if (vol_corrected) break;
    }
  for (auto& f : flagged_edge) f = 0;
  st.drift = drift;
  return kRemeshOk;
}

int remesh(Mesh& m, double e_thresh, double* stats) {
  if (!face_of_edge_consistent(m)) build_face_of_edge(m);
  std::vector<char> anchor(m.nv, 1), flagged_edge(m.ne, 0);
  Stats st;
  st.vol_melt = calculate_volume(m);
  int status = coarsen(m, e_thresh, anchor, flagged_edge, st);
  if (status == kRemeshOk) {
    st.vol_coarse = calculate_volume(m);
    const double target_dv = -(st.vol_coarse - st.vol_melt);
    status = smooth(m, st.vol_melt, target_dv, flagged_edge, st);
    st.vol_smooth = calculate_volume(m);
    // particle.f90:205-213: a remeshing residual stops the run
    if (status == kRemeshOk && std::fabs(st.vol_melt - st.vol_smooth) > 1.e-14) status = kRemeshResidual;
  }
  if (stats) {
    const double v[8] = {st.n_ecol, st.n_vdel, st.n_erel, st.vol_melt, st.vol_coarse, st.vol_smooth, st.drift,
                         st.refresh};
    std::memcpy(stats, v, sizeof v);
  }
  return status;
}

// face_of_edge of each context for the callback form (the reference keeps it
// with the mesh, allotri.f90:8; here it lives with the context's remesher)
std::mutex g_foe_mu;
std::map<int, std::vector<int>> g_foe;

}  // namespace

}  // namespace mibm

using namespace mibm;

extern "C" int mibm_remesh_mesh(int nv, int ne, int nf, double* xyzv, double* tri_nor, double* vmelt,
                                double* elengths, int* vert_of_face, int* edge_of_face, int* vert_of_edge,
                                int* face_of_edge, int* ghost_face, int* ghost_edge, int* ghost_vert,
                                double e_thresh, double* stats) {
  if (nv < 4 || ne < 6 || nf < 4 || !xyzv || !tri_nor || !vmelt || !elengths || !vert_of_face || !edge_of_face ||
      !vert_of_edge || !face_of_edge || !ghost_face || !ghost_edge || !ghost_vert)
    return kRemeshArgs;
  Mesh m{nv, ne, nf, xyzv, tri_nor, vmelt, elengths, vert_of_face, edge_of_face, vert_of_edge, face_of_edge,
         ghost_face, ghost_edge, ghost_vert};
  return remesh(m, e_thresh, stats);
}

extern "C" int mibm_remesh_builtin_(void* user) {
  (void)user;
  Ctx* c = current();
  if (!c || !c->inited || c->maxnf == 0) return kRemeshArgs;
  const int ne = c->maxne;
  std::vector<int>* foe = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_foe_mu);
    foe = &g_foe[c->id];                       // map nodes stay put
    if ((int)foe->size() != 2 * ne) foe->assign(2 * (size_t)ne, 0);
  }
  double stats[8];
  int st = mibm_remesh_mesh(c->maxnv, ne, c->maxnf, (double*)c->hm[MIBM_M_XYZV], (double*)c->hm[MIBM_M_TRI_NOR],
                            (double*)c->hm[MIBM_M_VMELT], (double*)c->hm[MIBM_M_ELENGTHS],
                            (int*)c->hm[MIBM_M_VERT_OF_FACE], (int*)c->hm[MIBM_M_EDGE_OF_FACE],
                            (int*)c->hm[MIBM_M_VERT_OF_EDGE], foe->data(), (int*)c->hm[MIBM_M_GHOST_FACE],
                            (int*)c->hm[MIBM_M_GHOST_EDGE], (int*)c->hm[MIBM_M_GHOST_VERT], c->S(MIBM_S_E_THRESH),
                            stats);
  std::memcpy(c->remesh_stats, stats, sizeof stats);
  return st;
}
