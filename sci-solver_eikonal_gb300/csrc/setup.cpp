// setup.cpp — host mesh preparation, partitioning and block layouts.
// See setup.hpp for the map to the reference.  Built with -ffp-contract=off.
#include "setup.hpp"

#include <algorithm>
#include <cmath>
#include <limits>
#include <cstring>
#include <numeric>
#include <set>
#include <thread>

namespace eikgb {

// =============================================================================
// triangle meshes
// =============================================================================
namespace {

inline int index_of(const int* f, int v) { return f[0] == v ? 0 : f[1] == v ? 1 : f[2] == v ? 2 : -1; }

inline float sq(float x) { return x * x; }

// dist() of core2d/include/Vec.h:406-418: sqrt of the squared differences summed
// in component order.
inline float vdist(const float* p, const float* q) {
  float d2 = sq(q[0] - p[0]);
  d2 += sq(q[1] - p[1]);
  d2 += sq(q[2] - p[2]);
  return sqrtf(d2);
}

// edge length as TriMesh::need_faceedges writes it (TriMesh_connectivity.cu:54-75)
inline float edge_len(const float* a, const float* b) {
  const float e0 = b[0] - a[0], e1 = b[1] - a[1], e2 = b[2] - a[2];
  return sqrtf(e0 * e0 + e1 * e1 + e2 * e2);
}

}  // namespace

// The reference tests `acos((b*b + c*c - a*a) / (2*b*c)) < M_PI/2.0f` with a float
// acos and a double comparison (TriMesh.h:191-212).  A correctly rounded float
// acos is below pi/2 exactly when its argument exceeds cos(m), m being the midpoint
// between pi/2's two neighbouring floats; that threshold (1.5893254773528196e-08)
// makes the decision independent of the platform's acosf.  Arguments above 1 give
// a NaN angle in the reference, which fails the test.
bool tri_corner_non_obtuse(const float* xyz, const int* f, int v) {
  const int iv = index_of(f, v);
  const float* A = xyz + 3 * v;
  const float* B = xyz + 3 * f[(iv + 1) % 3];
  const float* C = xyz + 3 * f[(iv + 2) % 3];
  const float a = vdist(B, C), b = vdist(A, C), c = vdist(A, B);
  if (!((a > 0) && (b > 0) && (c > 0))) return true;  // angle left at 0
  const float x = (b * b + c * c - a * a) / (2 * b * c);
  if (!(x <= 1.0f)) return false;
  return (double)x > 1.5893254773528196e-08;
}

namespace {

struct TriTopo {
  int nv, nf;
  const float* xyz;
  std::vector<int>& F;
  std::vector<std::vector<int>> adj;  // faces per vertex, ascending
  std::vector<int> across;            // 3 per face
};

void build_adjacency(TriTopo& T) {
  T.adj.assign(T.nv, {});
  for (int i = 0; i < T.nf; ++i)
    for (int j = 0; j < 3; ++j) T.adj[T.F[3 * i + j]].push_back(i);
}

float max_x(const TriTopo& T, int f) {
  const int* v = &T.F[3 * f];
  return std::max(std::max(T.xyz[3 * v[0]], T.xyz[3 * v[1]]), T.xyz[3 * v[2]]);
}

// Consistent orientation per connected component, then a global flip so the
// outward side faces +x at the component's extreme face (filter.cc:369-452).
void orient(TriTopo& T) {
  const unsigned NONE = ~0u;
  std::vector<unsigned> flag(T.nf, NONE);
  std::vector<int> far;
  unsigned cc = 0;
  std::vector<int> stack;
  for (int i = 0; i < T.nf; ++i) {
    if (flag[i] != NONE) continue;
    flag[i] = cc;
    far.push_back(i);
    float farv = max_x(T, i);
    stack.assign(1, i);
    while (!stack.empty()) {
      const int f = stack.back();
      stack.pop_back();
      for (int j = 0; j < 3; ++j) {
        const int v0 = T.F[3 * f + j], v1 = T.F[3 * f + (j + 1) % 3];
        for (int f1 : T.adj[v0]) {
          if (flag[f1] != NONE) continue;
          int* g = &T.F[3 * f1];
          const int i0 = index_of(g, v0), i1 = index_of(g, v1);
          if (i0 < 0 || i1 < 0) continue;
          if (i1 == (i0 + 1) % 3) std::swap(g[1], g[2]);
          flag[f1] = cc;
          const float mx = max_x(T, f1);
          if (mx > farv) { farv = mx; far[cc] = f1; }
          stack.push_back(f1);
        }
      }
    }
    ++cc;
  }
  std::vector<char> flip(cc, 0);
  for (unsigned c = 0; c < cc; ++c) {
    const int f = far[c];
    const float* p0 = T.xyz + 3 * T.F[3 * f];
    const float* p1 = T.xyz + 3 * T.F[3 * f + 1];
    const float* p2 = T.xyz + 3 * T.F[3 * f + 2];
    int j = 0;
    if (p1[0] > p0[0]) j = (p2[0] > p1[0]) ? 2 : 1;
    else if (p2[0] > p0[0]) j = 2;
    const int v = T.F[3 * f + j];
    float nx = 0.0f;
    for (int f1 : T.adj[v]) {
      const float* a = T.xyz + 3 * T.F[3 * f1];
      const float* b = T.xyz + 3 * T.F[3 * f1 + 1];
      const float* c2 = T.xyz + 3 * T.F[3 * f1 + 2];
      const float e1y = b[1] - a[1], e1z = b[2] - a[2];
      const float e2y = c2[1] - a[1], e2z = c2[2] - a[2];
      nx += 0.5f * (e1y * e2z - e1z * e2y);  // x of trinorm (Vec.h:376-379)
    }
    if (nx < 0.0f) flip[c] = 1;
  }
  for (int i = 0; i < T.nf; ++i)
    if (flip[flag[i]]) std::swap(T.F[3 * i + 1], T.F[3 * i + 2]);
}

// Face across each edge (-1 on the boundary), TriMesh_connectivity.cu:240-278.
void across_edges(TriTopo& T) {
  T.across.assign(3 * T.nf, -1);
  for (int i = 0; i < T.nf; ++i)
    for (int j = 0; j < 3; ++j) {
      if (T.across[3 * i + j] != -1) continue;
      const int v1 = T.F[3 * i + (j + 1) % 3], v2 = T.F[3 * i + (j + 2) % 3];
      const std::vector<int>& a1 = T.adj[v1];
      const std::vector<int>& a2 = T.adj[v2];
      for (int other : a1) {
        if (other == i) continue;
        if (std::find(a2.begin(), a2.end(), other) == a2.end()) continue;
        const int* g = &T.F[3 * other];
        const int ind = (index_of(g, v1) + 1) % 3;
        if (g[(ind + 1) % 3] != v2) continue;
        T.across[3 * i + j] = other;
        T.across[3 * other + ind] = i;
        break;
      }
    }
}

// Unfold the obtuse corner v of `cf` across face `nf_adj` until every new face is
// non-obtuse at v (TriMesh.h:215-313).  Virtual faces carry inverse speed 1, the
// reference's value for its default speed type.
bool split_face(const TriTopo& T, std::vector<int>& out, int v, const int cf[3], int nf_adj,
                int depth) {
  if (depth > kMaxSplitDepth) return false;
  const int iv = index_of(cf, v);
  const int v1 = v, v2 = cf[(iv + 1) % 3], v4 = cf[(iv + 2) % 3];
  const int* g = &T.F[3 * nf_adj];
  const int v3 = g[(index_of(g, v2) + 1) % 3];
  const int f1[3] = {v1, v3, v4};
  const int f2[3] = {v1, v2, v3};
  if (tri_corner_non_obtuse(T.xyz, f1, v)) {
    out.insert(out.end(), f1, f1 + 3);
  } else {
    const int nn = T.across[3 * nf_adj + index_of(g, v2)];
    if (nn > -1 && !split_face(T, out, v, f1, nn, depth + 1)) return false;
  }
  if (tri_corner_non_obtuse(T.xyz, f2, v)) {
    out.insert(out.end(), f2, f2 + 3);
  } else {
    const int nn = T.across[3 * nf_adj + index_of(g, v4)];
    if (nn > -1 && !split_face(T, out, v, f2, nn, depth + 1)) return false;
  }
  return true;
}

}  // namespace

std::string prepare_trimesh(int nv, const float* xyz, int nf, const int* faces, TriPrep& P) {
  P.nv = nv;
  P.nf = nf;
  P.faces.assign(faces, faces + 3 * (size_t)nf);
  for (int i = 0; i < 3 * nf; ++i)
    if (P.faces[i] < 0 || P.faces[i] >= nv) return "face index out of range";
  TriTopo T{nv, nf, xyz, P.faces, {}, {}};
  build_adjacency(T);
  orient(T);
  across_edges(T);
  P.obtuse.assign(nf, 0);
  P.vf_off.assign(nf + 1, 0);
  P.vf_verts.clear();
  for (int i = 0; i < nf; ++i) {
    const int* f = &P.faces[3 * i];
    std::vector<int> vf;
    for (int j = 0; j < 3; ++j) {
      if (tri_corner_non_obtuse(xyz, f, f[j])) continue;
      P.obtuse[i] |= (uint8_t)(1u << j);
      const int nfae = T.across[3 * i + j];
      if (nfae > -1 && !split_face(T, vf, f[j], f, nfae, 0))
        return "obtuse-corner unfolding did not terminate (degenerate mesh)";
    }
    P.vf_verts.insert(P.vf_verts.end(), vf.begin(), vf.end());
    P.vf_off[i + 1] = (int)(P.vf_verts.size() / 3);
  }
  P.edges.resize(3 * (size_t)nf);
  for (int i = 0; i < nf; ++i)
    for (int k = 0; k < 3; ++k)
      P.edges[3 * i + k] = edge_len(xyz + 3 * P.faces[3 * i + k], xyz + 3 * P.faces[3 * i + (k + 1) % 3]);
  const size_t nvf = P.vf_verts.size() / 3;
  P.vf_edges.resize(3 * nvf);
  for (size_t i = 0; i < nvf; ++i)
    for (int k = 0; k < 3; ++k)
      P.vf_edges[3 * i + k] = edge_len(xyz + 3 * P.vf_verts[3 * i + k], xyz + 3 * P.vf_verts[3 * i + (k + 1) % 3]);
  return "";
}

// =============================================================================
// tet meshes
// =============================================================================
void tet_metrics(int nt, const float* vals, size_t nvals, std::vector<float>& M) {
  M.resize(6 * (size_t)nt);
  for (int i = 0; i < nt; ++i) {
    float* m = &M[6 * (size_t)i];
    if (vals && nvals == 6 * (size_t)nt) {
      for (int j = 0; j < 6; ++j) m[j] = vals[6 * (size_t)i + j];
    } else if (vals && nvals == (size_t)nt) {
      m[0] = vals[i]; m[1] = 0.f; m[2] = 0.f; m[3] = vals[i]; m[4] = 0.f; m[5] = vals[i];
    } else {
      m[0] = 1.f; m[1] = 0.f; m[2] = 0.f; m[3] = 1.f; m[4] = 0.f; m[5] = 1.f;
    }
  }
}

void tet_gram(const float* xyz, const int* t, const float* m, float g[6]) {
  float P[4][3];
  for (int k = 0; k < 4; ++k)
    for (int d = 0; d < 3; ++d) P[k][d] = xyz[3 * t[k] + d];
  float AC[3], AD[3], BC[3], CD[3], BD[3];
  for (int d = 0; d < 3; ++d) {
    AC[d] = P[2][d] - P[0][d];
    AD[d] = P[3][d] - P[0][d];
    BC[d] = P[2][d] - P[1][d];
    CD[d] = P[3][d] - P[2][d];
    BD[d] = P[3][d] - P[1][d];
  }
  // u^T M w with M symmetric, association as in core3d/include/Vec.h:479-483
  auto uMw = [m](const float* u, const float* w) -> float {
    return (u[0] * m[0] + u[1] * m[1] + u[2] * m[2]) * w[0] +
           (u[0] * m[1] + u[1] * m[3] + u[2] * m[4]) * w[1] +
           (u[0] * m[2] + u[1] * m[4] + u[2] * m[5]) * w[2];
  };
  g[0] = uMw(AC, BC);
  g[1] = uMw(BC, CD);
  g[2] = uMw(AC, CD);
  g[3] = uMw(AD, BD);
  g[4] = uMw(AC, AD);
  g[5] = uMw(BC, BD);
}

std::string normalize_index_base(std::vector<int>& e, int nv) {
  if (e.empty()) return "no elements";
  const int mn = *std::min_element(e.begin(), e.end());
  if (mn == 1) for (int& x : e) x -= 1;
  else if (mn != 0) return "element indices must start from 0 or 1";
  for (int x : e)
    if (x < 0 || x >= nv) return "element index out of range";
  return "";
}

// =============================================================================
// partitions
// =============================================================================
int metis_rule_blocks(int nv, int k, int dim) {
  if (k <= 0) k = 1;
  long long nb = (dim == 2) ? (long long)nv / k : ((long long)nv + k - 1) / k;
  if (nb < 2) nb = 2;
  if (nb > nv) nb = nv;
  return (int)nb;
}

namespace {
// A point carries its coordinates so the selections below read contiguous memory.
struct RcbPoint {
  float c[3];
  int id;
};

// Recursive coordinate bisection: split the longest bounding-box axis at the
// element that gives the left half its share of parts.  Points are ordered by
// (coordinate, id), a total order, so each half is a fixed set whatever the
// selection algorithm and the threads that run the halves; the labels are a
// function of the coordinates alone.
void rcb(RcbPoint* p, int n, int nparts, int first, int* labels, int depth) {
  if (nparts <= 1 || n <= 1) {
    for (int i = 0; i < n; ++i) labels[p[i].id] = first;
    return;
  }
  float lo[3] = {p[0].c[0], p[0].c[1], p[0].c[2]};
  float hi[3] = {lo[0], lo[1], lo[2]};
  for (int i = 1; i < n; ++i)
    for (int d = 0; d < 3; ++d) {
      lo[d] = std::min(lo[d], p[i].c[d]);
      hi[d] = std::max(hi[d], p[i].c[d]);
    }
  int ax = 0;
  for (int d = 1; d < 3; ++d)
    if (hi[d] - lo[d] > hi[ax] - lo[ax]) ax = d;
  const int pl = nparts / 2;
  // left half gets a share proportional to its part count; sizes stay within one
  const int nl = (int)(((long long)n * pl) / nparts);
  std::nth_element(p, p + nl, p + n, [ax](const RcbPoint& a, const RcbPoint& b) {
    return a.c[ax] < b.c[ax] || (a.c[ax] == b.c[ax] && a.id < b.id);
  });
  // the two halves are independent: the first levels run them on two threads
  if (depth < 4 && n >= 32768) {
    std::thread left([=] { rcb(p, nl, pl, first, labels, depth + 1); });
    rcb(p + nl, n - nl, nparts - pl, first + pl, labels, depth + 1);
    left.join();
  } else {
    rcb(p, nl, pl, first, labels, depth + 1);
    rcb(p + nl, n - nl, nparts - pl, first + pl, labels, depth + 1);
  }
}
}  // namespace

void partition_rcb(int nv, const float* xyz, int nparts, std::vector<int>& labels) {
  labels.assign(nv, 0);
  if (nv <= 0) return;
  std::vector<RcbPoint> pts(nv);
  for (int v = 0; v < nv; ++v) pts[v] = RcbPoint{{xyz[3 * v], xyz[3 * v + 1], xyz[3 * v + 2]}, v};
  rcb(pts.data(), nv, std::max(1, std::min(nparts, nv)), 0, labels.data(), 0);
}

// METIS 5 (libmetis_static.a of the CUDA toolkit, linked when the build finds it):
// its two entry points, declared here because the toolkit ships no metis.h.  The
// library's integer type is 64-bit; the real-valued arguments are passed as null.
#ifdef EIK_HAVE_METIS
extern "C" {
int METIS_PartGraphKway(int64_t* nvtxs, int64_t* ncon, int64_t* xadj, int64_t* adjncy, int64_t* vwgt,
                        int64_t* vsize, int64_t* adjwgt, int64_t* nparts, void* tpwgts, void* ubvec,
                        int64_t* options, int64_t* edgecut, int64_t* part);
}
bool metis_available() { return true; }
#else
bool metis_available() { return false; }
#endif

std::string partition_metis(int nv, int ne, int nodes_per_elem, const int* elems, int nparts,
                            std::vector<int>& labels, int& nb) {
#ifndef EIK_HAVE_METIS
  (void)nv; (void)ne; (void)nodes_per_elem; (void)elems; (void)nparts; (void)labels; (void)nb;
  return "this build has no METIS (libmetis_static.a was not found at build time)";
#else
  labels.assign(nv, 0);
  nb = 1;
  if (nv <= 0) return "";
  if (nparts <= 1 || nv < 2) return "";
  // vertex graph: vertices sharing an element are adjacent (CSR, sorted, unique)
  std::vector<int64_t> deg(nv + 1, 0);
  for (int e = 0; e < ne; ++e)
    for (int i = 0; i < nodes_per_elem; ++i) deg[elems[(size_t)e * nodes_per_elem + i] + 1] += nodes_per_elem - 1;
  for (int v = 0; v < nv; ++v) deg[v + 1] += deg[v];
  std::vector<int64_t> nbr((size_t)deg[nv]);
  std::vector<int64_t> fill(deg.begin(), deg.end() - 1);
  for (int e = 0; e < ne; ++e) {
    const int* t = elems + (size_t)e * nodes_per_elem;
    for (int i = 0; i < nodes_per_elem; ++i)
      for (int j = 0; j < nodes_per_elem; ++j)
        if (i != j) nbr[(size_t)fill[t[i]]++] = t[j];
  }
  std::vector<int64_t> xadj(nv + 1, 0), adj;
  adj.reserve(nbr.size() / 2);
  for (int v = 0; v < nv; ++v) {
    auto b0 = nbr.begin() + deg[v], b1 = nbr.begin() + deg[v + 1];
    std::sort(b0, b1);
    b1 = std::unique(b0, b1);
    for (auto it = b0; it != b1; ++it)
      if (*it != v) adj.push_back(*it);
    xadj[v + 1] = (int64_t)adj.size();
  }
  int64_t n = nv, ncon = 1, np = std::min(nparts, nv), cut = 0;
  std::vector<int64_t> part(nv, 0);
  const int rc = METIS_PartGraphKway(&n, &ncon, xadj.data(), adj.data(), nullptr, nullptr, nullptr, &np, nullptr,
                                     nullptr, nullptr, &cut, part.data());
  if (rc != 1) return "METIS_PartGraphKway failed (status " + std::to_string(rc) + ")";
  // number the non-empty parts 0..nb-1 in order
  std::vector<int> id((size_t)np, -1);
  nb = 0;
  for (int v = 0; v < nv; ++v) {
    const int64_t q = part[v];
    if (q < 0 || q >= np) return "METIS returned a part out of range";
    if (id[(size_t)q] < 0) id[(size_t)q] = 0;
  }
  for (int64_t q = 0; q < np; ++q)
    if (id[(size_t)q] >= 0) id[(size_t)q] = nb++;
  for (int v = 0; v < nv; ++v) labels[v] = id[(size_t)part[v]];
  return "";
#endif
}

std::string partition_square(int nv, int dim, int L, int W, int D, int bl, int bw, int bd,
                             std::vector<int>& labels, int& nb) {
  if (bl <= 0 || bw <= 0 || (dim == 3 && bd <= 0)) return "block dimensions must be positive";
  const long long need = (long long)L * W * (dim == 3 ? D : 1);
  if (need != nv) return "structured grid dimensions do not match the vertex count";
  const int nbl = L / bl, nbw = W / bw, nbd = (dim == 3) ? D / bd : 1;
  if (nbl <= 0 || nbw <= 0 || nbd <= 0) return "block larger than the grid";
  nb = nbl * nbw * nbd;
  labels.assign(nv, 0);
  if (dim == 2) {
    for (int i = 0; i < W; ++i)
      for (int j = 0; j < L; ++j) labels[i * L + j] = std::min(i / bw, nbw - 1) * nbl + std::min(j / bl, nbl - 1);
  } else {
    for (int k = 0; k < D; ++k)
      for (int i = 0; i < W; ++i)
        for (int j = 0; j < L; ++j)
          labels[(size_t)k * L * W + (size_t)i * L + j] =
              std::min(k / bd, nbd - 1) * nbl * nbw + std::min(i / bw, nbw - 1) * nbl + std::min(j / bl, nbl - 1);
  }
  return "";
}

// =============================================================================
// layouts
// =============================================================================
namespace {

// owned-vertex renumbering: block b owns [vbase_b, vbase_b + n_b), in ascending
// original id (the reference's m_PartitionInVerts order)
void renumber(int nv, const int* labels, int nb, Layout& L, std::vector<int>& vbase) {
  vbase.assign(nb + 1, 0);
  for (int v = 0; v < nv; ++v) vbase[labels[v] + 1]++;
  for (int b = 0; b < nb; ++b) vbase[b + 1] += vbase[b];
  std::vector<int> cur(vbase.begin(), vbase.end() - 1);
  L.perm.assign(nv, 0);
  L.iperm.assign(nv, 0);
  for (int v = 0; v < nv; ++v) {
    const int n = cur[labels[v]]++;
    L.perm[v] = n;
    L.iperm[n] = v;
  }
}

void single_instance(Layout& L) {
  L.ninst = 1;
  L.blk_inst.assign(L.nb, 0);
  L.inst_bbeg = {0, L.nb};
  L.inst_vbeg = {0, L.nv};
}

void finish_stats(Layout& L) {
  L.max_slots = L.max_local = L.max_owned = L.max_halo = 0;
  double s = 0, h = 0;
  for (const BlockDesc& d : L.blocks) {
    L.max_slots = std::max(L.max_slots, d.nslots);
    L.max_owned = std::max(L.max_owned, d.nowned);
    L.max_halo = std::max(L.max_halo, d.nhalo);
    L.max_local = std::max(L.max_local, d.nowned + d.nhalo);
    s += d.nslots;
    h += d.nhalo;
  }
  L.mean_slots_per_block = L.nb ? s / L.nb : 0;
  L.mean_halo_per_block = L.nb ? h / L.nb : 0;
}

// Element lists per block: elements whose vertices all lie in the block first
// (ascending id), then elements shared with other blocks (ascending id) —
// the order of m_PartitionTets / m_PartitionNbTets.
void element_lists(int ne, int nper, const int* elems, const int* labels, int nb,
                   std::vector<std::vector<int>>& inside, std::vector<std::vector<int>>& shared,
                   std::vector<std::set<int>>& nbrs) {
  inside.assign(nb, {});
  shared.assign(nb, {});
  nbrs.assign(nb, {});
  int ls[4];
  for (int i = 0; i < ne; ++i) {
    int n = 0;
    for (int k = 0; k < nper; ++k) {
      const int l = labels[elems[nper * i + k]];
      bool seen = false;
      for (int j = 0; j < n; ++j) seen |= (ls[j] == l);
      if (!seen) ls[n++] = l;
    }
    for (int x = 1; x < n; ++x)  // sort the (at most 4) labels
      for (int y = x; y > 0 && ls[y - 1] > ls[y]; --y) std::swap(ls[y - 1], ls[y]);
    if (n == 1) {
      inside[ls[0]].push_back(i);
    } else {
      for (int j = 0; j < n; ++j) {
        shared[ls[j]].push_back(i);
        for (int k = 0; k < n; ++k)
          if (k != j) nbrs[ls[j]].insert(ls[k]);
      }
    }
  }
}

void store_nbrs(const std::vector<std::set<int>>& nbrs, Layout& L) {
  L.nbr_off.assign(L.nb + 1, 0);
  L.nbr.clear();
  for (int b = 0; b < L.nb; ++b) {
    L.nbr.insert(L.nbr.end(), nbrs[b].begin(), nbrs[b].end());
    L.nbr_off[b + 1] = (int)L.nbr.size();
  }
}

}  // namespace

std::string build_layout3d(int nv, const float* xyz, int nt, const int* tets, const float* M,
                           const int* labels, int nb, Layout& L) {
  L = Layout();
  L.dim = 3;
  L.nv = nv;
  L.ne = nt;
  L.nb = nb;
  for (int v = 0; v < nv; ++v)
    if (labels[v] < 0 || labels[v] >= nb) return "partition label out of range";
  std::vector<int> vbase;
  renumber(nv, labels, nb, L, vbase);
  std::vector<std::vector<int>> inside, shared;
  std::vector<std::set<int>> nbrs;
  element_lists(nt, 4, tets, labels, nb, inside, shared, nbrs);
  store_nbrs(nbrs, L);

  L.blocks.resize(nb);
  int slot = 0;
  for (int b = 0; b < nb; ++b) {
    BlockDesc& d = L.blocks[b];
    d.slot_begin = slot;
    d.ninside = (int)inside[b].size();
    d.nslots = d.ninside + (int)shared[b].size();
    d.nslots_pad = (d.nslots + 3) & ~3;
    d.vbase = vbase[b];
    d.nowned = vbase[b + 1] - vbase[b];
    slot += d.nslots_pad;
  }
  L.total_slots = slot;
  L.coef.assign(6 * (size_t)slot, 0.0f);
  L.lv.assign(4 * (size_t)slot, 0);
  L.slot_elem.assign(slot, -1);
  L.halo_ids.clear();
  std::vector<int> local(nv, -1);
  for (int b = 0; b < nb; ++b) {
    BlockDesc& d = L.blocks[b];
    d.halo_begin = (int)L.halo_ids.size();
    std::vector<int> halo;
    for (int pass = 0; pass < 2; ++pass)
      for (int t : (pass == 0 ? inside[b] : shared[b]))
        for (int k = 0; k < 4; ++k) {
          const int v = tets[4 * (size_t)t + k];
          if (labels[v] != b) halo.push_back(L.perm[v]);
        }
    std::sort(halo.begin(), halo.end());
    halo.erase(std::unique(halo.begin(), halo.end()), halo.end());
    d.nhalo = (int)halo.size();
    if (d.nowned + d.nhalo > 32767) return "block has too many local vertices (limit 32767)";
    for (int i = 0; i < d.nhalo; ++i) local[halo[i]] = d.nowned + i;  // keyed by renumbered id
    L.halo_ids.insert(L.halo_ids.end(), halo.begin(), halo.end());
    int j = 0;
    for (int pass = 0; pass < 2; ++pass)
      for (int t : (pass == 0 ? inside[b] : shared[b])) {
        const size_t s = (size_t)d.slot_begin + j;
        L.slot_elem[s] = t;
        for (int k = 0; k < 4; ++k) {
          const int v = tets[4 * (size_t)t + k];
          const int nvid = L.perm[v];
          const int lid = (labels[v] == b) ? nvid - d.vbase : local[nvid];
          L.lv[4 * s + k] = (uint16_t)lid;
        }
        ++j;
      }
    for (int i = 0; i < d.nhalo; ++i) local[halo[i]] = -1;
  }
  refresh_gram3d(xyz, tets, M, L);
  finish_stats(L);
  single_instance(L);
  return "";
}

void refresh_gram3d(const float* xyz, const int* tets, const float* M, Layout& L) {
  for (const BlockDesc& d : L.blocks) {
    float* base = &L.coef[6 * (size_t)d.slot_begin];
    for (int j = 0; j < d.nslots; ++j) {
      const int t = L.slot_elem[(size_t)d.slot_begin + j];
      float g[6];
      tet_gram(xyz, tets + 4 * (size_t)t, M + 6 * (size_t)t, g);
      for (int k = 0; k < 6; ++k) base[(size_t)k * d.nslots_pad + j] = g[k];
    }
  }
}

// 2D layout.  The reference keeps at most 6 slot addresses per vertex inside its
// own block and 6 in other blocks, in the order of its blockVertMapping list
// (meshFIM2d_eikonal.cu:404-614); slot copies beyond those are never refreshed
// and keep their initial value.  Such corners get bit 15 in `lv`.
std::string build_layout2d(int nv, const float* xyz, const TriPrep& P, const float* speed_inv,
                           const int* labels, int nb, Layout& L) {
  (void)xyz;
  L = Layout();
  L.dim = 2;
  L.nv = nv;
  L.ne = P.nf;
  L.nb = nb;
  for (int v = 0; v < nv; ++v)
    if (labels[v] < 0 || labels[v] >= nb) return "partition label out of range";
  std::vector<int> vbase;
  renumber(nv, labels, nb, L, vbase);
  std::vector<std::vector<int>> inside, shared;
  std::vector<std::set<int>> nbrs;
  element_lists(P.nf, 3, P.faces.data(), labels, nb, inside, shared, nbrs);
  store_nbrs(nbrs, L);
  // virtual faces attach to the block of each obtuse corner (PartitionFaces :281-287)
  std::vector<std::vector<int>> virt(nb);
  for (int i = 0; i < P.nf; ++i)
    for (int k = 0; k < 3; ++k)
      if (P.obtuse[i] & (1u << k))
        for (int j = P.vf_off[i]; j < P.vf_off[i + 1]; ++j) virt[labels[P.faces[3 * i + k]]].push_back(j);

  L.blocks.resize(nb);
  int slot = 0;
  for (int b = 0; b < nb; ++b) {
    BlockDesc& d = L.blocks[b];
    d.slot_begin = slot;
    d.ninside = (int)inside[b].size();
    d.nslots = d.ninside + (int)shared[b].size() + (int)virt[b].size();
    d.nslots_pad = (d.nslots + 3) & ~3;
    d.vbase = vbase[b];
    d.nowned = vbase[b + 1] - vbase[b];
    slot += d.nslots_pad;
  }
  L.total_slots = slot;
  L.coef.assign(4 * (size_t)slot, 0.0f);
  L.lv.assign(4 * (size_t)slot, 0);
  L.slot_elem.assign(slot, -1);

  // slot vertex lists in the reference's per-block order
  auto slot_verts = [&](int b, int j) -> const int* {
    const int ni = (int)inside[b].size(), ns = (int)shared[b].size();
    if (j < ni) return &P.faces[3 * (size_t)inside[b][j]];
    if (j < ni + ns) return &P.faces[3 * (size_t)shared[b][j - ni]];
    return &P.vf_verts[3 * (size_t)virt[b][j - ni - ns]];
  };
  // blockVertMapping: pass 1 = inside slots of every block, pass 2 = the rest
  std::vector<std::vector<long long>> vmap(nv);  // (block << 32) | (slot*4 + corner)
  auto enc = [](int b, int j, int k) { return ((long long)b << 32) | (long long)(j * 4 + k); };
  for (int b = 0; b < nb; ++b)
    for (int j = 0; j < (int)inside[b].size(); ++j)
      for (int k = 0; k < 3; ++k) vmap[slot_verts(b, j)[k]].push_back(enc(b, j, k));
  for (int b = 0; b < nb; ++b)
    for (int j = (int)inside[b].size(); j < L.blocks[b].nslots; ++j)
      for (int k = 0; k < 3; ++k) vmap[slot_verts(b, j)[k]].push_back(enc(b, j, k));
  // live copies: first own-block entry swapped to the front, then the first 6
  // own-block and the first 6 other-block entries
  std::vector<std::vector<char>> live(nb);
  for (int b = 0; b < nb; ++b) live[b].assign(4 * (size_t)L.blocks[b].nslots, 0);
  for (int v = 0; v < nv; ++v) {
    std::vector<long long>& m = vmap[v];
    if (m.empty()) continue;
    const int own = labels[v];
    if ((int)(m[0] >> 32) != own)
      for (size_t j = 1; j < m.size(); ++j)
        if ((int)(m[j] >> 32) == own) { std::swap(m[0], m[j]); break; }
    int ni = 0, no = 0;
    for (long long e : m) {
      const int b = (int)(e >> 32), sc = (int)(e & 0xffffffff);
      if (b == own) { if (ni++ < kSlotCap2D) live[b][sc] = 1; }
      else { if (no++ < kSlotCap2D) live[b][sc] = 1; }
    }
  }
  L.halo_ids.clear();
  std::vector<int> local(nv, -1);
  for (int b = 0; b < nb; ++b) {
    BlockDesc& d = L.blocks[b];
    d.halo_begin = (int)L.halo_ids.size();
    std::vector<int> halo;
    for (int j = 0; j < d.nslots; ++j)
      for (int k = 0; k < 3; ++k) {
        const int v = slot_verts(b, j)[k];
        if (labels[v] != b) halo.push_back(L.perm[v]);
      }
    std::sort(halo.begin(), halo.end());
    halo.erase(std::unique(halo.begin(), halo.end()), halo.end());
    d.nhalo = (int)halo.size();
    if (d.nowned + d.nhalo > 32767) return "block has too many local vertices (limit 32767)";
    for (int i = 0; i < d.nhalo; ++i) local[halo[i]] = d.nowned + i;
    L.halo_ids.insert(L.halo_ids.end(), halo.begin(), halo.end());
    const int ni = (int)inside[b].size(), ns = (int)shared[b].size();
    for (int j = 0; j < d.nslots; ++j) {
      const size_t s = (size_t)d.slot_begin + j;
      L.slot_elem[s] = (j < ni) ? inside[b][j] : (j < ni + ns) ? shared[b][j - ni] : -1;
      const int* fv = slot_verts(b, j);
      for (int k = 0; k < 3; ++k) {
        const int nvid = L.perm[fv[k]];
        const int lid = (labels[fv[k]] == b) ? nvid - d.vbase : local[nvid];
        L.lv[4 * s + k] = (uint16_t)(lid | (live[b][4 * j + k] ? 0 : 0x8000));
      }
      L.lv[4 * s + 3] = 0;
    }
    for (int i = 0; i < d.nhalo; ++i) local[halo[i]] = -1;
  }
  // store which virtual face each virtual slot holds (negative, -2 - index)
  for (int b = 0; b < nb; ++b) {
    const BlockDesc& d = L.blocks[b];
    const int ni = (int)inside[b].size(), ns = (int)shared[b].size();
    for (int j = ni + ns; j < d.nslots; ++j) L.slot_elem[(size_t)d.slot_begin + j] = -2 - virt[b][j - ni - ns];
  }
  refresh_speed2d(P, speed_inv, L);
  finish_stats(L);
  single_instance(L);
  return "";
}

void refresh_speed2d(const TriPrep& P, const float* speed_inv, Layout& L) {
  for (const BlockDesc& d : L.blocks) {
    float* base = &L.coef[4 * (size_t)d.slot_begin];
    const size_t np = d.nslots_pad;
    for (int j = 0; j < d.nslots; ++j) {
      const int e = L.slot_elem[(size_t)d.slot_begin + j];
      const float* ed;
      float F;
      if (e >= 0) { ed = &P.edges[3 * (size_t)e]; F = speed_inv ? speed_inv[e] : 1.0f; }
      else { ed = &P.vf_edges[3 * (size_t)(-2 - e)]; F = 1.0f; }
      base[0 * np + j] = ed[0];
      base[1 * np + j] = ed[1];
      base[2 * np + j] = ed[2];
      base[3 * np + j] = F;
    }
  }
}

double tet_condition(const float* xyz, const int* t, const float* m6) {
  double P[4][3];
  for (int k = 0; k < 4; ++k)
    for (int d = 0; d < 3; ++d) P[k][d] = (double)xyz[3 * (size_t)t[k] + d];
  double E[3][3];  // columns: B-A, C-A, D-A
  for (int c = 0; c < 3; ++c)
    for (int d = 0; d < 3; ++d) E[d][c] = P[c + 1][d] - P[0][d];
  const double M[3][3] = {{m6[0], m6[1], m6[2]}, {m6[1], m6[3], m6[4]}, {m6[2], m6[4], m6[5]}};
  double ME[3][3], G[3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      ME[i][j] = 0;
      for (int k = 0; k < 3; ++k) ME[i][j] += M[i][k] * E[k][j];
    }
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      G[i][j] = 0;
      for (int k = 0; k < 3; ++k) G[i][j] += E[k][i] * ME[k][j];
    }
  // adjugate and determinant
  const double c00 = G[1][1] * G[2][2] - G[1][2] * G[2][1], c01 = G[1][2] * G[2][0] - G[1][0] * G[2][2],
               c02 = G[1][0] * G[2][1] - G[1][1] * G[2][0];
  const double det = G[0][0] * c00 + G[0][1] * c01 + G[0][2] * c02;
  double fro = 0;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) fro += G[i][j] * G[i][j];
  if (!(det > 0.0)) return std::numeric_limits<double>::infinity();
  const double adj[9] = {c00, G[0][2] * G[2][1] - G[0][1] * G[2][2], G[0][1] * G[1][2] - G[0][2] * G[1][1],
                         c01, G[0][0] * G[2][2] - G[0][2] * G[2][0], G[0][2] * G[1][0] - G[0][0] * G[1][2],
                         c02, G[0][1] * G[2][0] - G[0][0] * G[2][1], G[0][0] * G[1][1] - G[0][1] * G[1][0]};
  double ifro = 0;
  for (double a : adj) ifro += a * a;
  return std::sqrt(fro) * std::sqrt(ifro) / det;
}

void build_precision3d(const float* xyz, const int* tets, const float* M, double kappa, Layout& L) {
  L.slot_f64.clear();
  L.coef64.clear();
  L.flagged_tets = 0;
  if (!(kappa > 0) || L.dim != 3) return;
  std::vector<int> idx(L.ne, -1);
  for (int t = 0; t < L.ne; ++t) {
    if (!(tet_condition(xyz, tets + 4 * (size_t)t, M + 6 * (size_t)t) > kappa)) continue;
    idx[t] = (int)L.flagged_tets++;
    // the six products of tet_gram, in FP64 from the FP32 inputs
    const int* v = tets + 4 * (size_t)t;
    const float* m = M + 6 * (size_t)t;
    double P[4][3];
    for (int k = 0; k < 4; ++k)
      for (int d = 0; d < 3; ++d) P[k][d] = (double)xyz[3 * (size_t)v[k] + d];
    double AC[3], AD[3], BC[3], CD[3], BD[3];
    for (int d = 0; d < 3; ++d) {
      AC[d] = P[2][d] - P[0][d];
      AD[d] = P[3][d] - P[0][d];
      BC[d] = P[2][d] - P[1][d];
      CD[d] = P[3][d] - P[2][d];
      BD[d] = P[3][d] - P[1][d];
    }
    const double md[6] = {m[0], m[1], m[2], m[3], m[4], m[5]};
    auto uMw = [&md](const double* u, const double* w) {
      return (u[0] * md[0] + u[1] * md[1] + u[2] * md[2]) * w[0] + (u[0] * md[1] + u[1] * md[3] + u[2] * md[4]) * w[1] +
             (u[0] * md[2] + u[1] * md[4] + u[2] * md[5]) * w[2];
    };
    L.coef64.push_back(uMw(AC, BC));
    L.coef64.push_back(uMw(BC, CD));
    L.coef64.push_back(uMw(AC, CD));
    L.coef64.push_back(uMw(AD, BD));
    L.coef64.push_back(uMw(AC, AD));
    L.coef64.push_back(uMw(BC, BD));
  }
  // Flagged slots move behind the unflagged ones inside each block's two slot
  // groups (all corners owned / some corners foreign), so the FP64 updates run in
  // few warps instead of diverging in most of them.  Slot order inside a block
  // does not change results: every vertex takes the minimum over its slots.
  std::vector<int> order;
  std::vector<float> c6;
  std::vector<uint16_t> lv4;
  std::vector<int> el;
  for (const BlockDesc& d : L.blocks) {
    order.clear();
    for (int part = 0; part < 2; ++part) {
      const int j0 = part ? d.ninside : 0, j1 = part ? d.nslots : d.ninside;
      for (int pass = 0; pass < 2; ++pass)
        for (int j = j0; j < j1; ++j) {
          const int t = L.slot_elem[(size_t)d.slot_begin + j];
          const bool f = t >= 0 && idx[t] >= 0;
          if (f == (pass == 1)) order.push_back(j);
        }
    }
    const size_t np = (size_t)d.nslots_pad, sb = (size_t)d.slot_begin;
    c6.assign(&L.coef[6 * sb], &L.coef[6 * sb] + 6 * np);
    lv4.assign(&L.lv[4 * sb], &L.lv[4 * sb] + 4 * np);
    el.assign(&L.slot_elem[sb], &L.slot_elem[sb] + np);
    for (int j = 0; j < d.nslots; ++j) {
      const int o = order[j];
      for (int k = 0; k < 6; ++k) L.coef[6 * sb + k * np + j] = c6[k * np + o];
      for (int k = 0; k < 4; ++k) L.lv[4 * (sb + j) + k] = lv4[4 * (size_t)o + k];
      L.slot_elem[sb + j] = el[o];
    }
  }
  L.slot_f64.assign(L.slot_elem.size(), -1);
  for (size_t s = 0; s < L.slot_elem.size(); ++s)
    if (L.slot_elem[s] >= 0) L.slot_f64[s] = idx[L.slot_elem[s]];
}

std::string concat_layouts(const std::vector<const Layout*>& parts, Layout& out) {
  out = Layout();
  if (parts.empty()) return "no instances";
  const int dim = parts[0]->dim;
  out.dim = dim;
  out.inst_bbeg.push_back(0);
  out.inst_vbeg.push_back(0);
  for (const Layout* p : parts) {
    if (p->dim != dim) return "instances of different dimension";
    const int boff = out.nb, voff = out.nv, soff = out.total_slots, hoff = (int)out.halo_ids.size();
    const int noff = (int)out.nbr.size();
    for (int v : p->perm) out.perm.push_back(v + voff);
    for (int v : p->iperm) out.iperm.push_back(v + voff);
    for (BlockDesc d : p->blocks) {
      d.slot_begin += soff;
      d.vbase += voff;
      d.halo_begin += hoff;
      out.blocks.push_back(d);
    }
    out.coef.insert(out.coef.end(), p->coef.begin(), p->coef.end());
    if (!p->slot_f64.empty() || !out.slot_f64.empty()) {
      // precision data: pad earlier parts with -1, offset this part's indices
      out.slot_f64.resize((size_t)soff, -1);
      const int f0 = (int)(out.coef64.size() / 6);
      if (p->slot_f64.empty()) out.slot_f64.resize((size_t)soff + p->slot_elem.size(), -1);
      for (int f : p->slot_f64) out.slot_f64.push_back(f >= 0 ? f + f0 : -1);
      out.coef64.insert(out.coef64.end(), p->coef64.begin(), p->coef64.end());
      out.flagged_tets += p->flagged_tets;
    }
    out.lv.insert(out.lv.end(), p->lv.begin(), p->lv.end());
    for (int e : p->slot_elem) out.slot_elem.push_back(e);
    for (int h : p->halo_ids) out.halo_ids.push_back(h + voff);
    if (out.nbr_off.empty()) out.nbr_off.push_back(0);
    for (int b = 0; b < p->nb; ++b) out.nbr_off.push_back(p->nbr_off[b + 1] + noff);
    for (int n : p->nbr) out.nbr.push_back(n + boff);
    out.nb += p->nb;
    out.nv += p->nv;
    out.ne += p->ne;
    out.total_slots += p->total_slots;
    out.inst_bbeg.push_back(out.nb);
    out.inst_vbeg.push_back(out.nv);
  }
  out.ninst = (int)parts.size();
  // instance of every block from the block ranges
  out.blk_inst.assign(out.nb, 0);
  for (int i = 0; i < out.ninst; ++i)
    for (int b = out.inst_bbeg[i]; b < out.inst_bbeg[i + 1]; ++b) out.blk_inst[b] = i;
  finish_stats(out);
  return "";
}

std::string concat_layout_headers(const std::vector<const Layout*>& parts, const std::vector<int>& nhalo,
                                  Layout& out) {
  out = Layout();
  if (parts.empty()) return "no instances";
  if (nhalo.size() != parts.size()) return "one halo length per instance expected";
  const int dim = parts[0]->dim;
  out.dim = dim;
  out.inst_bbeg.push_back(0);
  out.inst_vbeg.push_back(0);
  long long hoff = 0;
  for (size_t i = 0; i < parts.size(); ++i) {
    const Layout* p = parts[i];
    if (p->dim != dim) return "instances of different dimension";
    const int voff = out.nv, soff = out.total_slots;
    for (int v : p->perm) out.perm.push_back(v + voff);
    for (BlockDesc d : p->blocks) {
      d.slot_begin += soff;
      d.vbase += voff;
      d.halo_begin += (int)hoff;
      out.blocks.push_back(d);
    }
    hoff += nhalo[i];
    if (hoff > 0x7fffffffll) return "halo lists too long";
    out.nb += p->nb;
    out.nv += p->nv;
    out.ne += p->ne;
    out.total_slots += p->total_slots;
    out.inst_bbeg.push_back(out.nb);
    out.inst_vbeg.push_back(out.nv);
  }
  out.ninst = (int)parts.size();
  out.blk_inst.assign(out.nb, 0);
  for (int i = 0; i < out.ninst; ++i)
    for (int b = out.inst_bbeg[i]; b < out.inst_bbeg[i + 1]; ++b) out.blk_inst[b] = i;
  finish_stats(out);
  return "";
}

}  // namespace eikgb
