// Host-side mesh preprocessing for the edge-based median-dual finite-volume path.
//
// This file builds, on the host and in FP64, the integer maps and dual metrics
// that the reference computes before its first Newton step, following the
// reference's algorithms and traversal orders so that the resulting arrays are
// the ones the reference's kernels would see for the same element list:
//
//   element-surrounding-point map ......... ucs/mesh.tcc:397   (Mesh::BuildElsp)
//   point-surrounding-point map + dedup ... ucs/mesh.tcc:517   (Mesh::BuildPsp, cl table :541-548)
//                                            ucs/mesh.tcc:1341  (Mesh::EliminateRepeats)
//   interior edges and boundary half-edges  ucs/mesh.tcc:1056  (Mesh::BuildEdges)
//   median-dual areas and volumes .......... ucs/mesh.tcc:1653  (Mesh::CalcAreasVolumes)
//   closure check + normalisation .......... ucs/mesh.tcc:2274  (Mesh::CheckForClosure)
//   boundary winding check ................. ucs/mesh.tcc:2336  (Mesh::FixBoundaryWindings)
//   weighted LSQ normal matrices ........... ucs/gradient.tcc:115,461 (ComputeNodeLSQCoefficients)
//   reverse Cuthill-McKee renumbering ...... ucs/mesh.tcc:2412  (Mesh::ReorderMeshCuthillMcKee)
//   ... applied to the elements ............ ucs/mesh.tcc:224   (Mesh::ReorderC2nMap)
//
// It also holds the synthetic workload generator: an Nx x Ny x Nz node box
// split into 6 Kuhn tetrahedra per hex (all sharing the hex's (0,0,0)-(1,1,1)
// diagonal), with seeded jitter of interior nodes, an optional sheared ramp
// and optional geometric wall clustering.  Only tetrahedra and boundary
// triangles occur, so only the TET/TRI rows of the reference's element tables
// are used.
//
// Everything here is plain C++ with a C ABI (declared in include/pcfd.h);
// nothing depends on CUDA.

#include "../../include/pcfd.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <deque>
#include <exception>
#include <new>
#include <string>
#include <thread>
#include <vector>

namespace {

enum { ETRI = 0, ETET = 2 };

struct HostMesh {
  // geometry
  int nnode = 0;
  std::vector<double> xyz;          // [nnode][3]
  // element list in reference order (boundary triangles first, then tets)
  std::vector<int> etype;           // ETRI / ETET
  std::vector<int> enodes;          // [nelem][4] (triangles use 3)
  std::vector<int> efactag;         // triangles: boundary tag; tets: 0
  // maps
  std::vector<int> ielsp, elsp;
  std::vector<int> ipsp, psp;
  std::vector<int> edges;           // [nedge][2]
  std::vector<double> ea;           // [nedge][4]
  std::vector<int> bedges;          // [nbedge][2]  (node, phantom id)
  std::vector<int> belem;           // [nbedge] owning boundary element
  std::vector<int> bfactag;         // [nbedge]
  std::vector<double> ba;           // [nbedge][4]
  std::vector<double> vol;          // [nnode]
  std::vector<double> sw;           // [nnode][6]
  int nedge = 0, nbedge = 0;
  int maps_built = 0, metrics_built = 0;
  int rewound = 0;
  int unclosed = 0;
  int inverted = 0;
  double max_open = 0.0;
  std::string err;
};

// ---- small geometry helpers with the reference's operation order ----------
// (ucs/geometry.h: Subtract :12, Magnitude :41, Normalize :51, CrossProduct
//  :68, Centroid :133-215, CalcTriArea, CalcTetVol)
inline void sub3(const double* a, const double* b, double* r) {
  r[0] = a[0] - b[0]; r[1] = a[1] - b[1]; r[2] = a[2] - b[2];
}
inline void cross3(const double* v1, const double* v2, double* rv) {
  rv[0] = v1[1] * v2[2] - v2[1] * v1[2];
  rv[1] = v1[2] * v2[0] - v2[2] * v1[0];
  rv[2] = v1[0] * v2[1] - v2[0] * v1[1];
}
inline double mag3(const double* v) { return std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]); }
inline double normalize3(const double* v, double* rv) {
  double m = mag3(v);
  rv[0] = v[0] / m; rv[1] = v[1] / m; rv[2] = v[2] / m;
  return m;
}
inline void mid2(const double* p1, const double* p2, double* r) {
  r[0] = (p1[0] + p2[0]); r[1] = (p1[1] + p2[1]); r[2] = (p1[2] + p2[2]);
  r[0] *= 0.5; r[1] *= 0.5; r[2] *= 0.5;
}
inline void cen3(const double* p1, const double* p2, const double* p3, double* r) {
  double frac = 1.0 / 3.0;
  r[0] = (p1[0] + p2[0] + p3[0]); r[1] = (p1[1] + p2[1] + p3[1]); r[2] = (p1[2] + p2[2] + p3[2]);
  r[0] *= frac; r[1] *= frac; r[2] *= frac;
}
inline void cen4(const double* p1, const double* p2, const double* p3, const double* p4, double* r) {
  r[0] = (p1[0] + p2[0] + p3[0] + p4[0]);
  r[1] = (p1[1] + p2[1] + p3[1] + p4[1]);
  r[2] = (p1[2] + p2[2] + p3[2] + p4[2]);
  r[0] *= 0.25; r[1] *= 0.25; r[2] *= 0.25;
}
inline void tri_area(const double* p1, const double* p2, const double* p3, double* r) {
  double v1[3], v2[3];
  sub3(p2, p1, v1); sub3(p3, p1, v2);
  cross3(v1, v2, r);
  r[0] = 0.5 * r[0]; r[1] = 0.5 * r[1]; r[2] = 0.5 * r[2];
}
inline double tet_vol(const double* p1, const double* p2, const double* p3, const double* p4) {
  double v1[3], v2[3], v3[3], t[3];
  sub3(p2, p1, v1); sub3(p3, p1, v2); sub3(p4, p1, v3);
  cross3(v1, v2, t);
  return (v3[0] * t[0] + v3[1] * t[1] + v3[2] * t[2]) / 6.0;
}

// ---- deterministic, platform-independent random numbers --------------------
struct SplitMix64 {
  uint64_t s;
  explicit SplitMix64(uint64_t seed) : s(seed) {}
  uint64_t next() {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  }
  // uniform in [-1, 1)
  double sym() { return ((double)(next() >> 11) * (1.0 / 9007199254740992.0)) * 2.0 - 1.0; }
};

// Reference element-local neighbour tables (ucs/mesh.tcc:541-548) for TRI/TET.
const int kClTri[6] = {1, 2, 2, 0, 0, 1};
const int kClTet[12] = {1, 2, 3, 2, 0, 3, 0, 1, 3, 0, 1, 2};
// Tet edge orientation, edge->face and face->node tables (ucs/mesh.tcc:1696-1790)
const int kTetEorder[12] = {0, 1, 0, 2, 0, 3, 1, 2, 1, 3, 2, 3};
const int kTetE2f[12] = {0, 1, 2, 0, 1, 2, 0, 3, 3, 1, 2, 3};
const int kTetFl[12] = {0, 1, 2, 0, 3, 1, 0, 2, 3, 1, 3, 2};

int elem_nnodes(int t) { return t == ETRI ? 3 : 4; }

// Mesh::EliminateRepeats (ucs/mesh.tcc:1341): keeps the first occurrence of
// each value, in order.  The lists are a node's element neighbours (a few
// dozen values), so a search of the kept prefix is enough.
int eliminate_repeats(int* a, int n) {
  int unique = 0;
  for (int i = 0; i < n; i++) {
    const int v = a[i];
    bool seen = false;
    for (int j = 0; j < unique; j++)
      if (a[j] == v) { seen = true; break; }
    if (!seen) a[unique++] = v;
  }
  return unique;
}

// Splits [0, n) into contiguous chunks, one per host thread (one chunk below
// a size where threads do not pay), and runs body(begin, end, chunk) on
// each.  Each chunk writes only its own outputs, so results do not depend on
// the thread count.  A chunk whose thread cannot be started runs on the
// calling thread; an exception in any chunk is raised again here after all
// chunks finished.  Returns the number of chunks.
template <class F>
int parallel_chunks(long long n, F body) {
  unsigned nt = std::thread::hardware_concurrency();
  if (nt == 0) nt = 1;
  if (nt > 64) nt = 64;
  if (n < 65536 || nt == 1) {
    body(0LL, n, 0);
    return 1;
  }
  const long long chunk = (n + nt - 1) / nt;
  std::vector<std::thread> pool;
  std::vector<std::exception_ptr> fail(nt);
  auto run = [&](long long b, long long e, int c) {
    try {
      body(b, e, c);
    } catch (...) {
      fail[c] = std::current_exception();
    }
  };
  int nc = 0;
  for (unsigned t = 0; t < nt; t++) {
    const long long b = (long long)t * chunk, e = std::min(n, b + chunk);
    if (b >= e) break;
    const int c = nc++;
    try {
      pool.emplace_back(run, b, e, c);
    } catch (...) {
      run(b, e, c);
    }
  }
  for (auto& th : pool) th.join();
  for (auto& f : fail)
    if (f) std::rethrow_exception(f);
  return nc;
}
template <class F>
void parallel_ranges(long long n, F body) {
  parallel_chunks(n, [&](long long b, long long e, int) { body(b, e); });
}

int build_psp_only(HostMesh& m) {
  const int nn = m.nnode;
  const int ne = (int)m.etype.size();
  // BuildElsp
  m.ielsp.assign(nn + 1, 0);
  for (int e = 0; e < ne; e++)
    for (int j = 0; j < elem_nnodes(m.etype[e]); j++) {
      int node = m.enodes[4 * e + j];
      if (node < 0 || node >= nn) { m.err = "element node id out of range"; return -1; }
      m.ielsp[node + 1]++;
    }
  for (int i = 1; i <= nn; i++) m.ielsp[i] += m.ielsp[i - 1];
  m.elsp.assign(m.ielsp[nn], 0);
  {
    std::vector<int> fill(m.ielsp.begin(), m.ielsp.end() - 1);
    for (int e = 0; e < ne; e++)
      for (int j = 0; j < elem_nnodes(m.etype[e]); j++) {
        int node = m.enodes[4 * e + j];
        m.elsp[fill[node]++] = e;
      }
  }
  // BuildPsp: per node, the other nodes of its elements in elsp order
  // (kClTri / kClTet), first occurrences kept.  Nodes are independent: each
  // chunk of nodes builds its own lists, concatenated in node order.
  m.ipsp.assign(nn + 1, 0);
  std::vector<std::vector<int>> part(64);
  parallel_chunks(nn, [&](long long b, long long e, int c) {
    std::vector<int>& out = part[c];
    out.reserve((size_t)(e - b) * 16);
    std::vector<int> tmp;
    for (long long i = b; i < e; i++) {
      tmp.clear();
      for (int k = m.ielsp[i]; k < m.ielsp[i + 1]; k++) {
        const int el = m.elsp[k];
        const int* nodes = &m.enodes[4 * (size_t)el];
        const int nl = elem_nnodes(m.etype[el]);
        int lnode = -1;
        for (int q = 0; q < nl; q++)
          if (nodes[q] == i) { lnode = q; break; }
        if (m.etype[el] == ETRI) {
          for (int q = 0; q < 2; q++) tmp.push_back(nodes[kClTri[2 * lnode + q]]);
        } else {
          for (int q = 0; q < 3; q++) tmp.push_back(nodes[kClTet[3 * lnode + q]]);
        }
      }
      const int u = eliminate_repeats(tmp.data(), (int)tmp.size());
      out.insert(out.end(), tmp.begin(), tmp.begin() + u);
      m.ipsp[i + 1] = u;
    }
  });
  for (int i = 0; i < nn; i++) m.ipsp[i + 1] += m.ipsp[i];
  m.psp.resize((size_t)m.ipsp[nn]);
  {
    size_t off = 0;
    for (auto& pv : part) {
      std::copy(pv.begin(), pv.end(), m.psp.begin() + off);
      off += pv.size();
      std::vector<int>().swap(pv);
    }
  }
  return 0;
}

int build_maps(HostMesh& m) {
  if (build_psp_only(m) != 0) return -1;
  const int nn = m.nnode;
  const int ne = (int)m.etype.size();
  // FixBoundaryWindings: every boundary triangle must face away from its tet.
  // The generator winds them outward already; this counts any that are not
  // and rewinds them the way the reference does (nodes 2,1,0).
  {
    m.rewound = 0;
    for (int e = 0; e < ne; e++) {
      if (m.etype[e] != ETRI) continue;
      int* tn = &m.enodes[4 * e];
      // find the unique tet holding all three nodes
      int owner = -1;
      for (int k = m.ielsp[tn[0]]; k < m.ielsp[tn[0] + 1]; k++) {
        int t = m.elsp[k];
        if (m.etype[t] != ETET) continue;
        const int* q = &m.enodes[4 * t];
        int hits = 0;
        for (int a = 0; a < 3; a++)
          for (int b = 0; b < 4; b++) hits += (tn[a] == q[b]);
        if (hits == 3) { owner = t; break; }
      }
      if (owner < 0) { m.err = "boundary face without a volume element"; return -1; }
      double bpt[3], ept[3], ne3[3], nb[3];
      cen3(&m.xyz[3 * tn[0]], &m.xyz[3 * tn[1]], &m.xyz[3 * tn[2]], bpt);
      const int* q = &m.enodes[4 * owner];
      cen4(&m.xyz[3 * q[0]], &m.xyz[3 * q[1]], &m.xyz[3 * q[2]], &m.xyz[3 * q[3]], ept);
      sub3(bpt, ept, ne3);
      tri_area(&m.xyz[3 * tn[0]], &m.xyz[3 * tn[1]], &m.xyz[3 * tn[2]], nb);
      normalize3(ne3, ne3);
      normalize3(nb, nb);
      double dot = ne3[0] * nb[0] + ne3[1] * nb[1] + ne3[2] * nb[2];
      if (!(dot > 0.0)) {
        std::swap(tn[0], tn[2]);
        m.rewound++;
      }
    }
  }
  // BuildEdges: interior edges (i < psp[j]) in node-then-psp order
  m.edges.clear();
  for (int i = 0; i < nn; i++)
    for (int j = m.ipsp[i]; j < m.ipsp[i + 1]; j++)
      if (m.psp[j] > i) { m.edges.push_back(i); m.edges.push_back(m.psp[j]); }
  m.nedge = (int)m.edges.size() / 2;
  // boundary half-edges: one per (boundary face, face node), phantom ids from nnode
  m.bedges.clear(); m.belem.clear(); m.bfactag.clear();
  int jj = nn;
  for (int e = 0; e < ne; e++) {
    if (m.etype[e] != ETRI) continue;
    for (int j = 0; j < 3; j++) {
      m.bedges.push_back(m.enodes[4 * e + j]);
      m.bedges.push_back(jj++);
      m.belem.push_back(e);
      m.bfactag.push_back(m.efactag[e]);
    }
  }
  m.nbedge = (int)m.belem.size();
  m.maps_built = 1;
  return 0;
}

// The median-dual pieces of edge (n1, n2) inside element e, as
// CalcAreasVolumes forms them (ucs/mesh.tcc:1822-1985): the edge midpoint,
// the centroids of the two faces that share the edge, the element centroid,
// and the orientation of the edge in the element's edge table.  False when e
// is not a tet holding both nodes.
struct EdgeTetGeom {
  double o, edgept[3], f1[3], f2[3], ept[3];
};
inline bool edge_tet_geom(const HostMesh& m, int n1, int n2, int e, EdgeTetGeom& g) {
  if (m.etype[e] != ETET) return false;
  const int* nodes = &m.enodes[4 * (size_t)e];
  int l1 = -1, l2 = -1;
  for (int q = 0; q < 4; q++) {
    if (nodes[q] == n1) l1 = q;
    else if (nodes[q] == n2) l2 = q;
  }
  if (l1 < 0 || l2 < 0) return false;  // edge not in this element
  int orientation = 0, eid = -1;
  for (int j = 0; j < 6; j++) {
    if (kTetEorder[2 * j] == l1 && kTetEorder[2 * j + 1] == l2) { eid = j; orientation = 1; break; }
    if (kTetEorder[2 * j + 1] == l1 && kTetEorder[2 * j] == l2) { eid = j; orientation = -1; break; }
  }
  const double* X = m.xyz.data();
  const int face1 = kTetE2f[2 * eid], face2 = kTetE2f[2 * eid + 1];
  mid2(&X[3 * (size_t)n1], &X[3 * (size_t)n2], g.edgept);
  const int* fa = &kTetFl[3 * face1];
  cen3(&X[3 * (size_t)nodes[fa[0]]], &X[3 * (size_t)nodes[fa[1]]], &X[3 * (size_t)nodes[fa[2]]], g.f1);
  const int* fb = &kTetFl[3 * face2];
  cen3(&X[3 * (size_t)nodes[fb[0]]], &X[3 * (size_t)nodes[fb[1]]], &X[3 * (size_t)nodes[fb[2]]], g.f2);
  cen4(&X[3 * (size_t)nodes[0]], &X[3 * (size_t)nodes[1]], &X[3 * (size_t)nodes[2]], &X[3 * (size_t)nodes[3]],
       g.ept);
  g.o = (double)orientation;
  return true;
}

// Calls fn(g) for each tet holding edge (n1, n2), in the order the
// reference visits them: the second node's elements in elsp order.  Every
// node's elsp list is in ascending element order (BuildElsp fills them
// element by element), so the tets holding both nodes are the merge
// intersection of the two lists, in that same order; only those tets' node
// lists are read.
template <class F>
inline void for_edge_tets(const HostMesh& m, int n1, int n2, EdgeTetGeom& g, F fn) {
  int a = m.ielsp[n1], ae = m.ielsp[n1 + 1];
  int b = m.ielsp[n2], be = m.ielsp[n2 + 1];
  while (a < ae && b < be) {
    const int ea = m.elsp[a], eb = m.elsp[b];
    if (ea < eb) {
      a++;
    } else if (eb < ea) {
      b++;
    } else {
      if (edge_tet_geom(m, n1, n2, eb, g)) fn(g);
      a++;
      b++;
    }
  }
}

int calc_metrics(HostMesh& m) {
  const int nn = m.nnode;
  m.vol.assign(nn, 0.0);
  // every tet must be right-handed (positive volume in the reference's
  // CalcTetVol convention) for the dual areas to point from n[0] to n[1]
  {
    std::atomic<int> inverted(0);
    parallel_ranges((long long)m.etype.size(), [&](long long b, long long e) {
      int bad = 0;
      for (long long t = b; t < e; t++) {
        if (m.etype[t] != ETET) continue;
        const int* q = &m.enodes[4 * t];
        if (!(tet_vol(&m.xyz[3 * (size_t)q[0]], &m.xyz[3 * (size_t)q[1]], &m.xyz[3 * (size_t)q[2]],
                      &m.xyz[3 * (size_t)q[3]]) > 0.0))
          bad++;
      }
      inverted += bad;
    });
    m.inverted = inverted.load();
  }
  if (m.inverted) {
    m.err = "mesh has " + std::to_string(m.inverted) + " inverted or degenerate tetrahedra";
    return -1;
  }
  m.ea.assign((size_t)4 * m.nedge, 0.0);
  m.ba.assign((size_t)4 * m.nbedge, 0.0);
  const double* X = m.xyz.data();
  // interior edges: two dual-face triangles and four sub-volumes per
  // surrounding element (CalcAreasVolumes, ucs/mesh.tcc:1822-1985).  The
  // reference visits the edges in order and, per edge, the elements of its
  // second node in elsp order, adding the face triangles to the edge's area
  // and two sub-volumes to each end's volume.  Here the areas are formed per
  // edge (in parallel: each edge owns its area), and each node's volume by
  // one thread that visits the node's edges in ascending edge order - the
  // reference's sequence of additions to that node, so the sums are
  // bit-identical whatever the thread count.
  parallel_ranges(m.nedge, [&](long long b, long long e) {
    EdgeTetGeom g;
    for (long long i = b; i < e; i++) {
      const int n1 = m.edges[2 * i], n2 = m.edges[2 * i + 1];
      double* a = &m.ea[4 * i];
      for_edge_tets(m, n1, n2, g, [&](const EdgeTetGeom& t) {
        double area[3];
        tri_area(t.ept, t.f2, t.edgept, area);
        area[0] = t.o * area[0]; area[1] = t.o * area[1]; area[2] = t.o * area[2];
        a[0] = a[0] + area[0]; a[1] = a[1] + area[1]; a[2] = a[2] + area[2];
        tri_area(t.edgept, t.f1, t.ept, area);
        area[0] = t.o * area[0]; area[1] = t.o * area[1]; area[2] = t.o * area[2];
        a[0] = a[0] + area[0]; a[1] = a[1] + area[1]; a[2] = a[2] + area[2];
      });
    }
  });
  // boundary half-edges: two triangles of the boundary face's median dual
  // (ucs/mesh.tcc:2148-2190); each half-edge owns its area
  parallel_ranges(m.nbedge, [&](long long b, long long e) {
    for (long long i = b; i < e; i++) {
      const int n1 = m.bedges[2 * i];
      const int* nodes = &m.enodes[4 * (size_t)m.belem[i]];
      int nid = -1;
      for (int q = 0; q < 3; q++)
        if (nodes[q] == n1) nid = q;
      double ept[3], edgept[3], area[3];
      cen3(&X[3 * (size_t)nodes[0]], &X[3 * (size_t)nodes[1]], &X[3 * (size_t)nodes[2]], ept);
      int alt = nodes[kClTri[2 * nid]];
      mid2(&X[3 * (size_t)n1], &X[3 * (size_t)alt], edgept);
      tri_area(ept, &X[3 * (size_t)n1], edgept, area);
      double* a = &m.ba[4 * i];
      a[0] = a[0] + area[0]; a[1] = a[1] + area[1]; a[2] = a[2] + area[2];
      alt = nodes[kClTri[2 * nid + 1]];
      mid2(&X[3 * (size_t)n1], &X[3 * (size_t)alt], edgept);
      tri_area(edgept, &X[3 * (size_t)n1], ept, area);
      a[0] = a[0] + area[0]; a[1] = a[1] + area[1]; a[2] = a[2] + area[2];
    }
  });
  // Per node: the dual volume, the closure sum of CheckForClosure
  // (ucs/mesh.tcc:2274; the signed face areas, before they are normalised)
  // and the weighted LSQ normal matrix (Kernel_LSQ_CoefficientsWeighted,
  // ucs/gradient.tcc:461; the boundary variant only adds for ghost nodes,
  // which a single partition does not have).  The reference accumulates all
  // three edge by edge into both ends; here one thread forms a node's sums
  // over its edges in ascending edge order (then, for the closure sum, its
  // half-edges in ascending order): the same additions in the same order.
  m.sw.assign((size_t)6 * nn, 0.0);
  {
    // a node's interior edges, ascending, with the node's end (bit 0: 0 the
    // edge's first node, 1 its second); its boundary half-edges, ascending
    std::vector<int> iptr(nn + 1, 0), bptr(nn + 1, 0);
    for (int i = 0; i < m.nedge; i++) {
      iptr[m.edges[2 * i] + 1]++;
      iptr[m.edges[2 * i + 1] + 1]++;
    }
    for (int i = 0; i < m.nbedge; i++) bptr[m.bedges[2 * i] + 1]++;
    for (int i = 0; i < nn; i++) {
      iptr[i + 1] += iptr[i];
      bptr[i + 1] += bptr[i];
    }
    std::vector<uint32_t> inc((size_t)iptr[nn]);
    std::vector<int> binc((size_t)bptr[nn]);
    {
      std::vector<int> fill(iptr.begin(), iptr.end() - 1);
      for (int i = 0; i < m.nedge; i++) {
        inc[fill[m.edges[2 * i]]++] = (uint32_t)i << 1;
        inc[fill[m.edges[2 * i + 1]]++] = ((uint32_t)i << 1) | 1u;
      }
      std::vector<int> bfill(bptr.begin(), bptr.end() - 1);
      for (int i = 0; i < m.nbedge; i++) binc[bfill[m.bedges[2 * i]]++] = i;
    }
    std::vector<double> open(nn);
    parallel_ranges(nn, [&](long long b, long long e) {
      EdgeTetGeom g;
      for (long long n = b; n < e; n++) {
        double v = 0.0, sc[3] = {0.0, 0.0, 0.0}, w[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
        for (int t = iptr[n]; t < iptr[n + 1]; t++) {
          const uint32_t i = inc[t] >> 1;
          const bool second = (inc[t] & 1u) != 0;
          const int n1 = m.edges[2 * (size_t)i], n2 = m.edges[2 * (size_t)i + 1];
          for_edge_tets(m, n1, n2, g, [&](const EdgeTetGeom& t) {
            if (!second) {
              const double* p1 = &X[3 * (size_t)n1];
              v += t.o * tet_vol(p1, t.ept, t.f2, t.edgept);
              v += t.o * tet_vol(p1, t.f1, t.ept, t.edgept);
            } else {
              const double* p2 = &X[3 * (size_t)n2];
              v += t.o * tet_vol(p2, t.ept, t.f1, t.edgept);
              v += t.o * tet_vol(p2, t.f2, t.ept, t.edgept);
            }
          });
          const double* a = &m.ea[4 * (size_t)i];
          for (int c = 0; c < 3; c++) sc[c] = second ? sc[c] + a[c] : sc[c] - a[c];
          double dx[3];
          sub3(&X[3 * (size_t)n1], &X[3 * (size_t)n2], dx);
          const double ds2 = 1.0 / (dx[0] * dx[0] + dx[1] * dx[1] + dx[2] * dx[2]);
          double tt[6];
          if (!second) {
            tt[0] = dx[0] * dx[0] * ds2;
            tt[1] = dx[0] * dx[1] * ds2;
            tt[2] = dx[0] * dx[2] * ds2;
            tt[3] = dx[1] * dx[1] * ds2;
            tt[4] = dx[1] * dx[2] * ds2;
            tt[5] = dx[2] * dx[2] * ds2;
          } else {
            // the second node's terms are formed from the negated difference
            tt[0] = dx[0] * dx[0] * ds2;
            tt[3] = dx[1] * dx[1] * ds2;
            tt[5] = dx[2] * dx[2] * ds2;
            dx[0] = -dx[0]; dx[1] = -dx[1]; dx[2] = -dx[2];
            tt[1] = (dx[0] * dx[1]) * ds2;
            tt[2] = (dx[0] * dx[2]) * ds2;
            tt[4] = (dx[1] * dx[2]) * ds2;
          }
          for (int c = 0; c < 6; c++) w[c] += tt[c];
        }
        for (int t = bptr[n]; t < bptr[n + 1]; t++) {
          const double* a = &m.ba[4 * (size_t)binc[t]];
          for (int c = 0; c < 3; c++) sc[c] = sc[c] - a[c];
        }
        m.vol[n] = v;
        for (int c = 0; c < 6; c++) m.sw[6 * n + c] = w[c];
        open[n] = mag3(sc);
      }
    });
    m.unclosed = 0;
    m.max_open = 0.0;
    for (int i = 0; i < nn; i++) {
      if (open[i] > m.max_open) m.max_open = open[i];
      if (open[i] > 1.0e-10) m.unclosed++;
    }
  }
  parallel_ranges(m.nedge, [&](long long b, long long e) {
    for (long long i = b; i < e; i++) m.ea[4 * i + 3] = normalize3(&m.ea[4 * i], &m.ea[4 * i]);
  });
  parallel_ranges(m.nbedge, [&](long long b, long long e) {
    for (long long i = b; i < e; i++) m.ba[4 * i + 3] = normalize3(&m.ba[4 * i], &m.ba[4 * i]);
  });
  m.metrics_built = 1;
  return 0;
}

// Cuthill-McKee ordering exactly as Mesh::ReorderMeshCuthillMcKee computes it
// (ucs/mesh.tcc:2412-2490): node 0 is the first vertex; the unused
// neighbours of the current vertex, in psp order, are queued as (node,
// degree) pairs, sorted by ascending degree with std::sort and the
// reference's comparison (DegreeCompare, ucs/oddsNends.cpp:4-7) - the same
// libstdc++ sort on the same sequence, so equal-degree ties fall the same
// way - appended to the ordering and to the breadth-first queue; when that
// queue runs dry the next vertex is the first unused node.  The list is then
// reversed.  The reference scans every node each pass to test for unused
// ones (NegativeQueue, :9-17, O(N^2)); a running count gives the same test.
struct IntInt {
  int a, b;
};
bool degree_compare(IntInt i, IntInt j) { return i.b < j.b; }

int ref_cuthill_mckee(const HostMesh& m, std::vector<int>& ordering, std::string& err) {
  const int nn = m.nnode;
  ordering.assign(nn, 0);
  if (nn == 0) return 0;
  std::vector<IntInt> Q(nn);
  for (int j = 0; j < nn; j++) {
    Q[j].a = j;
    Q[j].b = m.ipsp[j + 1] - m.ipsp[j];
  }
  std::deque<int> S;
  std::deque<IntInt> R;
  int i = 0;
  const int startnode = 0;
  ordering[i] = startnode;
  int z = ordering[i];
  Q[startnode].a = -1;
  long long unused = nn - 1;
  long long stalls = 0;
  while (unused > 0) {
    const long long before = unused;
    for (int k = m.ipsp[z]; k < m.ipsp[z + 1]; k++) {
      const int nb = m.psp[k];
      if (nb < nn && Q[nb].a >= 0) {
        R.push_back(Q[nb]);
        Q[nb].a = -1;
        unused--;
      }
    }
    std::sort(R.begin(), R.end(), degree_compare);
    while (!R.empty()) {
      i++;
      ordering[i] = R.front().a;
      R.pop_front();
      S.push_back(ordering[i]);
    }
    if (!S.empty()) {
      z = S.front();
      S.pop_front();
    } else {
      for (int j = 0; j < nn; j++)
        if (Q[j].a >= 0) { z = j; break; }
    }
    // The reference never marks a re-seeded vertex used, so a component whose
    // re-seed has no unused neighbour would loop forever there; stop instead.
    stalls = (unused == before && S.empty()) ? stalls + 1 : 0;
    if (stalls > 1) {
      err = "Cuthill-McKee: disconnected mesh (an isolated node) cannot be ordered";
      return -1;
    }
  }
  // reverse (ReorderMeshCuthillMcKee(1))
  std::reverse(ordering.begin(), ordering.end());
  return 0;
}

// Mesh::ReorderC2nMap (ucs/mesh.tcc:224-262): the reference applies the
// ordering as an old-to-new map, node n of every element becomes ordering[n]
// and the coordinates of node i move to ordering[i].
void apply_c2n_map(HostMesh& m, const std::vector<int>& ordering) {
  for (size_t e = 0; e < m.etype.size(); e++)
    for (int q = 0; q < elem_nnodes(m.etype[e]); q++) m.enodes[4 * e + q] = ordering[m.enodes[4 * e + q]];
  std::vector<double> x2((size_t)3 * m.nnode);
  for (int i = 0; i < m.nnode; i++)
    for (int c = 0; c < 3; c++) x2[3 * (size_t)ordering[i] + c] = m.xyz[3 * (size_t)i + c];
  m.xyz.swap(x2);
  m.maps_built = m.metrics_built = 0;
}

// Element-surrounding-point and point-surrounding-point maps only
// (Mesh::BuildMapsDecomp, ucs/mesh.tcc:316), as the reorder needs them.
int build_psp_only(HostMesh& m);

thread_local std::string g_last_mesh_error;

}  // namespace

extern "C" {

PCFD_API pcfd_mesh_t pcfd_mesh_box_create(const pcfd_box_params* p) {
  if (!p || p->nx < 2 || p->ny < 2 || p->nz < 2) {
    g_last_mesh_error = "pcfd_mesh_box_create: need nx, ny, nz >= 2";
    return nullptr;
  }
  const long long nnode_ll = (long long)p->nx * p->ny * p->nz;
  if (nnode_ll > 400000000LL) {
    g_last_mesh_error = "pcfd_mesh_box_create: box too large";
    return nullptr;
  }
  HostMesh* m = new (std::nothrow) HostMesh();
  if (!m) return nullptr;
  const int nx = p->nx, ny = p->ny, nz = p->nz;
  m->nnode = (int)nnode_ll;
  auto id = [&](int i, int j, int k) { return i + nx * (j + ny * k); };
  // 1-D node coordinates per axis; y may be geometrically clustered toward y=0
  std::vector<double> cx(nx), cy(ny), cz(nz);
  for (int i = 0; i < nx; i++) cx[i] = p->lx * (double)i / (double)(nx - 1);
  for (int k = 0; k < nz; k++) cz[k] = p->lz * (double)k / (double)(nz - 1);
  if (p->y_ratio > 1.0) {
    // spacings in units of ly: h0 r^k, capped at hc
    double h0 = (p->y_ratio - 1.0) / (std::pow(p->y_ratio, (double)(ny - 1)) - 1.0);
    double hc = 1e300;
    const double h0_min = p->wall_ar_max > 0.0 ? p->lx / (double)(nx - 1) / p->ly / p->wall_ar_max : 0.0;
    if (h0 < h0_min) {
      // the cap hc that makes the ny-1 spacings sum to 1, by bisection
      h0 = h0_min;
      auto total = [&](double cap) {
        double s = 0.0, h = h0;
        for (int j = 0; j < ny - 1; j++) {
          s += std::min(h, cap);
          h *= p->y_ratio;
        }
        return s;
      };
      double lo = h0, hi = 1.0;
      for (int it = 0; it < 200; it++) {
        const double mid = 0.5 * (lo + hi);
        if (mid <= lo || mid >= hi) break;
        if (total(mid) < 1.0) lo = mid; else hi = mid;
      }
      hc = hi;
    }
    double y = 0.0, h = h0;
    for (int j = 0; j < ny; j++) {
      cy[j] = p->ly * y;
      y += std::min(h, hc);
      h *= p->y_ratio;
    }
    cy[ny - 1] = p->ly;
  } else {
    for (int j = 0; j < ny; j++) cy[j] = p->ly * (double)j / (double)(ny - 1);
  }
  auto local_h = [](const std::vector<double>& c, int i) {
    int n = (int)c.size();
    double hl = i > 0 ? c[i] - c[i - 1] : 1e300;
    double hr = i < n - 1 ? c[i + 1] - c[i] : 1e300;
    return std::min(hl, hr);
  };
  m->xyz.resize((size_t)3 * m->nnode);
  SplitMix64 rng(p->seed);
  const double tanr = std::tan(p->ramp_deg * 3.14159265358979323846 / 180.0);
  for (int k = 0; k < nz; k++)
    for (int j = 0; j < ny; j++)
      for (int i = 0; i < nx; i++) {
        double x = cx[i], y = cy[j], z = cz[k];
        bool interior = i > 0 && i < nx - 1 && j > 0 && j < ny - 1 && k > 0 && k < nz - 1;
        if (interior && p->jitter > 0.0) {
          double hx = local_h(cx, i), hy = local_h(cy, j), hz = local_h(cz, k);
          if (p->jitter_mode == 1) hx = hy = hz = std::min(hx, std::min(hy, hz));
          x += p->jitter * hx * rng.sym();
          y += p->jitter * hy * rng.sym();
          z += p->jitter * hz * rng.sym();
        }
        if (p->ramp_deg != 0.0 && x > p->ramp_x0) {
          // shear y so the bottom wall ramps up by ramp_deg and the top stays flat
          y = y + tanr * (x - p->ramp_x0) * (p->ly - y) / p->ly;
        }
        size_t n = (size_t)id(i, j, k);
        m->xyz[3 * n + 0] = x;
        m->xyz[3 * n + 1] = y;
        m->xyz[3 * n + 2] = z;
      }
  // boundary triangles: two per boundary quad, split along the diagonal the
  // Kuhn tets use (the one through the hex corner (0,0,0) or (1,1,1)),
  // wound so the normal points out of the box.
  auto push_tri = [&](int a, int b, int c, int tag, const double* out) {
    double n[3];
    tri_area(&m->xyz[3 * (size_t)a], &m->xyz[3 * (size_t)b], &m->xyz[3 * (size_t)c], n);
    if (n[0] * out[0] + n[1] * out[1] + n[2] * out[2] < 0.0) std::swap(a, c);
    m->etype.push_back(ETRI);
    m->enodes.push_back(a); m->enodes.push_back(b); m->enodes.push_back(c); m->enodes.push_back(-1);
    m->efactag.push_back(tag);
  };
  // face order: x=0, x=max, y=0, y=max, z=0, z=max
  for (int f = 0; f < 6; f++) {
    int axis = f / 2, side = f % 2;
    double out[3] = {0, 0, 0};
    out[axis] = side ? 1.0 : -1.0;
    const int tag_f = p->tags[f];
    int na = axis == 0 ? ny : nx;  // first in-face axis extent
    int nb = axis == 2 ? ny : nz;  // second in-face axis extent
    for (int b = 0; b < nb - 1; b++)
      for (int a = 0; a < na - 1; a++) {
        int c[2][2][2];
        int ci, cj, ck;
        if (axis == 0) { ci = side ? nx - 2 : 0; cj = a; ck = b; }
        else if (axis == 1) { ci = a; cj = side ? ny - 2 : 0; ck = b; }
        else { ci = a; cj = b; ck = side ? nz - 2 : 0; }
        const int tag = (f == 2 && ci < p->wall_start_i) ? p->upstream_tag : tag_f;
        for (int u = 0; u < 2; u++)
          for (int v = 0; v < 2; v++)
            for (int w = 0; w < 2; w++) c[u][v][w] = id(ci + u, cj + v, ck + w);
        // the four face corners in cyclic order and the diagonal endpoints
        int q0, q1, q2, q3;  // q0 and q2 are the diagonal
        if (axis == 0) {
          int s = side;
          // face corners (s, v, w)
          if (!s) { q0 = c[0][0][0]; q1 = c[0][1][0]; q2 = c[0][1][1]; q3 = c[0][0][1]; }
          else { q0 = c[1][0][0]; q1 = c[1][1][0]; q2 = c[1][1][1]; q3 = c[1][0][1]; }
        } else if (axis == 1) {
          int s = side;
          if (!s) { q0 = c[0][0][0]; q1 = c[1][0][0]; q2 = c[1][0][1]; q3 = c[0][0][1]; }
          else { q0 = c[0][1][0]; q1 = c[1][1][0]; q2 = c[1][1][1]; q3 = c[0][1][1]; }
        } else {
          int s = side;
          if (!s) { q0 = c[0][0][0]; q1 = c[1][0][0]; q2 = c[1][1][0]; q3 = c[0][1][0]; }
          else { q0 = c[0][0][1]; q1 = c[1][0][1]; q2 = c[1][1][1]; q3 = c[0][1][1]; }
        }
        push_tri(q0, q1, q2, tag, out);
        push_tri(q0, q2, q3, tag, out);
      }
  }
  // Kuhn tets: for each permutation (s0,s1,s2) of the axes, the path
  // c000 -> +e_s0 -> +e_s1 -> c111; odd permutations are flipped so every tet
  // is right-handed (positive reference volume).
  const int perms[6][3] = {{0, 1, 2}, {0, 2, 1}, {1, 0, 2}, {1, 2, 0}, {2, 0, 1}, {2, 1, 0}};
  const int parity[6] = {0, 1, 1, 0, 0, 1};
  for (int k = 0; k < nz - 1; k++)
    for (int j = 0; j < ny - 1; j++)
      for (int i = 0; i < nx - 1; i++)
        for (int t = 0; t < 6; t++) {
          int off[3] = {0, 0, 0};
          int v[4];
          v[0] = id(i, j, k);
          off[perms[t][0]] = 1;
          v[1] = id(i + off[0], j + off[1], k + off[2]);
          off[perms[t][1]] = 1;
          v[2] = id(i + off[0], j + off[1], k + off[2]);
          v[3] = id(i + 1, j + 1, k + 1);
          if (parity[t]) std::swap(v[1], v[2]);
          m->etype.push_back(ETET);
          for (int q = 0; q < 4; q++) m->enodes.push_back(v[q]);
          m->efactag.push_back(0);
        }
  return (pcfd_mesh_t)m;
}

PCFD_API pcfd_mesh_t pcfd_mesh_from_elements(int nnode, const double* xyz, int ntri, const int* tri,
                                             const int* tri_tag, int ntet, const int* tet) {
  if (nnode <= 0 || !xyz || ntri < 0 || ntet <= 0 || !tet || (ntri > 0 && (!tri || !tri_tag))) {
    g_last_mesh_error = "pcfd_mesh_from_elements: bad arguments";
    return nullptr;
  }
  HostMesh* m = new (std::nothrow) HostMesh();
  if (!m) return nullptr;
  m->nnode = nnode;
  m->xyz.assign(xyz, xyz + (size_t)3 * nnode);
  for (int e = 0; e < ntri; e++) {
    m->etype.push_back(ETRI);
    for (int q = 0; q < 3; q++) m->enodes.push_back(tri[3 * e + q]);
    m->enodes.push_back(-1);
    m->efactag.push_back(tri_tag[e]);
  }
  for (int e = 0; e < ntet; e++) {
    m->etype.push_back(ETET);
    for (int q = 0; q < 4; q++) m->enodes.push_back(tet[4 * e + q]);
    m->efactag.push_back(0);
  }
  return (pcfd_mesh_t)m;
}

PCFD_API int pcfd_mesh_build(pcfd_mesh_t h) {
  if (!h) return PCFD_ERR_ARG;
  HostMesh* m = (HostMesh*)h;
  try {
    if (build_maps(*m) != 0) { g_last_mesh_error = m->err; return PCFD_ERR_MESH; }
    if (calc_metrics(*m) != 0) { g_last_mesh_error = m->err; return PCFD_ERR_MESH; }
  } catch (const std::bad_alloc&) {
    g_last_mesh_error = "pcfd_mesh_build: out of host memory";
    return PCFD_ERR_NOMEM;
  } catch (const std::exception& e) {
    g_last_mesh_error = std::string("pcfd_mesh_build: ") + e.what();
    return PCFD_ERR_MESH;
  }
  return PCFD_OK;
}

PCFD_API int pcfd_mesh_view_get(pcfd_mesh_t h, pcfd_mesh_view* v) {
  if (!h || !v) return PCFD_ERR_ARG;
  HostMesh* m = (HostMesh*)h;
  if (!m->maps_built || !m->metrics_built) return PCFD_ERR_STATE;
  std::memset(v, 0, sizeof(*v));
  v->nnode = m->nnode;
  v->nbnode = m->nbedge;
  v->nedge = m->nedge;
  v->nbedge = m->nbedge;
  v->edges = m->edges.data();
  v->edge_area = m->ea.data();
  v->bedges = m->bedges.data();
  v->bedge_area = m->ba.data();
  v->bfactag = m->bfactag.data();
  v->xyz = m->xyz.data();
  v->vol = m->vol.data();
  v->sw = m->sw.data();
  v->ipsp = m->ipsp.data();
  v->psp = m->psp.data();
  return PCFD_OK;
}

PCFD_API int pcfd_mesh_stats(pcfd_mesh_t h, int* nelem_tri, int* nelem_tet, int* rewound, int* unclosed,
                             double* max_open, double* total_vol) {
  if (!h) return PCFD_ERR_ARG;
  HostMesh* m = (HostMesh*)h;
  int nt = 0, nk = 0;
  for (int t : m->etype) (t == ETRI ? nt : nk)++;
  if (nelem_tri) *nelem_tri = nt;
  if (nelem_tet) *nelem_tet = nk;
  if (rewound) *rewound = m->rewound;
  if (unclosed) *unclosed = m->unclosed;
  if (max_open) *max_open = m->max_open;
  if (total_vol) {
    double s = 0.0;
    for (double x : m->vol) s += x;
    *total_vol = s;
  }
  return PCFD_OK;
}

PCFD_API int pcfd_mesh_rcm_order(pcfd_mesh_t h, int* order_out) {
  if (!h || !order_out) return PCFD_ERR_ARG;
  HostMesh* m = (HostMesh*)h;
  if (!m->maps_built && build_psp_only(*m) != 0) { g_last_mesh_error = m->err; return PCFD_ERR_MESH; }
  std::vector<int> ordering;
  if (ref_cuthill_mckee(*m, ordering, m->err) != 0) { g_last_mesh_error = m->err; return PCFD_ERR_MESH; }
  std::memcpy(order_out, ordering.data(), sizeof(int) * ordering.size());
  return PCFD_OK;
}

PCFD_API int pcfd_mesh_reorder_rcm(pcfd_mesh_t h, int* order_out) {
  if (!h) return PCFD_ERR_ARG;
  HostMesh* m = (HostMesh*)h;
  if (build_psp_only(*m) != 0) { g_last_mesh_error = m->err; return PCFD_ERR_MESH; }
  std::vector<int> ordering;
  if (ref_cuthill_mckee(*m, ordering, m->err) != 0) { g_last_mesh_error = m->err; return PCFD_ERR_MESH; }
  apply_c2n_map(*m, ordering);
  if (order_out) std::memcpy(order_out, ordering.data(), sizeof(int) * ordering.size());
  return PCFD_OK;
}

PCFD_API int pcfd_mesh_renumber(pcfd_mesh_t h, const int* order) {
  // order[new] = old; renumbers nodes and element connectivity, then the
  // maps and metrics must be rebuilt with pcfd_mesh_build.
  if (!h || !order) return PCFD_ERR_ARG;
  HostMesh* m = (HostMesh*)h;
  const int nn = m->nnode;
  std::vector<int> old2new(nn, -1);
  for (int i = 0; i < nn; i++) {
    int o = order[i];
    if (o < 0 || o >= nn || old2new[o] >= 0) return PCFD_ERR_ARG;
    old2new[o] = i;
  }
  std::vector<double> x2((size_t)3 * nn);
  for (int i = 0; i < nn; i++)
    for (int c = 0; c < 3; c++) x2[3 * (size_t)i + c] = m->xyz[3 * (size_t)order[i] + c];
  m->xyz.swap(x2);
  for (size_t e = 0; e < m->etype.size(); e++)
    for (int q = 0; q < elem_nnodes(m->etype[e]); q++) m->enodes[4 * e + q] = old2new[m->enodes[4 * e + q]];
  m->maps_built = m->metrics_built = 0;
  return PCFD_OK;
}

PCFD_API void pcfd_mesh_destroy(pcfd_mesh_t h) { delete (HostMesh*)h; }

PCFD_API const char* pcfd_mesh_last_error(void) { return g_last_mesh_error.c_str(); }

}  // extern "C"
