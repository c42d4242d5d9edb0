/*
 * CPU ORACLE - test infrastructure only.  Plain-C restatement of the mesh
 * side of the path, independent of the product library:
 *
 *   - the synthetic workload generator: an nx x ny x nz node box split into
 *     six Kuhn tetrahedra per hex along its (0,0,0)-(1,1,1) diagonal, seeded
 *     jitter of interior nodes (SplitMix64), optional sheared ramp and
 *     geometric clustering toward y = 0; boundary triangles per face with
 *     tags; the same element list and coordinates the product generates;
 *   - the reference's preprocessing of an element list (triangles first,
 *     then tetrahedra):
 *       elements surrounding points ....... ucs/mesh.tcc:397 (BuildElsp)
 *       points surrounding points ......... ucs/mesh.tcc:517 (BuildPsp, its
 *                                           local tables :541-548) with
 *                                           EliminateRepeats (:1341)
 *       boundary winding check ............ ucs/mesh.tcc:2336 (FixBoundaryWindings)
 *       interior edges, half-edges ........ ucs/mesh.tcc:1056 (BuildEdges)
 *       median-dual areas and volumes ..... ucs/mesh.tcc:1653 (CalcAreasVolumes,
 *                                           element tables :1696-1790)
 *       normalisation ..................... ucs/mesh.tcc:2320-2325
 *       weighted LSQ normal matrices ...... ucs/gradient.tcc:461
 *                                           (Kernel_LSQ_CoefficientsWeighted
 *                                           through DriverScatter)
 *
 * tests/test_oracle_mesh.py pins it to the reference's own maps and metrics
 * (tests/golden/ref_*.npz) and to the product's box.  bench.py's reference
 * arm builds its workload with it, so that arm loads nothing of the product.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "oracle.h"

enum { OT_TRI = 0, OT_TET = 2 };

typedef struct {
  uint64_t s;
} splitmix64;

static uint64_t sm_next(splitmix64* r) {
  uint64_t z = (r->s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

/* uniform in [-1, 1) from the top 53 bits */
static double sm_sym(splitmix64* r) {
  return ((double)(sm_next(r) >> 11) * (1.0 / 9007199254740992.0)) * 2.0 - 1.0;
}

/* geometry in the reference's operation order (ucs/geometry.h) */
static void sub3(const double* a, const double* b, double* r) {
  r[0] = a[0] - b[0];
  r[1] = a[1] - b[1];
  r[2] = a[2] - b[2];
}
static void cross3(const double* v1, const double* v2, double* r) {
  r[0] = v1[1] * v2[2] - v2[1] * v1[2];
  r[1] = v1[2] * v2[0] - v2[2] * v1[0];
  r[2] = v1[0] * v2[1] - v2[0] * v1[1];
}
static double mag3(const double* v) { return sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]); }
static double normalize3(const double* v, double* r) {
  double m = mag3(v);
  r[0] = v[0] / m;
  r[1] = v[1] / m;
  r[2] = v[2] / m;
  return m;
}
static void mid2(const double* a, const double* b, double* r) {
  r[0] = (a[0] + b[0]);
  r[1] = (a[1] + b[1]);
  r[2] = (a[2] + b[2]);
  r[0] *= 0.5;
  r[1] *= 0.5;
  r[2] *= 0.5;
}
static void cen3(const double* a, const double* b, const double* c, double* r) {
  double f = 1.0 / 3.0;
  r[0] = (a[0] + b[0] + c[0]);
  r[1] = (a[1] + b[1] + c[1]);
  r[2] = (a[2] + b[2] + c[2]);
  r[0] *= f;
  r[1] *= f;
  r[2] *= f;
}
static void cen4(const double* a, const double* b, const double* c, const double* d, double* r) {
  r[0] = (a[0] + b[0] + c[0] + d[0]);
  r[1] = (a[1] + b[1] + c[1] + d[1]);
  r[2] = (a[2] + b[2] + c[2] + d[2]);
  r[0] *= 0.25;
  r[1] *= 0.25;
  r[2] *= 0.25;
}
static void tri_area(const double* p1, const double* p2, const double* p3, double* r) {
  double v1[3], v2[3];
  sub3(p2, p1, v1);
  sub3(p3, p1, v2);
  cross3(v1, v2, r);
  r[0] = 0.5 * r[0];
  r[1] = 0.5 * r[1];
  r[2] = 0.5 * r[2];
}
static double tet_vol(const double* p1, const double* p2, const double* p3, const double* p4) {
  double v1[3], v2[3], v3[3], t[3];
  sub3(p2, p1, v1);
  sub3(p3, p1, v2);
  sub3(p4, p1, v3);
  cross3(v1, v2, t);
  return (v3[0] * t[0] + v3[1] * t[1] + v3[2] * t[2]) / 6.0;
}

struct oracle_mesh_s {
  int nnode, nelem, ntri;
  double* xyz;   /* [nnode][3] */
  int* etype;    /* [nelem] */
  int* en;       /* [nelem][4] (triangles use 3) */
  int* etag;     /* [nelem] */
  /* maps and metrics */
  int* ipsp;
  int* psp;
  int nedge, nbedge;
  int* edges;    /* [nedge][2] */
  double* ea;    /* [nedge][4] */
  int* bedges;   /* [nbedge][2] */
  int* belem;
  int* bfactag;
  double* ba;    /* [nbedge][4] */
  double* vol;
  double* sw;    /* [nnode][6] */
};

static void* xcalloc(size_t n, size_t sz) { return calloc(n ? n : 1, sz); }

oracle_mesh* oracle_mesh_box(const pcfd_box_params* p) {
  const int nx = p->nx, ny = p->ny, nz = p->nz;
  if (nx < 2 || ny < 2 || nz < 2) return NULL;
  oracle_mesh* m = (oracle_mesh*)xcalloc(1, sizeof(*m));
  m->nnode = nx * ny * nz;
  m->xyz = (double*)xcalloc((size_t)3 * m->nnode, sizeof(double));
  double* cx = (double*)xcalloc(nx, sizeof(double));
  double* cy = (double*)xcalloc(ny, sizeof(double));
  double* cz = (double*)xcalloc(nz, sizeof(double));
  for (int i = 0; i < nx; i++) cx[i] = p->lx * (double)i / (double)(nx - 1);
  for (int k = 0; k < nz; k++) cz[k] = p->lz * (double)k / (double)(nz - 1);
  if (p->y_ratio > 1.0) {
    /* spacings in units of ly: h0 r^k, capped at hc (the first cell floored at
     * the x spacing / wall_ar_max, the cap then fills the height) */
    double h0 = (p->y_ratio - 1.0) / (pow(p->y_ratio, (double)(ny - 1)) - 1.0), y = 0.0;
    double hc = 1e300;
    const double h0_min = p->wall_ar_max > 0.0 ? p->lx / (double)(nx - 1) / p->ly / p->wall_ar_max : 0.0;
    if (h0 < h0_min) {
      h0 = h0_min;
      double lo = h0, hi = 1.0;
      for (int it = 0; it < 200; it++) {
        const double mid = 0.5 * (lo + hi);
        if (mid <= lo || mid >= hi) break;
        double s = 0.0, hk = h0;
        for (int j = 0; j < ny - 1; j++) {
          s += fmin(hk, mid);
          hk *= p->y_ratio;
        }
        if (s < 1.0) lo = mid; else hi = mid;
      }
      hc = hi;
    }
    double h = h0;
    for (int j = 0; j < ny; j++) {
      cy[j] = p->ly * y;
      y += fmin(h, hc);
      h *= p->y_ratio;
    }
    cy[ny - 1] = p->ly;
  } else {
    for (int j = 0; j < ny; j++) cy[j] = p->ly * (double)j / (double)(ny - 1);
  }
  splitmix64 rng = {p->seed};
  const double tanr = tan(p->ramp_deg * 3.14159265358979323846 / 180.0);
#define LH(c, n, i) fmin((i) > 0 ? (c)[i] - (c)[(i)-1] : 1e300, (i) < (n)-1 ? (c)[(i) + 1] - (c)[i] : 1e300)
  for (int k = 0; k < nz; k++)
    for (int j = 0; j < ny; j++)
      for (int i = 0; i < nx; i++) {
        double x = cx[i], y = cy[j], z = cz[k];
        int interior = i > 0 && i < nx - 1 && j > 0 && j < ny - 1 && k > 0 && k < nz - 1;
        if (interior && p->jitter > 0.0) {
          double hx = LH(cx, nx, i), hy = LH(cy, ny, j), hz = LH(cz, nz, k);
          if (p->jitter_mode == 1) hx = hy = hz = fmin(hx, fmin(hy, hz));
          x += p->jitter * hx * sm_sym(&rng);
          y += p->jitter * hy * sm_sym(&rng);
          z += p->jitter * hz * sm_sym(&rng);
        }
        if (p->ramp_deg != 0.0 && x > p->ramp_x0) y = y + tanr * (x - p->ramp_x0) * (p->ly - y) / p->ly;
        size_t n = (size_t)i + (size_t)nx * (j + (size_t)ny * k);
        m->xyz[3 * n] = x;
        m->xyz[3 * n + 1] = y;
        m->xyz[3 * n + 2] = z;
      }
#undef LH
  free(cx);
  free(cy);
  free(cz);
  const int ntri = 4 * ((nx - 1) * (ny - 1) + (ny - 1) * (nz - 1) + (nx - 1) * (nz - 1));
  const int ntet = 6 * (nx - 1) * (ny - 1) * (nz - 1);
  m->ntri = ntri;
  m->nelem = ntri + ntet;
  m->etype = (int*)xcalloc(m->nelem, sizeof(int));
  m->en = (int*)xcalloc((size_t)4 * m->nelem, sizeof(int));
  m->etag = (int*)xcalloc(m->nelem, sizeof(int));
#define ID(i, j, k) ((i) + nx * ((j) + ny * (k)))
  int e = 0;
  for (int f = 0; f < 6; f++) {
    const int axis = f / 2, side = f % 2;
    double out[3] = {0.0, 0.0, 0.0};
    out[axis] = side ? 1.0 : -1.0;
    const int na = axis == 0 ? ny : nx, nb = axis == 2 ? ny : nz;
    for (int b = 0; b < nb - 1; b++)
      for (int a = 0; a < na - 1; a++) {
        int ci, cj, ck;
        if (axis == 0) { ci = side ? nx - 2 : 0; cj = a; ck = b; }
        else if (axis == 1) { ci = a; cj = side ? ny - 2 : 0; ck = b; }
        else { ci = a; cj = b; ck = side ? nz - 2 : 0; }
        int q[4];
        const int s1 = side;
        if (axis == 0) {
          q[0] = ID(ci + s1, cj, ck); q[1] = ID(ci + s1, cj + 1, ck);
          q[2] = ID(ci + s1, cj + 1, ck + 1); q[3] = ID(ci + s1, cj, ck + 1);
        } else if (axis == 1) {
          q[0] = ID(ci, cj + s1, ck); q[1] = ID(ci + 1, cj + s1, ck);
          q[2] = ID(ci + 1, cj + s1, ck + 1); q[3] = ID(ci, cj + s1, ck + 1);
        } else {
          q[0] = ID(ci, cj, ck + s1); q[1] = ID(ci + 1, cj, ck + s1);
          q[2] = ID(ci + 1, cj + 1, ck + s1); q[3] = ID(ci, cj + 1, ck + s1);
        }
        const int tris[2][3] = {{q[0], q[1], q[2]}, {q[0], q[2], q[3]}};
        for (int t = 0; t < 2; t++) {
          int v0 = tris[t][0], v1 = tris[t][1], v2 = tris[t][2];
          double nrm[3];
          tri_area(&m->xyz[3 * (size_t)v0], &m->xyz[3 * (size_t)v1], &m->xyz[3 * (size_t)v2], nrm);
          if (nrm[0] * out[0] + nrm[1] * out[1] + nrm[2] * out[2] < 0.0) {
            int tmp = v0;
            v0 = v2;
            v2 = tmp;
          }
          m->etype[e] = OT_TRI;
          m->en[4 * e] = v0;
          m->en[4 * e + 1] = v1;
          m->en[4 * e + 2] = v2;
          m->en[4 * e + 3] = -1;
          m->etag[e] = (f == 2 && ci < p->wall_start_i) ? p->upstream_tag : p->tags[f];
          e++;
        }
      }
  }
  static const int perms[6][3] = {{0, 1, 2}, {0, 2, 1}, {1, 0, 2}, {1, 2, 0}, {2, 0, 1}, {2, 1, 0}};
  static const int parity[6] = {0, 1, 1, 0, 0, 1};
  for (int k = 0; k < nz - 1; k++)
    for (int j = 0; j < ny - 1; j++)
      for (int i = 0; i < nx - 1; i++)
        for (int t = 0; t < 6; t++) {
          int off[3] = {0, 0, 0}, v[4];
          v[0] = ID(i, j, k);
          off[perms[t][0]] = 1;
          v[1] = ID(i + off[0], j + off[1], k + off[2]);
          off[perms[t][1]] = 1;
          v[2] = ID(i + off[0], j + off[1], k + off[2]);
          v[3] = ID(i + 1, j + 1, k + 1);
          if (parity[t]) {
            int tmp = v[1];
            v[1] = v[2];
            v[2] = tmp;
          }
          m->etype[e] = OT_TET;
          for (int q = 0; q < 4; q++) m->en[4 * e + q] = v[q];
          m->etag[e] = 0;
          e++;
        }
#undef ID
  return m;
}

oracle_mesh* oracle_mesh_elements(int nnode, const double* xyz, int ntri, const int* tri, const int* tri_tag, int ntet,
                                  const int* tet) {
  oracle_mesh* m = (oracle_mesh*)xcalloc(1, sizeof(*m));
  m->nnode = nnode;
  m->ntri = ntri;
  m->nelem = ntri + ntet;
  m->xyz = (double*)xcalloc((size_t)3 * nnode, sizeof(double));
  memcpy(m->xyz, xyz, sizeof(double) * 3 * (size_t)nnode);
  m->etype = (int*)xcalloc(m->nelem, sizeof(int));
  m->en = (int*)xcalloc((size_t)4 * m->nelem, sizeof(int));
  m->etag = (int*)xcalloc(m->nelem, sizeof(int));
  for (int e = 0; e < ntri; e++) {
    m->etype[e] = OT_TRI;
    for (int q = 0; q < 3; q++) m->en[4 * e + q] = tri[3 * e + q];
    m->en[4 * e + 3] = -1;
    m->etag[e] = tri_tag[e];
  }
  for (int e = 0; e < ntet; e++) {
    m->etype[ntri + e] = OT_TET;
    for (int q = 0; q < 4; q++) m->en[4 * (ntri + e) + q] = tet[4 * e + q];
  }
  return m;
}

static int nn_of(int t) { return t == OT_TRI ? 3 : 4; }

/* BuildMaps + CalcMetrics + the LSQ normal matrices; 0 on success */
int oracle_mesh_build(oracle_mesh* m) {
  static const int clTri[6] = {1, 2, 2, 0, 0, 1};
  static const int clTet[12] = {1, 2, 3, 2, 0, 3, 0, 1, 3, 0, 1, 2};
  static const int eorder[12] = {0, 1, 0, 2, 0, 3, 1, 2, 1, 3, 2, 3};
  static const int e2f[12] = {0, 1, 2, 0, 1, 2, 0, 3, 3, 1, 2, 3};
  static const int fl[12] = {0, 1, 2, 0, 3, 1, 0, 2, 3, 1, 3, 2};
  const int nn = m->nnode, ne = m->nelem;
  const double* X = m->xyz;
  /* BuildElsp: counts, prefix sums, fill in element order */
  int* ielsp = (int*)xcalloc((size_t)nn + 1, sizeof(int));
  for (int e = 0; e < ne; e++)
    for (int j = 0; j < nn_of(m->etype[e]); j++) {
      int v = m->en[4 * e + j];
      if (v < 0 || v >= nn) { free(ielsp); return -1; }
      ielsp[v + 1]++;
    }
  for (int i = 1; i <= nn; i++) ielsp[i] += ielsp[i - 1];
  int* elsp = (int*)xcalloc((size_t)ielsp[nn], sizeof(int));
  int* fill = (int*)xcalloc((size_t)nn, sizeof(int));
  memcpy(fill, ielsp, sizeof(int) * (size_t)nn);
  for (int e = 0; e < ne; e++)
    for (int j = 0; j < nn_of(m->etype[e]); j++) elsp[fill[m->en[4 * e + j]]++] = e;
  /* BuildPsp: per node, the element-local neighbours in elsp order, first occurrences kept */
  size_t cap = (size_t)nn * 16 + 16, used = 0;
  m->psp = (int*)malloc(cap * sizeof(int));
  m->ipsp = (int*)xcalloc((size_t)nn + 1, sizeof(int));
  int* stamp = fill; /* reuse: last node that saw each value */
  for (int i = 0; i < nn; i++) stamp[i] = -1;
  for (int i = 0; i < nn; i++) {
    for (int k = ielsp[i]; k < ielsp[i + 1]; k++) {
      const int e = elsp[k];
      const int* nodes = &m->en[4 * e];
      int l = 0;
      while (nodes[l] != i) l++;
      const int cnt = m->etype[e] == OT_TRI ? 2 : 3;
      const int* cl = m->etype[e] == OT_TRI ? &clTri[2 * l] : &clTet[3 * l];
      for (int q = 0; q < cnt; q++) {
        int v = nodes[cl[q]];
        if (stamp[v] == i) continue;
        stamp[v] = i;
        if (used == cap) {
          cap *= 2;
          m->psp = (int*)realloc(m->psp, cap * sizeof(int));
        }
        m->psp[used++] = v;
      }
    }
    m->ipsp[i + 1] = (int)used;
  }
  /* FixBoundaryWindings: a boundary triangle faces away from its tetrahedron */
  for (int e = 0; e < ne; e++) {
    if (m->etype[e] != OT_TRI) continue;
    int* tn = &m->en[4 * e];
    int owner = -1;
    for (int k = ielsp[tn[0]]; k < ielsp[tn[0] + 1] && owner < 0; k++) {
      int t = elsp[k], hits = 0;
      if (m->etype[t] != OT_TET) continue;
      for (int a = 0; a < 3; a++)
        for (int b = 0; b < 4; b++) hits += tn[a] == m->en[4 * t + b];
      if (hits == 3) owner = t;
    }
    if (owner < 0) return -2;
    const int* q = &m->en[4 * owner];
    double bpt[3], ept[3], d[3], nb[3];
    cen3(&X[3 * tn[0]], &X[3 * tn[1]], &X[3 * tn[2]], bpt);
    cen4(&X[3 * q[0]], &X[3 * q[1]], &X[3 * q[2]], &X[3 * q[3]], ept);
    sub3(bpt, ept, d);
    tri_area(&X[3 * tn[0]], &X[3 * tn[1]], &X[3 * tn[2]], nb);
    normalize3(d, d);
    normalize3(nb, nb);
    if (!(d[0] * nb[0] + d[1] * nb[1] + d[2] * nb[2] > 0.0)) {
      int tmp = tn[0];
      tn[0] = tn[2];
      tn[2] = tmp;
    }
  }
  /* BuildEdges: i < psp in node-then-psp order; one half-edge per (triangle, node) */
  m->nedge = 0;
  for (int i = 0; i < nn; i++)
    for (int j = m->ipsp[i]; j < m->ipsp[i + 1]; j++) m->nedge += m->psp[j] > i;
  m->edges = (int*)xcalloc((size_t)2 * m->nedge, sizeof(int));
  {
    int c = 0;
    for (int i = 0; i < nn; i++)
      for (int j = m->ipsp[i]; j < m->ipsp[i + 1]; j++)
        if (m->psp[j] > i) {
          m->edges[2 * c] = i;
          m->edges[2 * c + 1] = m->psp[j];
          c++;
        }
  }
  m->nbedge = 3 * m->ntri;
  m->bedges = (int*)xcalloc((size_t)2 * m->nbedge, sizeof(int));
  m->belem = (int*)xcalloc((size_t)m->nbedge, sizeof(int));
  m->bfactag = (int*)xcalloc((size_t)m->nbedge, sizeof(int));
  {
    int c = 0;
    for (int e = 0; e < ne; e++) {
      if (m->etype[e] != OT_TRI) continue;
      for (int j = 0; j < 3; j++) {
        m->bedges[2 * c] = m->en[4 * e + j];
        m->bedges[2 * c + 1] = nn + c;
        m->belem[c] = e;
        m->bfactag[c] = m->etag[e];
        c++;
      }
    }
  }
  /* CalcAreasVolumes: per interior edge, the elements around its second node */
  m->ea = (double*)xcalloc((size_t)4 * m->nedge, sizeof(double));
  m->ba = (double*)xcalloc((size_t)4 * m->nbedge, sizeof(double));
  m->vol = (double*)xcalloc((size_t)nn, sizeof(double));
  for (int i = 0; i < m->nedge; i++) {
    const int n1 = m->edges[2 * i], n2 = m->edges[2 * i + 1];
    for (int k = ielsp[n2]; k < ielsp[n2 + 1]; k++) {
      const int e = elsp[k];
      if (m->etype[e] != OT_TET) continue;
      const int* nodes = &m->en[4 * e];
      int l1 = -1, l2 = -1;
      for (int q = 0; q < 4; q++) {
        if (nodes[q] == n1) l1 = q;
        else if (nodes[q] == n2) l2 = q;
      }
      if (l1 < 0 || l2 < 0) continue;
      int eid = -1, orient = 0;
      for (int j = 0; j < 6 && eid < 0; j++) {
        if (eorder[2 * j] == l1 && eorder[2 * j + 1] == l2) { eid = j; orient = 1; }
        else if (eorder[2 * j + 1] == l1 && eorder[2 * j] == l2) { eid = j; orient = -1; }
      }
      const int f1 = e2f[2 * eid], f2 = e2f[2 * eid + 1];
      double edgept[3], c1[3], c2[3], ept[3], ar[3];
      mid2(&X[3 * n1], &X[3 * n2], edgept);
      cen3(&X[3 * nodes[fl[3 * f1]]], &X[3 * nodes[fl[3 * f1 + 1]]], &X[3 * nodes[fl[3 * f1 + 2]]], c1);
      cen3(&X[3 * nodes[fl[3 * f2]]], &X[3 * nodes[fl[3 * f2 + 1]]], &X[3 * nodes[fl[3 * f2 + 2]]], c2);
      cen4(&X[3 * nodes[0]], &X[3 * nodes[1]], &X[3 * nodes[2]], &X[3 * nodes[3]], ept);
      const double o = (double)orient;
      double* a = &m->ea[4 * i];
      tri_area(ept, c2, edgept, ar);
      ar[0] = o * ar[0]; ar[1] = o * ar[1]; ar[2] = o * ar[2];
      a[0] = a[0] + ar[0]; a[1] = a[1] + ar[1]; a[2] = a[2] + ar[2];
      tri_area(edgept, c1, ept, ar);
      ar[0] = o * ar[0]; ar[1] = o * ar[1]; ar[2] = o * ar[2];
      a[0] = a[0] + ar[0]; a[1] = a[1] + ar[1]; a[2] = a[2] + ar[2];
      const double t0 = o * tet_vol(&X[3 * n1], ept, c2, edgept);
      const double t1 = o * tet_vol(&X[3 * n1], c1, ept, edgept);
      const double t2 = o * tet_vol(&X[3 * n2], ept, c1, edgept);
      const double t3 = o * tet_vol(&X[3 * n2], c2, ept, edgept);
      m->vol[n1] += t0;
      m->vol[n1] += t1;
      m->vol[n2] += t2;
      m->vol[n2] += t3;
    }
  }
  for (int i = 0; i < m->nbedge; i++) {
    const int n1 = m->bedges[2 * i];
    const int* nodes = &m->en[4 * m->belem[i]];
    int nid = 0;
    for (int q = 0; q < 3; q++)
      if (nodes[q] == n1) nid = q;
    double ept[3], edgept[3], ar[3];
    cen3(&X[3 * nodes[0]], &X[3 * nodes[1]], &X[3 * nodes[2]], ept);
    double* a = &m->ba[4 * i];
    mid2(&X[3 * n1], &X[3 * nodes[clTri[2 * nid]]], edgept);
    tri_area(ept, &X[3 * n1], edgept, ar);
    a[0] = a[0] + ar[0]; a[1] = a[1] + ar[1]; a[2] = a[2] + ar[2];
    mid2(&X[3 * n1], &X[3 * nodes[clTri[2 * nid + 1]]], edgept);
    tri_area(edgept, &X[3 * n1], ept, ar);
    a[0] = a[0] + ar[0]; a[1] = a[1] + ar[1]; a[2] = a[2] + ar[2];
  }
  for (int i = 0; i < m->nedge; i++) m->ea[4 * i + 3] = normalize3(&m->ea[4 * i], &m->ea[4 * i]);
  for (int i = 0; i < m->nbedge; i++) m->ba[4 * i + 3] = normalize3(&m->ba[4 * i], &m->ba[4 * i]);
  /* LSQ normal matrices: right node first, then left, per edge (DriverScatter) */
  m->sw = (double*)xcalloc((size_t)6 * nn, sizeof(double));
  for (int i = 0; i < m->nedge; i++) {
    const int l = m->edges[2 * i], r = m->edges[2 * i + 1];
    double dx[3], tl[6], tr[6];
    sub3(&X[3 * l], &X[3 * r], dx);
    const double ds2 = 1.0 / (dx[0] * dx[0] + dx[1] * dx[1] + dx[2] * dx[2]);
    tl[0] = dx[0] * dx[0] * ds2;
    tl[1] = dx[0] * dx[1] * ds2;
    tl[2] = dx[0] * dx[2] * ds2;
    tl[3] = dx[1] * dx[1] * ds2;
    tl[4] = dx[1] * dx[2] * ds2;
    tl[5] = dx[2] * dx[2] * ds2;
    dx[0] = -dx[0];
    dx[1] = -dx[1];
    dx[2] = -dx[2];
    tr[0] = tl[0];
    tr[1] = (dx[0] * dx[1]) * ds2;
    tr[2] = (dx[0] * dx[2]) * ds2;
    tr[3] = tl[3];
    tr[4] = (dx[1] * dx[2]) * ds2;
    tr[5] = tl[5];
    for (int c = 0; c < 6; c++) m->sw[6 * r + c] += tr[c];
    for (int c = 0; c < 6; c++) m->sw[6 * l + c] += tl[c];
  }
  free(ielsp);
  free(elsp);
  free(fill);
  return 0;
}

int oracle_mesh_view(const oracle_mesh* m, pcfd_mesh_view* v) {
  if (!m->ipsp) return -1;
  memset(v, 0, sizeof(*v));
  v->nnode = m->nnode;
  v->nbnode = m->nbedge;
  v->nedge = m->nedge;
  v->nbedge = m->nbedge;
  v->edges = m->edges;
  v->edge_area = m->ea;
  v->bedges = m->bedges;
  v->bedge_area = m->ba;
  v->bfactag = m->bfactag;
  v->xyz = m->xyz;
  v->vol = m->vol;
  v->sw = m->sw;
  v->ipsp = m->ipsp;
  v->psp = m->psp;
  return 0;
}

void oracle_mesh_free(oracle_mesh* m) {
  if (!m) return;
  free(m->xyz); free(m->etype); free(m->en); free(m->etag); free(m->ipsp); free(m->psp);
  free(m->edges); free(m->ea); free(m->bedges); free(m->belem); free(m->bfactag); free(m->ba);
  free(m->vol); free(m->sw);
  free(m);
}
