/*
 * CPU ORACLE - test infrastructure only.  Plain-C restatement of the learned
 * right preconditioner's network (declared in include/pcfd.h, pcfd_lp_*),
 * used by the tests to check the CUDA forward and backward kernels.  The
 * network has no reference counterpart; it plugs in where
 * CRS<T>::PrecondBackSolve sits (ucs/crs.tcc:591).
 *
 * All arithmetic is double.  With emulate = 1 the values the GPU keeps in
 * BF16 are rounded to BF16 at the same points (matrices, stored activations
 * h and m, the backward operand dz) and the node features are rounded to
 * FP32; with emulate = 0 nothing is rounded, which is what the
 * finite-difference check of the backward pass uses.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "oracle.h"

enum {
  NIN = PCFD_LP_NIN,
  H = PCFD_LP_HIDDEN,
  NE = PCFD_LP_NEDGE,
  NOUT = PCFD_LP_NOUT,
  NL = PCFD_LP_LAYERS,
  OFF_WIN = 0,
  OFF_BIN = H * NIN,
  OFF_L0 = OFF_BIN + H,
  L_WE = 0,
  L_CE = H * NE,
  L_WS = L_CE + H,
  L_WM = L_WS + H * H,
  L_B = L_WM + H * H,
  L_SIZE = L_B + H,
  OFF_WOUT = OFF_L0 + NL * L_SIZE,
  OFF_BOUT = OFF_WOUT + NOUT * H,
  NPARAM = OFF_BOUT + NOUT
};

double oracle_bf16(double v) {
  float f = (float)v;
  uint32_t u;
  memcpy(&u, &f, 4);
  if ((u & 0x7f800000u) == 0x7f800000u) {
    if (u & 0x7fffffu) u |= 0x400000u;
    u &= 0xffff0000u;
  } else {
    u += 0x7fffu + ((u >> 16) & 1u);
    u &= 0xffff0000u;
  }
  memcpy(&f, &u, 4);
  return (double)f;
}

int oracle_lp_nparam(void) { return NPARAM; }

/* node -> neighbour CSR in ascending edge id, with the edge features seen
 * from the node: unit normal times +1 (node is the edge's first node) or -1,
 * and the edge length over the mean edge length */
void oracle_lp_graph(const pcfd_mesh_view* m, int* nptr, int* nbr, float* ef) {
  const int nn = (int)m->nnode, ne = (int)m->nedge;
  memset(nptr, 0, sizeof(int) * (nn + 1));
  for (int e = 0; e < ne; e++) {
    nptr[m->edges[2 * e] + 1]++;
    nptr[m->edges[2 * e + 1] + 1]++;
  }
  for (int i = 0; i < nn; i++) nptr[i + 1] += nptr[i];
  double lsum = 0.0;
  for (int e = 0; e < ne; e++) {
    const double* a = &m->xyz[3 * m->edges[2 * e]];
    const double* b = &m->xyz[3 * m->edges[2 * e + 1]];
    double dx = b[0] - a[0], dy = b[1] - a[1], dz = b[2] - a[2];
    lsum += sqrt(dx * dx + dy * dy + dz * dz);
  }
  const double lmean = ne > 0 ? lsum / ne : 1.0;
  int* fill = (int*)malloc(sizeof(int) * (nn + 1));
  memcpy(fill, nptr, sizeof(int) * (nn + 1));
  for (int e = 0; e < ne; e++) {
    const int L = m->edges[2 * e], R = m->edges[2 * e + 1];
    const double* a = &m->xyz[3 * L];
    const double* b = &m->xyz[3 * R];
    double dx = b[0] - a[0], dy = b[1] - a[1], dz = b[2] - a[2];
    float lh = (float)(sqrt(dx * dx + dy * dy + dz * dz) / lmean);
    const double* n = &m->edge_area[4 * e];
    int p = fill[L]++;
    nbr[p] = R;
    ef[4 * p + 0] = (float)n[0];
    ef[4 * p + 1] = (float)n[1];
    ef[4 * p + 2] = (float)n[2];
    ef[4 * p + 3] = lh;
    p = fill[R]++;
    nbr[p] = L;
    ef[4 * p + 0] = -(float)n[0];
    ef[4 * p + 1] = -(float)n[1];
    ef[4 * p + 2] = -(float)n[2];
    ef[4 * p + 3] = lh;
  }
  free(fill);
}

/* node features of y (see pcfd_lp_features); returns sigma */
double oracle_lp_features(int nnode, const double* y, const double* q, const double* vol, const double* qinf,
                          double gamma, float* x) {
  double ss = 0.0, vs = 0.0;
  for (long long i = 0; i < (long long)nnode * 5; i++) ss += y[i] * y[i];
  for (int i = 0; i < nnode; i++) vs += vol[i];
  double sigma = sqrt(ss / (5.0 * nnode));
  double isig = sigma > 0.0 ? 1.0 / sigma : 0.0;
  double vmean = vs / nnode;
  double cinf = sqrt(gamma * qinf[6] / qinf[0]);
  for (int i = 0; i < nnode; i++) {
    const double* Q = &q[(size_t)i * 10];
    float* xi = &x[(size_t)i * NIN];
    for (int k = 0; k < 5; k++) xi[k] = (float)(y[(size_t)i * 5 + k] * isig);
    xi[5] = (float)(Q[0] / qinf[0] - 1.0);
    xi[6] = (float)(Q[7] / cinf);
    xi[7] = (float)(Q[8] / cinf);
    xi[8] = (float)(Q[9] / cinf);
    xi[9] = (float)(Q[6] / qinf[6] - 1.0);
    xi[10] = (float)log(vol[i] / vmean);
  }
  return sigma;
}

static double rnd(int emulate, double v) { return emulate ? oracle_bf16(v) : v; }

/* matrices in the precision the network uses them */
static void prep_weights(const float* w, int emulate, double* wd) {
  for (int i = 0; i < NPARAM; i++) wd[i] = w[i];
  if (!emulate) return;
  for (int i = 0; i < H * NIN; i++) wd[OFF_WIN + i] = oracle_bf16(w[OFF_WIN + i]);
  for (int l = 0; l < NL; l++) {
    int o = OFF_L0 + l * L_SIZE;
    for (int i = 0; i < H * NE; i++) wd[o + L_WE + i] = oracle_bf16(w[o + L_WE + i]);
    for (int i = 0; i < H * H; i++) wd[o + L_WS + i] = oracle_bf16(w[o + L_WS + i]);
    for (int i = 0; i < H * H; i++) wd[o + L_WM + i] = oracle_bf16(w[o + L_WM + i]);
  }
  for (int i = 0; i < NOUT * H; i++) wd[OFF_WOUT + i] = oracle_bf16(w[OFF_WOUT + i]);
}

static double gate(const double* wl, const float* e, int c, double sgn) {
  const double* We = wl + L_WE;
  return wl[L_CE + c] + We[c * NE + 0] * (sgn * e[0]) + We[c * NE + 1] * (sgn * e[1]) +
         We[c * NE + 2] * (sgn * e[2]) + We[c * NE + 3] * e[3];
}

/* forward pass; hs: (NL+1) * n * H, ms: NL * n * H (stored activations) */
static void forward(int n, const int* nptr, const int* nbr, const float* ef, const float* x, const double* wd,
                    int emulate, double* hs, double* ms, double* out) {
  for (int i = 0; i < n; i++)
    for (int c = 0; c < H; c++) {
      double a = wd[OFF_BIN + c];
      for (int k = 0; k < NIN; k++) a += wd[OFF_WIN + c * NIN + k] * (double)x[(size_t)i * NIN + k];
      hs[(size_t)i * H + c] = rnd(emulate, a > 0.0 ? a : 0.0);
    }
  for (int l = 0; l < NL; l++) {
    const double* wl = wd + OFF_L0 + l * L_SIZE;
    const double* h = hs + (size_t)l * n * H;
    double* hn = hs + (size_t)(l + 1) * n * H;
    double* m = ms + (size_t)l * n * H;
    for (int i = 0; i < n; i++) {
      int deg = nptr[i + 1] - nptr[i];
      double idg = deg > 0 ? 1.0 / deg : 0.0;
      for (int c = 0; c < H; c++) {
        double a = 0.0;
        for (int p = nptr[i]; p < nptr[i + 1]; p++) a += gate(wl, &ef[4 * p], c, 1.0) * h[(size_t)nbr[p] * H + c];
        m[(size_t)i * H + c] = rnd(emulate, a * idg);
      }
    }
    for (int i = 0; i < n; i++)
      for (int c = 0; c < H; c++) {
        double a = 0.0;
        for (int k = 0; k < H; k++) a += wl[L_WS + c * H + k] * h[(size_t)i * H + k];
        for (int k = 0; k < H; k++) a += wl[L_WM + c * H + k] * m[(size_t)i * H + k];
        a += wl[L_B + c];
        hn[(size_t)i * H + c] = rnd(emulate, a > 0.0 ? a : 0.0);
      }
  }
  const double* h3 = hs + (size_t)NL * n * H;
  for (int i = 0; i < n; i++)
    for (int o = 0; o < NOUT; o++) {
      double a = wd[OFF_BOUT + o];
      for (int k = 0; k < H; k++) a += wd[OFF_WOUT + o * H + k] * h3[(size_t)i * H + k];
      out[(size_t)i * NOUT + o] = a;
    }
}

void oracle_lp_forward(int n, const int* nptr, const int* nbr, const float* ef, const float* x, const float* w,
                       int emulate, double* out) {
  double* wd = (double*)malloc(sizeof(double) * NPARAM);
  double* hs = (double*)malloc(sizeof(double) * (size_t)(NL + 1) * n * H);
  double* ms = (double*)malloc(sizeof(double) * (size_t)NL * n * H);
  prep_weights(w, emulate, wd);
  forward(n, nptr, nbr, ef, x, wd, emulate, hs, ms, out);
  free(wd);
  free(hs);
  free(ms);
}

/* loss = sum (out - t)^2 / (5 n) and d loss / d params (straight-through
 * for the BF16 rounding of the matrices) */
double oracle_lp_loss_grad(int n, const int* nptr, const int* nbr, const float* ef, const float* x, const float* t,
                           const float* w, int emulate, double* grad) {
  double* wd = (double*)malloc(sizeof(double) * NPARAM);
  double* hs = (double*)malloc(sizeof(double) * (size_t)(NL + 1) * n * H);
  double* ms = (double*)malloc(sizeof(double) * (size_t)NL * n * H);
  double* out = (double*)malloc(sizeof(double) * (size_t)n * NOUT);
  double* dh = (double*)malloc(sizeof(double) * (size_t)n * H);
  double* dz = (double*)malloc(sizeof(double) * (size_t)n * H);
  double* dm = (double*)malloc(sizeof(double) * (size_t)n * H);
  double* dhn = (double*)malloc(sizeof(double) * (size_t)n * H);
  prep_weights(w, emulate, wd);
  forward(n, nptr, nbr, ef, x, wd, emulate, hs, ms, out);
  memset(grad, 0, sizeof(double) * NPARAM);
  const double scale = 2.0 / (5.0 * n);
  double loss = 0.0;
  const double* h3 = hs + (size_t)NL * n * H;
  for (int i = 0; i < n; i++) {
    double dout[NOUT];
    for (int o = 0; o < NOUT; o++) {
      double r = out[(size_t)i * NOUT + o] - (double)t[(size_t)i * NOUT + o];
      loss += r * r;
      dout[o] = scale * r;
      grad[OFF_BOUT + o] += dout[o];
      for (int k = 0; k < H; k++) grad[OFF_WOUT + o * H + k] += dout[o] * h3[(size_t)i * H + k];
    }
    for (int k = 0; k < H; k++) {
      double a = 0.0;
      for (int o = 0; o < NOUT; o++) a += wd[OFF_WOUT + o * H + k] * dout[o];
      dh[(size_t)i * H + k] = a;
    }
  }
  loss /= 5.0 * n;
  for (int l = NL - 1; l >= 0; l--) {
    const double* wl = wd + OFF_L0 + l * L_SIZE;
    double* gl = grad + OFF_L0 + l * L_SIZE;
    const double* h = hs + (size_t)l * n * H;
    const double* hn = hs + (size_t)(l + 1) * n * H;
    const double* m = ms + (size_t)l * n * H;
    for (size_t i = 0; i < (size_t)n * H; i++) dz[i] = rnd(emulate, hn[i] > 0.0 ? dh[i] : 0.0);
    for (int i = 0; i < n; i++)
      for (int c = 0; c < H; c++) {
        double d = dz[(size_t)i * H + c];
        gl[L_B + c] += d;
        for (int k = 0; k < H; k++) {
          gl[L_WS + c * H + k] += d * h[(size_t)i * H + k];
          gl[L_WM + c * H + k] += d * m[(size_t)i * H + k];
        }
      }
    for (int i = 0; i < n; i++)
      for (int k = 0; k < H; k++) {
        double a = 0.0, b = 0.0;
        for (int c = 0; c < H; c++) {
          a += wl[L_WS + c * H + k] * dz[(size_t)i * H + c];
          b += wl[L_WM + c * H + k] * dz[(size_t)i * H + c];
        }
        dhn[(size_t)i * H + k] = a;
        dm[(size_t)i * H + k] = b;
      }
    /* m_i = idg_i sum_j g_ij h_j: gather the transpose over the symmetric graph */
    for (int j = 0; j < n; j++)
      for (int p = nptr[j]; p < nptr[j + 1]; p++) {
        int i = nbr[p];
        int degi = nptr[i + 1] - nptr[i];
        double idg = degi > 0 ? 1.0 / degi : 0.0;
        const float* e = &ef[4 * p]; /* oriented j -> i; seen from i it is flipped */
        for (int c = 0; c < H; c++) {
          double g = gate(wl, e, c, -1.0);
          double dmi = dm[(size_t)i * H + c] * idg;
          dhn[(size_t)j * H + c] += g * dmi;
          double dg = dmi * h[(size_t)j * H + c];
          gl[L_CE + c] += dg;
          gl[L_WE + c * NE + 0] -= dg * e[0];
          gl[L_WE + c * NE + 1] -= dg * e[1];
          gl[L_WE + c * NE + 2] -= dg * e[2];
          gl[L_WE + c * NE + 3] += dg * e[3];
        }
      }
    memcpy(dh, dhn, sizeof(double) * (size_t)n * H);
  }
  for (int i = 0; i < n; i++)
    for (int c = 0; c < H; c++) {
      double d = hs[(size_t)i * H + c] > 0.0 ? dh[(size_t)i * H + c] : 0.0;
      grad[OFF_BIN + c] += d;
      for (int k = 0; k < NIN; k++) grad[OFF_WIN + c * NIN + k] += d * (double)x[(size_t)i * NIN + k];
    }
  free(wd);
  free(hs);
  free(ms);
  free(out);
  free(dh);
  free(dz);
  free(dm);
  free(dhn);
  return loss;
}
