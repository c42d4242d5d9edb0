// Reference pin - test infrastructure only.
//
// Compiles the reference's own self-contained headers ucs/matrix.h (block LU,
// LuSolve, MatVecMult) and ucs/geometry.h (dual-metric primitives) from the
// reference source tree, unmodified, and exposes them through a C ABI so the
// tests can check the oracle's restatements bit for bit.  Built into
// oracle/_ref/ only where the reference tree is present; never shipped.
#include "matrix.h"
#include "geometry.h"

extern "C" {

int ref_lu(double* a, int* p, int n) { return LU(a, p, n); }

void ref_lusolve(double* a, double* b, int* p, double* x, int n) { LuSolve(a, b, p, x, n); }

void ref_matvec(const double* a, const double* x, double* y, int n) { MatVecMult(a, x, y, n); }

void ref_tri_area(const double* p1, const double* p2, const double* p3, double* r) { CalcTriArea(p1, p2, p3, r); }

double ref_tet_vol(const double* p1, const double* p2, const double* p3, const double* p4) {
  return CalcTetVol(p1, p2, p3, p4);
}

void ref_centroid3(const double* p1, const double* p2, const double* p3, double* r) { Centroid(p1, p2, p3, r); }

void ref_centroid4(const double* p1, const double* p2, const double* p3, const double* p4, double* r) {
  Centroid(p1, p2, p3, p4, r);
}

}  // extern "C"
