// FP64 CPU oracle: small vector/matrix helpers.
//
// TEST INFRASTRUCTURE ONLY.  Nothing in the shipped library includes, links or
// calls anything under oracle/; only tests/, the smoke check and the CPU-baseline
// leg of bench.py do.
//
// The reference (FCL 0.7.0) does all linear algebra through Eigen 3.  Eigen is not
// vendored by the reference and is not available here, so the evaluation order of
// its fixed-size reductions cannot be checked.  This oracle fixes one order and the
// GPU FP64 paths follow the same order:
//   dot(a,b)         = (a0*b0 + a1*b1) + a2*b2
//   (A*B)(i,j)       = (A(i,0)*B(0,j) + A(i,1)*B(1,j)) + A(i,2)*B(2,j)
//   squaredNorm(a)   = (a0*a0 + a1*a1) + a2*a2
//   cross(a,b)       = (a1*b2 - a2*b1, a2*b0 - a0*b2, a0*b1 - a1*b0)
// Elementwise expressions are evaluated left to right, one rounding per operation.
// The file must be compiled with -ffp-contract=off (no fused multiply-add), as the
// reference is built with -msse2 -mfpmath=sse and no -march (CMakeLists.txt:84).
#pragma once
#include <cmath>
#include <cstdint>

namespace oracle {

struct V3 {
  double v[3];
  double& operator[](int i) { return v[i]; }
  double operator[](int i) const { return v[i]; }
};

// Row-major 3x3: m[r][c].
struct M3 {
  double m[3][3];
  double& operator()(int r, int c) { return m[r][c]; }
  double operator()(int r, int c) const { return m[r][c]; }
};

inline V3 mk(double a, double b, double c) { V3 r; r[0] = a; r[1] = b; r[2] = c; return r; }
inline V3 add(const V3& a, const V3& b) { return mk(a[0] + b[0], a[1] + b[1], a[2] + b[2]); }
inline V3 sub(const V3& a, const V3& b) { return mk(a[0] - b[0], a[1] - b[1], a[2] - b[2]); }
inline V3 scale(const V3& a, double s) { return mk(a[0] * s, a[1] * s, a[2] * s); }
inline V3 neg(const V3& a) { return mk(-a[0], -a[1], -a[2]); }
inline double dot(const V3& a, const V3& b) { return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2]; }
inline double sqnorm(const V3& a) { return (a[0] * a[0] + a[1] * a[1]) + a[2] * a[2]; }
inline double norm(const V3& a) { return std::sqrt(sqnorm(a)); }
inline V3 cross(const V3& a, const V3& b) {
  return mk(a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]);
}
inline V3 col(const M3& A, int c) { return mk(A(0, c), A(1, c), A(2, c)); }
inline V3 row(const M3& A, int r) { return mk(A(r, 0), A(r, 1), A(r, 2)); }
inline void setcol(M3& A, int c, const V3& v) { A(0, c) = v[0]; A(1, c) = v[1]; A(2, c) = v[2]; }
// A*v
inline V3 mulv(const M3& A, const V3& v) {
  return mk((A(0, 0) * v[0] + A(0, 1) * v[1]) + A(0, 2) * v[2],
            (A(1, 0) * v[0] + A(1, 1) * v[1]) + A(1, 2) * v[2],
            (A(2, 0) * v[0] + A(2, 1) * v[1]) + A(2, 2) * v[2]);
}
// A^T*v  (== v^T*A as a row vector)
inline V3 mulTv(const M3& A, const V3& v) {
  return mk((A(0, 0) * v[0] + A(1, 0) * v[1]) + A(2, 0) * v[2],
            (A(0, 1) * v[0] + A(1, 1) * v[1]) + A(2, 1) * v[2],
            (A(0, 2) * v[0] + A(1, 2) * v[1]) + A(2, 2) * v[2]);
}
// A*B
inline M3 mul(const M3& A, const M3& B) {
  M3 C;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j)
      C(i, j) = (A(i, 0) * B(0, j) + A(i, 1) * B(1, j)) + A(i, 2) * B(2, j);
  return C;
}
// A^T*B
inline M3 mulT(const M3& A, const M3& B) {
  M3 C;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j)
      C(i, j) = (A(0, i) * B(0, j) + A(1, i) * B(1, j)) + A(2, i) * B(2, j);
  return C;
}
inline M3 ident() {
  M3 I;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) I(i, j) = (i == j) ? 1.0 : 0.0;
  return I;
}
inline M3 transpose(const M3& A) {
  M3 T;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) T(i, j) = A(j, i);
  return T;
}

// Rigid transform: x -> R*x + t  (fcl::Transform3<double> restricted to isometries).
struct Tf {
  M3 R;
  V3 t;
};
inline V3 apply(const Tf& f, const V3& p) { return add(mulv(f.R, p), f.t); }

}  // namespace oracle
