// Device geometry for the OBBRSS mesh path, templated on the scalar type.
//
// The double instantiation is the exact form: it follows FCL 0.7.0 operation by
// operation (3-term sums left to right, no fused multiply-add -- the translation
// units including this header are compiled with -fmad=false and FP32 code that wants
// fusion calls fmaf explicitly), so its decisions equal the FP64 reference's.
#pragma once
#include <cuda_runtime.h>
#include <math.h>
#include <string.h>

#include "fclgpu_types.h"

#ifndef FCLG_HD
#define FCLG_HD __host__ __device__ __forceinline__
#endif

namespace fclgpu {

template <class S>
struct V3 {
  S x, y, z;
};
template <class S>
FCLG_HD V3<S> v3(S a, S b, S c) { return V3<S>{a, b, c}; }
template <class S>
FCLG_HD V3<S> operator+(const V3<S>& a, const V3<S>& b) { return v3<S>(a.x + b.x, a.y + b.y, a.z + b.z); }
template <class S>
FCLG_HD V3<S> operator-(const V3<S>& a, const V3<S>& b) { return v3<S>(a.x - b.x, a.y - b.y, a.z - b.z); }
template <class S>
FCLG_HD V3<S> operator*(const V3<S>& a, S s) { return v3<S>(a.x * s, a.y * s, a.z * s); }
template <class S>
FCLG_HD S dot(const V3<S>& a, const V3<S>& b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
template <class S>
FCLG_HD V3<S> cross(const V3<S>& a, const V3<S>& b) {
  return v3<S>(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
template <class S>
FCLG_HD S sqnorm(const V3<S>& a) { return (a.x * a.x + a.y * a.y) + a.z * a.z; }

// Row-major 3x3.
template <class S>
struct M3 {
  S m[9];
  FCLG_HD S operator()(int r, int c) const { return m[3 * r + c]; }
  FCLG_HD S& operator()(int r, int c) { return m[3 * r + c]; }
};
template <class S>
FCLG_HD V3<S> mulv(const M3<S>& A, const V3<S>& v) {
  return v3<S>((A(0, 0) * v.x + A(0, 1) * v.y) + A(0, 2) * v.z, (A(1, 0) * v.x + A(1, 1) * v.y) + A(1, 2) * v.z,
               (A(2, 0) * v.x + A(2, 1) * v.y) + A(2, 2) * v.z);
}
template <class S>
FCLG_HD V3<S> mulTv(const M3<S>& A, const V3<S>& v) {
  return v3<S>((A(0, 0) * v.x + A(1, 0) * v.y) + A(2, 0) * v.z, (A(0, 1) * v.x + A(1, 1) * v.y) + A(2, 1) * v.z,
               (A(0, 2) * v.x + A(1, 2) * v.y) + A(2, 2) * v.z);
}
template <class S>
FCLG_HD M3<S> mul(const M3<S>& A, const M3<S>& B) {
  M3<S> C;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) C(i, j) = (A(i, 0) * B(0, j) + A(i, 1) * B(1, j)) + A(i, 2) * B(2, j);
  return C;
}
template <class S>
FCLG_HD M3<S> mulT(const M3<S>& A, const M3<S>& B) {
  M3<S> C;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) C(i, j) = (A(0, i) * B(0, j) + A(1, i) * B(1, j)) + A(2, i) * B(2, j);
  return C;
}

// Relative transform for collide (math/geometry-inl.h:655-682): R = R1^T R2,
// T = R1^T (t2 - t1).  tf arrays are 3x4 row-major.
FCLG_HD void rel_collide(const double* tf1, const double* tf2, M3<double>& R, V3<double>& T) {
  M3<double> R1, R2;
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) {
      R1(r, c) = tf1[4 * r + c];
      R2(r, c) = tf2[4 * r + c];
    }
  R = mulT(R1, R2);
  V3<double> d = v3<double>(tf2[3] - tf1[3], tf2[7] - tf1[7], tf2[11] - tf1[11]);
  T = mulTv(R1, d);
}
// Relative transform for distance (mesh_distance_traversal_node-inl.h:631):
// tf = tf1.inverse(Isometry) * tf2 -> R = R1^T R2, T = R1^T t2 + (-(R1^T t1)).
FCLG_HD void rel_distance(const double* tf1, const double* tf2, M3<double>& R, V3<double>& T) {
  M3<double> Ri, R2;
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) {
      Ri(r, c) = tf1[4 * c + r];
      R2(r, c) = tf2[4 * r + c];
    }
  V3<double> t1 = v3<double>(tf1[3], tf1[7], tf1[11]);
  V3<double> t2 = v3<double>(tf2[3], tf2[7], tf2[11]);
  V3<double> ti = mulv(Ri, t1);
  ti = v3<double>(-ti.x, -ti.y, -ti.z);
  R = mul(Ri, R2);
  T = mulv(Ri, t2) + ti;
}

// ---------------------------------------------------------------------------------
// OBB overlap (math/bv/OBB-inl.h:383-523)
// ---------------------------------------------------------------------------------
template <class S>
FCLG_HD bool obb_disjoint(const M3<S>& B, const V3<S>& T, const V3<S>& a, const V3<S>& b) {
  const S reps = (S)1e-6;
  M3<S> Bf;
#pragma unroll
  for (int i = 0; i < 9; ++i) Bf.m[i] = fabs(B.m[i]) + reps;
  S t, s;
  t = ((T.x < 0.0) ? -T.x : T.x);
  if (t > (a.x + ((Bf(0, 0) * b.x + Bf(0, 1) * b.y) + Bf(0, 2) * b.z))) return true;
  s = (B(0, 0) * T.x + B(1, 0) * T.y) + B(2, 0) * T.z;
  t = ((s < 0.0) ? -s : s);
  if (t > (b.x + ((Bf(0, 0) * a.x + Bf(1, 0) * a.y) + Bf(2, 0) * a.z))) return true;
  t = ((T.y < 0.0) ? -T.y : T.y);
  if (t > (a.y + ((Bf(1, 0) * b.x + Bf(1, 1) * b.y) + Bf(1, 2) * b.z))) return true;
  t = ((T.z < 0.0) ? -T.z : T.z);
  if (t > (a.z + ((Bf(2, 0) * b.x + Bf(2, 1) * b.y) + Bf(2, 2) * b.z))) return true;
  s = (B(0, 1) * T.x + B(1, 1) * T.y) + B(2, 1) * T.z;
  t = ((s < 0.0) ? -s : s);
  if (t > (b.y + ((Bf(0, 1) * a.x + Bf(1, 1) * a.y) + Bf(2, 1) * a.z))) return true;
  s = (B(0, 2) * T.x + B(1, 2) * T.y) + B(2, 2) * T.z;
  t = ((s < 0.0) ? -s : s);
  if (t > (b.z + ((Bf(0, 2) * a.x + Bf(1, 2) * a.y) + Bf(2, 2) * a.z))) return true;

  s = T.z * B(1, 0) - T.y * B(2, 0);
  t = ((s < 0.0) ? -s : s);
  if (t > (a.y * Bf(2, 0) + a.z * Bf(1, 0) + b.y * Bf(0, 2) + b.z * Bf(0, 1))) return true;
  s = T.z * B(1, 1) - T.y * B(2, 1);
  t = ((s < 0.0) ? -s : s);
  if (t > (a.y * Bf(2, 1) + a.z * Bf(1, 1) + b.x * Bf(0, 2) + b.z * Bf(0, 0))) return true;
  s = T.z * B(1, 2) - T.y * B(2, 2);
  t = ((s < 0.0) ? -s : s);
  if (t > (a.y * Bf(2, 2) + a.z * Bf(1, 2) + b.x * Bf(0, 1) + b.y * Bf(0, 0))) return true;
  s = T.x * B(2, 0) - T.z * B(0, 0);
  t = ((s < 0.0) ? -s : s);
  if (t > (a.x * Bf(2, 0) + a.z * Bf(0, 0) + b.y * Bf(1, 2) + b.z * Bf(1, 1))) return true;
  s = T.x * B(2, 1) - T.z * B(0, 1);
  t = ((s < 0.0) ? -s : s);
  if (t > (a.x * Bf(2, 1) + a.z * Bf(0, 1) + b.x * Bf(1, 2) + b.z * Bf(1, 0))) return true;
  s = T.x * B(2, 2) - T.z * B(0, 2);
  t = ((s < 0.0) ? -s : s);
  if (t > (a.x * Bf(2, 2) + a.z * Bf(0, 2) + b.x * Bf(1, 1) + b.y * Bf(1, 0))) return true;
  s = T.y * B(0, 0) - T.x * B(1, 0);
  t = ((s < 0.0) ? -s : s);
  if (t > (a.x * Bf(1, 0) + a.y * Bf(0, 0) + b.y * Bf(2, 2) + b.z * Bf(2, 1))) return true;
  s = T.y * B(0, 1) - T.x * B(1, 1);
  t = ((s < 0.0) ? -s : s);
  if (t > (a.x * Bf(1, 1) + a.y * Bf(0, 1) + b.x * Bf(2, 2) + b.z * Bf(2, 0))) return true;
  s = T.y * B(0, 2) - T.x * B(1, 2);
  t = ((s < 0.0) ? -s : s);
  if (t > (a.x * Bf(1, 2) + a.y * Bf(0, 2) + b.x * Bf(2, 1) + b.y * Bf(2, 0))) return true;
  return false;
}

// Exact FP64 overlap of two FP64 nodes under (R0, T0).
FCLG_HD bool obb_overlap64(const M3<double>& R0, const V3<double>& T0, const NodeD& b1, const NodeD& b2) {
  M3<double> A1, A2;
#pragma unroll
  for (int i = 0; i < 9; ++i) {
    A1.m[i] = b1.axis[i];
    A2.m[i] = b2.axis[i];
  }
  const M3<double> R0b2 = mul(R0, A2);
  const M3<double> R = mulT(A1, R0b2);
  const V3<double> To1 = v3(b1.To[0], b1.To[1], b1.To[2]);
  const V3<double> To2 = v3(b2.To[0], b2.To[1], b2.To[2]);
  const V3<double> Ttemp = (mulv(R0, To2) + T0) - To1;
  const V3<double> T = mulTv(A1, Ttemp);
  return !obb_disjoint<double>(R, T, v3(b1.ext[0], b1.ext[1], b1.ext[2]), v3(b2.ext[0], b2.ext[1], b2.ext[2]));
}

// ---------------------------------------------------------------------------------
// Triangle-triangle SAT (narrowphase/detail/traversal/collision/intersect-inl.h:597-617,
// 727-798, 1085-1106)
// ---------------------------------------------------------------------------------
// std::min / std::max semantics (first argument wins ties and NaN comparisons).
template <class S>
FCLG_HD S smin(S a, S b) { return (b < a) ? b : a; }
template <class S>
FCLG_HD S smax(S a, S b) { return (a < b) ? b : a; }

template <class S>
FCLG_HD bool project6(const V3<S>& ax, const V3<S>& p1, const V3<S>& p2, const V3<S>& p3, const V3<S>& q1,
                      const V3<S>& q2, const V3<S>& q3) {
  const S P1 = dot(ax, p1), P2 = dot(ax, p2), P3 = dot(ax, p3);
  const S Q1 = dot(ax, q1), Q2 = dot(ax, q2), Q3 = dot(ax, q3);
  const S mn1 = smin(P1, smin(P2, P3));
  const S mx2 = smax(Q1, smax(Q2, Q3));
  if (mn1 > mx2) return false;
  const S mx1 = smax(P1, smax(P2, P3));
  const S mn2 = smin(Q1, smin(Q2, Q3));
  if (mn2 > mx1) return false;
  return true;
}

template <class S>
FCLG_HD bool tri_intersect(const V3<S>& P1, const V3<S>& P2, const V3<S>& P3, const V3<S>& Q1, const V3<S>& Q2,
                           const V3<S>& Q3, const M3<S>& R, const V3<S>& T) {
  const V3<S> Q1_ = mulv(R, Q1) + T, Q2_ = mulv(R, Q2) + T, Q3_ = mulv(R, Q3) + T;
  const V3<S> p1 = P1 - P1, p2 = P2 - P1, p3 = P3 - P1;
  const V3<S> q1 = Q1_ - P1, q2 = Q2_ - P1, q3 = Q3_ - P1;
  const V3<S> e1 = p2 - p1, e2 = p3 - p2;
  const V3<S> n1 = cross(e1, e2);
  if (!project6(n1, p1, p2, p3, q1, q2, q3)) return false;
  const V3<S> f1 = q2 - q1, f2 = q3 - q2;
  const V3<S> m1 = cross(f1, f2);
  if (!project6(m1, p1, p2, p3, q1, q2, q3)) return false;
  if (!project6(cross(e1, f1), p1, p2, p3, q1, q2, q3)) return false;
  if (!project6(cross(e1, f2), p1, p2, p3, q1, q2, q3)) return false;
  const V3<S> f3 = q1 - q3;
  if (!project6(cross(e1, f3), p1, p2, p3, q1, q2, q3)) return false;
  if (!project6(cross(e2, f1), p1, p2, p3, q1, q2, q3)) return false;
  if (!project6(cross(e2, f2), p1, p2, p3, q1, q2, q3)) return false;
  if (!project6(cross(e2, f3), p1, p2, p3, q1, q2, q3)) return false;
  const V3<S> e3 = p1 - p3;
  if (!project6(cross(e3, f1), p1, p2, p3, q1, q2, q3)) return false;
  if (!project6(cross(e3, f2), p1, p2, p3, q1, q2, q3)) return false;
  if (!project6(cross(e3, f3), p1, p2, p3, q1, q2, q3)) return false;
  if (!project6(cross(e1, n1), p1, p2, p3, q1, q2, q3)) return false;
  if (!project6(cross(e2, n1), p1, p2, p3, q1, q2, q3)) return false;
  if (!project6(cross(e3, n1), p1, p2, p3, q1, q2, q3)) return false;
  if (!project6(cross(f1, m1), p1, p2, p3, q1, q2, q3)) return false;
  if (!project6(cross(f2, m1), p1, p2, p3, q1, q2, q3)) return false;
  if (!project6(cross(f3, m1), p1, p2, p3, q1, q2, q3)) return false;
  return true;
}

// ---------------------------------------------------------------------------------
// RSS distance (math/bv/RSS-inl.h:450-1224, 1956-1974)
// ---------------------------------------------------------------------------------
template <class S>
FCLG_HD void clip_range(S& val, S a, S b) {
  if (val < a) val = a;
  else if (val > b) val = b;
}

template <class S>
FCLG_HD void seg_coords(S& t, S& u, S a, S b, S A_dot_B, S A_dot_T, S B_dot_T) {
  const S denom = 1 - A_dot_B * A_dot_B;
  if (denom == 0) {
    t = 0;
  } else {
    t = (A_dot_T - B_dot_T * A_dot_B) / denom;
    clip_range<S>(t, (S)0, a);
  }
  u = t * A_dot_B - B_dot_T;
  if (u < 0) {
    u = 0;
    t = A_dot_T;
    clip_range<S>(t, (S)0, a);
  } else if (u > b) {
    u = b;
    t = u * A_dot_B + A_dot_T;
    clip_range<S>(t, (S)0, a);
  }
}

template <class S>
FCLG_HD bool in_voronoi(S a, S b, S Anorm_dot_B, S Anorm_dot_T, S A_dot_B, S A_dot_T, S B_dot_T) {
  if (fabs(Anorm_dot_B) < (S)1e-7) return false;
  S u = -Anorm_dot_T / Anorm_dot_B;
  clip_range<S>(u, (S)0, b);
  S t = u * A_dot_B + A_dot_T;
  clip_range<S>(t, (S)0, a);
  const S v = t * A_dot_B - B_dot_T;
  if (Anorm_dot_B > 0) {
    if (v > (u + (S)1e-7)) return true;
  } else {
    if (v < (u - (S)1e-7)) return true;
  }
  return false;
}

// Rectangle-rectangle distance (PQP's RectDist as restated in FCL).  Returns the
// distance; when P != nullptr also the closest points in the first frame.
template <class S>
FCLG_HD S rect_distance(const M3<S>& Rab, const V3<S>& Tab, const S a[2], const S b[2], V3<S>* P, V3<S>* Q) {
  const S A0_dot_B0 = Rab(0, 0), A0_dot_B1 = Rab(0, 1), A1_dot_B0 = Rab(1, 0), A1_dot_B1 = Rab(1, 1);
  const S aA0_dot_B0 = a[0] * A0_dot_B0, aA0_dot_B1 = a[0] * A0_dot_B1;
  const S aA1_dot_B0 = a[1] * A1_dot_B0, aA1_dot_B1 = a[1] * A1_dot_B1;
  const S bA0_dot_B0 = b[0] * A0_dot_B0, bA1_dot_B0 = b[0] * A1_dot_B0;
  const S bA0_dot_B1 = b[1] * A0_dot_B1, bA1_dot_B1 = b[1] * A1_dot_B1;
  const V3<S> Tba = mulTv(Rab, Tab);
  V3<S> D;
  S t, u;
#define FCLG_RECT_RETURN(px, py)                 \
  do {                                           \
    if (P) {                                     \
      *P = v3<S>((px), (py), (S)0);              \
      *Q = D + *P;                               \
    }                                            \
    return sqrt(sqnorm(D));                      \
  } while (0)

  const S ALL_x = -Tba.x;
  const S ALU_x = ALL_x + aA1_dot_B0;
  const S AUL_x = ALL_x + aA0_dot_B0;
  const S AUU_x = ALU_x + aA0_dot_B0;
  S LA1_lx, LA1_ux, UA1_lx, UA1_ux, LB1_lx, LB1_ux, UB1_lx, UB1_ux;
  if (ALL_x < ALU_x) { LA1_lx = ALL_x; LA1_ux = ALU_x; UA1_lx = AUL_x; UA1_ux = AUU_x; }
  else { LA1_lx = ALU_x; LA1_ux = ALL_x; UA1_lx = AUU_x; UA1_ux = AUL_x; }
  const S BLL_x = Tab.x;
  const S BLU_x = BLL_x + bA0_dot_B1;
  const S BUL_x = BLL_x + bA0_dot_B0;
  const S BUU_x = BLU_x + bA0_dot_B0;
  if (BLL_x < BLU_x) { LB1_lx = BLL_x; LB1_ux = BLU_x; UB1_lx = BUL_x; UB1_ux = BUU_x; }
  else { LB1_lx = BLU_x; LB1_ux = BLL_x; UB1_lx = BUU_x; UB1_ux = BUL_x; }

  if ((UA1_ux > b[0]) && (UB1_ux > a[0])) {
    if (((UA1_lx > b[0]) || in_voronoi<S>(b[1], a[1], A1_dot_B0, aA0_dot_B0 - b[0] - Tba.x, A1_dot_B1,
                                            aA0_dot_B1 - Tba.y, -Tab.y - bA1_dot_B0)) &&
        ((UB1_lx > a[0]) || in_voronoi<S>(a[1], b[1], A0_dot_B1, Tab.x + bA0_dot_B0 - a[0], A1_dot_B1,
                                            Tab.y + bA1_dot_B0, Tba.y - aA0_dot_B1))) {
      seg_coords<S>(t, u, a[1], b[1], A1_dot_B1, Tab.y + bA1_dot_B0, Tba.y - aA0_dot_B1);
      D.x = Tab.x + Rab(0, 0) * b[0] + Rab(0, 1) * u - a[0];
      D.y = Tab.y + Rab(1, 0) * b[0] + Rab(1, 1) * u - t;
      D.z = Tab.z + Rab(2, 0) * b[0] + Rab(2, 1) * u;
      FCLG_RECT_RETURN(a[0], t);
    }
  }
  if ((UA1_lx < 0) && (LB1_ux > a[0])) {
    if (((UA1_ux < 0) || in_voronoi<S>(b[1], a[1], -A1_dot_B0, Tba.x - aA0_dot_B0, A1_dot_B1, aA0_dot_B1 - Tba.y,
                                         -Tab.y)) &&
        ((LB1_lx > a[0]) ||
         in_voronoi<S>(a[1], b[1], A0_dot_B1, Tab.x - a[0], A1_dot_B1, Tab.y, Tba.y - aA0_dot_B1))) {
      seg_coords<S>(t, u, a[1], b[1], A1_dot_B1, Tab.y, Tba.y - aA0_dot_B1);
      D.x = Tab.x + Rab(0, 1) * u - a[0];
      D.y = Tab.y + Rab(1, 1) * u - t;
      D.z = Tab.z + Rab(2, 1) * u;
      FCLG_RECT_RETURN(a[0], t);
    }
  }
  if ((LA1_ux > b[0]) && (UB1_lx < 0)) {
    if (((LA1_lx > b[0]) ||
         in_voronoi<S>(b[1], a[1], A1_dot_B0, -Tba.x - b[0], A1_dot_B1, -Tba.y, -Tab.y - bA1_dot_B0)) &&
        ((UB1_ux < 0) || in_voronoi<S>(a[1], b[1], -A0_dot_B1, -Tab.x - bA0_dot_B0, A1_dot_B1,
                                         Tab.y + bA1_dot_B0, Tba.y))) {
      seg_coords<S>(t, u, a[1], b[1], A1_dot_B1, Tab.y + bA1_dot_B0, Tba.y);
      D.x = Tab.x + Rab(0, 0) * b[0] + Rab(0, 1) * u;
      D.y = Tab.y + Rab(1, 0) * b[0] + Rab(1, 1) * u - t;
      D.z = Tab.z + Rab(2, 0) * b[0] + Rab(2, 1) * u;
      FCLG_RECT_RETURN((S)0, t);
    }
  }
  if ((LA1_lx < 0) && (LB1_lx < 0)) {
    if (((LA1_ux < 0) || in_voronoi<S>(b[1], a[1], -A1_dot_B0, Tba.x, A1_dot_B1, -Tba.y, -Tab.y)) &&
        ((LB1_ux < 0) || in_voronoi<S>(a[1], b[1], -A0_dot_B1, -Tab.x, A1_dot_B1, Tab.y, Tba.y))) {
      seg_coords<S>(t, u, a[1], b[1], A1_dot_B1, Tab.y, Tba.y);
      D.x = Tab.x + Rab(0, 1) * u;
      D.y = Tab.y + Rab(1, 1) * u - t;
      D.z = Tab.z + Rab(2, 1) * u;
      FCLG_RECT_RETURN((S)0, t);
    }
  }

  const S ALL_y = -Tba.y;
  const S ALU_y = ALL_y + aA1_dot_B1;
  const S AUL_y = ALL_y + aA0_dot_B1;
  const S AUU_y = ALU_y + aA0_dot_B1;
  S LA1_ly, LA1_uy, UA1_ly, UA1_uy, LB0_lx, LB0_ux, UB0_lx, UB0_ux;
  if (ALL_y < ALU_y) { LA1_ly = ALL_y; LA1_uy = ALU_y; UA1_ly = AUL_y; UA1_uy = AUU_y; }
  else { LA1_ly = ALU_y; LA1_uy = ALL_y; UA1_ly = AUU_y; UA1_uy = AUL_y; }
  if (BLL_x < BUL_x) { LB0_lx = BLL_x; LB0_ux = BUL_x; UB0_lx = BLU_x; UB0_ux = BUU_x; }
  else { LB0_lx = BUL_x; LB0_ux = BLL_x; UB0_lx = BUU_x; UB0_ux = BLU_x; }

  if ((UA1_uy > b[1]) && (UB0_ux > a[0])) {
    if (((UA1_ly > b[1]) || in_voronoi<S>(b[0], a[1], A1_dot_B1, aA0_dot_B1 - Tba.y - b[1], A1_dot_B0,
                                            aA0_dot_B0 - Tba.x, -Tab.y - bA1_dot_B1)) &&
        ((UB0_lx > a[0]) || in_voronoi<S>(a[1], b[0], A0_dot_B0, Tab.x - a[0] + bA0_dot_B1, A1_dot_B0,
                                            Tab.y + bA1_dot_B1, Tba.x - aA0_dot_B0))) {
      seg_coords<S>(t, u, a[1], b[0], A1_dot_B0, Tab.y + bA1_dot_B1, Tba.x - aA0_dot_B0);
      D.x = Tab.x + Rab(0, 1) * b[1] + Rab(0, 0) * u - a[0];
      D.y = Tab.y + Rab(1, 1) * b[1] + Rab(1, 0) * u - t;
      D.z = Tab.z + Rab(2, 1) * b[1] + Rab(2, 0) * u;
      FCLG_RECT_RETURN(a[0], t);
    }
  }
  if ((UA1_ly < 0) && (LB0_ux > a[0])) {
    if (((UA1_uy < 0) || in_voronoi<S>(b[0], a[1], -A1_dot_B1, Tba.y - aA0_dot_B1, A1_dot_B0, aA0_dot_B0 - Tba.x,
                                         -Tab.y)) &&
        ((LB0_lx > a[0]) ||
         in_voronoi<S>(a[1], b[0], A0_dot_B0, Tab.x - a[0], A1_dot_B0, Tab.y, Tba.x - aA0_dot_B0))) {
      seg_coords<S>(t, u, a[1], b[0], A1_dot_B0, Tab.y, Tba.x - aA0_dot_B0);
      D.x = Tab.x + Rab(0, 0) * u - a[0];
      D.y = Tab.y + Rab(1, 0) * u - t;
      D.z = Tab.z + Rab(2, 0) * u;
      FCLG_RECT_RETURN(a[0], t);
    }
  }
  if ((LA1_uy > b[1]) && (UB0_lx < 0)) {
    if (((LA1_ly > b[1]) ||
         in_voronoi<S>(b[0], a[1], A1_dot_B1, -Tba.y - b[1], A1_dot_B0, -Tba.x, -Tab.y - bA1_dot_B1)) &&
        ((UB0_ux < 0) || in_voronoi<S>(a[1], b[0], -A0_dot_B0, -Tab.x - bA0_dot_B1, A1_dot_B0,
                                         Tab.y + bA1_dot_B1, Tba.x))) {
      seg_coords<S>(t, u, a[1], b[0], A1_dot_B0, Tab.y + bA1_dot_B1, Tba.x);
      D.x = Tab.x + Rab(0, 1) * b[1] + Rab(0, 0) * u;
      D.y = Tab.y + Rab(1, 1) * b[1] + Rab(1, 0) * u - t;
      D.z = Tab.z + Rab(2, 1) * b[1] + Rab(2, 0) * u;
      FCLG_RECT_RETURN((S)0, t);
    }
  }
  if ((LA1_ly < 0) && (LB0_lx < 0)) {
    if (((LA1_uy < 0) || in_voronoi<S>(b[0], a[1], -A1_dot_B1, Tba.y, A1_dot_B0, -Tba.x, -Tab.y)) &&
        ((LB0_ux < 0) || in_voronoi<S>(a[1], b[0], -A0_dot_B0, -Tab.x, A1_dot_B0, Tab.y, Tba.x))) {
      seg_coords<S>(t, u, a[1], b[0], A1_dot_B0, Tab.y, Tba.x);
      D.x = Tab.x + Rab(0, 0) * u;
      D.y = Tab.y + Rab(1, 0) * u - t;
      D.z = Tab.z + Rab(2, 0) * u;
      FCLG_RECT_RETURN((S)0, t);
    }
  }

  const S BLL_y = Tab.y;
  const S BLU_y = BLL_y + bA1_dot_B1;
  const S BUL_y = BLL_y + bA1_dot_B0;
  const S BUU_y = BLU_y + bA1_dot_B0;
  S LA0_lx, LA0_ux, UA0_lx, UA0_ux, LB1_ly, LB1_uy, UB1_ly, UB1_uy;
  if (ALL_x < AUL_x) { LA0_lx = ALL_x; LA0_ux = AUL_x; UA0_lx = ALU_x; UA0_ux = AUU_x; }
  else { LA0_lx = AUL_x; LA0_ux = ALL_x; UA0_lx = AUU_x; UA0_ux = ALU_x; }
  if (BLL_y < BLU_y) { LB1_ly = BLL_y; LB1_uy = BLU_y; UB1_ly = BUL_y; UB1_uy = BUU_y; }
  else { LB1_ly = BLU_y; LB1_uy = BLL_y; UB1_ly = BUU_y; UB1_uy = BUL_y; }

  if ((UA0_ux > b[0]) && (UB1_uy > a[1])) {
    if (((UA0_lx > b[0]) || in_voronoi<S>(b[1], a[0], A0_dot_B0, aA1_dot_B0 - Tba.x - b[0], A0_dot_B1,
                                            aA1_dot_B1 - Tba.y, -Tab.x - bA0_dot_B0)) &&
        ((UB1_ly > a[1]) || in_voronoi<S>(a[0], b[1], A1_dot_B1, Tab.y - a[1] + bA1_dot_B0, A0_dot_B1,
                                            Tab.x + bA0_dot_B0, Tba.y - aA1_dot_B1))) {
      seg_coords<S>(t, u, a[0], b[1], A0_dot_B1, Tab.x + bA0_dot_B0, Tba.y - aA1_dot_B1);
      D.x = Tab.x + Rab(0, 0) * b[0] + Rab(0, 1) * u - t;
      D.y = Tab.y + Rab(1, 0) * b[0] + Rab(1, 1) * u - a[1];
      D.z = Tab.z + Rab(2, 0) * b[0] + Rab(2, 1) * u;
      FCLG_RECT_RETURN(t, a[1]);
    }
  }
  if ((UA0_lx < 0) && (LB1_uy > a[1])) {
    if (((UA0_ux < 0) || in_voronoi<S>(b[1], a[0], -A0_dot_B0, Tba.x - aA1_dot_B0, A0_dot_B1, aA1_dot_B1 - Tba.y,
                                         -Tab.x)) &&
        ((LB1_ly > a[1]) ||
         in_voronoi<S>(a[0], b[1], A1_dot_B1, Tab.y - a[1], A0_dot_B1, Tab.x, Tba.y - aA1_dot_B1))) {
      seg_coords<S>(t, u, a[0], b[1], A0_dot_B1, Tab.x, Tba.y - aA1_dot_B1);
      D.x = Tab.x + Rab(0, 1) * u - t;
      D.y = Tab.y + Rab(1, 1) * u - a[1];
      D.z = Tab.z + Rab(2, 1) * u;
      FCLG_RECT_RETURN(t, a[1]);
    }
  }
  if ((LA0_ux > b[0]) && (UB1_ly < 0)) {
    if (((LA0_lx > b[0]) ||
         in_voronoi<S>(b[1], a[0], A0_dot_B0, -b[0] - Tba.x, A0_dot_B1, -Tba.y, -bA0_dot_B0 - Tab.x)) &&
        ((UB1_uy < 0) || in_voronoi<S>(a[0], b[1], -A1_dot_B1, -Tab.y - bA1_dot_B0, A0_dot_B1,
                                         Tab.x + bA0_dot_B0, Tba.y))) {
      seg_coords<S>(t, u, a[0], b[1], A0_dot_B1, Tab.x + bA0_dot_B0, Tba.y);
      D.x = Tab.x + Rab(0, 0) * b[0] + Rab(0, 1) * u - t;
      D.y = Tab.y + Rab(1, 0) * b[0] + Rab(1, 1) * u;
      D.z = Tab.z + Rab(2, 0) * b[0] + Rab(2, 1) * u;
      FCLG_RECT_RETURN(t, (S)0);
    }
  }
  if ((LA0_lx < 0) && (LB1_ly < 0)) {
    if (((LA0_ux < 0) || in_voronoi<S>(b[1], a[0], -A0_dot_B0, Tba.x, A0_dot_B1, -Tba.y, -Tab.x)) &&
        ((LB1_uy < 0) || in_voronoi<S>(a[0], b[1], -A1_dot_B1, -Tab.y, A0_dot_B1, Tab.x, Tba.y))) {
      seg_coords<S>(t, u, a[0], b[1], A0_dot_B1, Tab.x, Tba.y);
      D.x = Tab.x + Rab(0, 1) * u - t;
      D.y = Tab.y + Rab(1, 1) * u;
      D.z = Tab.z + Rab(2, 1) * u;
      FCLG_RECT_RETURN(t, (S)0);
    }
  }

  S LA0_ly, LA0_uy, UA0_ly, UA0_uy, LB0_ly, LB0_uy, UB0_ly, UB0_uy;
  if (ALL_y < AUL_y) { LA0_ly = ALL_y; LA0_uy = AUL_y; UA0_ly = ALU_y; UA0_uy = AUU_y; }
  else { LA0_ly = AUL_y; LA0_uy = ALL_y; UA0_ly = AUU_y; UA0_uy = ALU_y; }
  if (BLL_y < BUL_y) { LB0_ly = BLL_y; LB0_uy = BUL_y; UB0_ly = BLU_y; UB0_uy = BUU_y; }
  else { LB0_ly = BUL_y; LB0_uy = BLL_y; UB0_ly = BUU_y; UB0_uy = BLU_y; }

  if ((UA0_uy > b[1]) && (UB0_uy > a[1])) {
    if (((UA0_ly > b[1]) || in_voronoi<S>(b[0], a[0], A0_dot_B1, aA1_dot_B1 - Tba.y - b[1], A0_dot_B0,
                                            aA1_dot_B0 - Tba.x, -Tab.x - bA0_dot_B1)) &&
        ((UB0_ly > a[1]) || in_voronoi<S>(a[0], b[0], A1_dot_B0, Tab.y - a[1] + bA1_dot_B1, A0_dot_B0,
                                            Tab.x + bA0_dot_B1, Tba.x - aA1_dot_B0))) {
      seg_coords<S>(t, u, a[0], b[0], A0_dot_B0, Tab.x + bA0_dot_B1, Tba.x - aA1_dot_B0);
      D.x = Tab.x + Rab(0, 1) * b[1] + Rab(0, 0) * u - t;
      D.y = Tab.y + Rab(1, 1) * b[1] + Rab(1, 0) * u - a[1];
      D.z = Tab.z + Rab(2, 1) * b[1] + Rab(2, 0) * u;
      FCLG_RECT_RETURN(t, a[1]);
    }
  }
  if ((UA0_ly < 0) && (LB0_uy > a[1])) {
    if (((UA0_uy < 0) || in_voronoi<S>(b[0], a[0], -A0_dot_B1, Tba.y - aA1_dot_B1, A0_dot_B0, aA1_dot_B0 - Tba.x,
                                         -Tab.x)) &&
        ((LB0_ly > a[1]) ||
         in_voronoi<S>(a[0], b[0], A1_dot_B0, Tab.y - a[1], A0_dot_B0, Tab.x, Tba.x - aA1_dot_B0))) {
      seg_coords<S>(t, u, a[0], b[0], A0_dot_B0, Tab.x, Tba.x - aA1_dot_B0);
      D.x = Tab.x + Rab(0, 0) * u - t;
      D.y = Tab.y + Rab(1, 0) * u - a[1];
      D.z = Tab.z + Rab(2, 0) * u;
      FCLG_RECT_RETURN(t, a[1]);
    }
  }
  if ((LA0_uy > b[1]) && (UB0_ly < 0)) {
    if (((LA0_ly > b[1]) ||
         in_voronoi<S>(b[0], a[0], A0_dot_B1, -Tba.y - b[1], A0_dot_B0, -Tba.x, -Tab.x - bA0_dot_B1)) &&
        ((UB0_uy < 0) || in_voronoi<S>(a[0], b[0], -A1_dot_B0, -Tab.y - bA1_dot_B1, A0_dot_B0,
                                         Tab.x + bA0_dot_B1, Tba.x))) {
      seg_coords<S>(t, u, a[0], b[0], A0_dot_B0, Tab.x + bA0_dot_B1, Tba.x);
      D.x = Tab.x + Rab(0, 1) * b[1] + Rab(0, 0) * u - t;
      D.y = Tab.y + Rab(1, 1) * b[1] + Rab(1, 0) * u;
      D.z = Tab.z + Rab(2, 1) * b[1] + Rab(2, 0) * u;
      FCLG_RECT_RETURN(t, (S)0);
    }
  }
  if ((LA0_ly < 0) && (LB0_ly < 0)) {
    if (((LA0_uy < 0) || in_voronoi<S>(b[0], a[0], -A0_dot_B1, Tba.y, A0_dot_B0, -Tba.x, -Tab.x)) &&
        ((LB0_uy < 0) || in_voronoi<S>(a[0], b[0], -A1_dot_B0, -Tab.y, A0_dot_B0, Tab.x, Tba.x))) {
      seg_coords<S>(t, u, a[0], b[0], A0_dot_B0, Tab.x, Tba.x);
      D.x = Tab.x + Rab(0, 0) * u - t;
      D.y = Tab.y + Rab(1, 0) * u;
      D.z = Tab.z + Rab(2, 0) * u;
      FCLG_RECT_RETURN(t, (S)0);
    }
  }
#undef FCLG_RECT_RETURN

  S sep1, sep2;
  if (Tab.z > 0.0) {
    sep1 = Tab.z;
    if (Rab(2, 0) < 0.0) sep1 += b[0] * Rab(2, 0);
    if (Rab(2, 1) < 0.0) sep1 += b[1] * Rab(2, 1);
  } else {
    sep1 = -Tab.z;
    if (Rab(2, 0) > 0.0) sep1 -= b[0] * Rab(2, 0);
    if (Rab(2, 1) > 0.0) sep1 -= b[1] * Rab(2, 1);
  }
  if (Tba.z < 0) {
    sep2 = -Tba.z;
    if (Rab(0, 2) < 0.0) sep2 += a[0] * Rab(0, 2);
    if (Rab(1, 2) < 0.0) sep2 += a[1] * Rab(1, 2);
  } else {
    sep2 = Tba.z;
    if (Rab(0, 2) > 0.0) sep2 -= a[0] * Rab(0, 2);
    if (Rab(1, 2) > 0.0) sep2 -= a[1] * Rab(1, 2);
  }
  if (P) {
    if (sep1 >= sep2 && sep1 >= 0) {
      D = v3<S>(0, 0, Tab.z > 0 ? sep1 : -sep1);
      *Q = D;
      *P = v3<S>(0, 0, 0);
    }
    if (sep2 >= sep1 && sep2 >= 0) {
      const V3<S> Q_ = Tab;
      V3<S> P_;
      if (Tba.z < 0) {
        P_.x = Rab(0, 2) * sep2 + Tab.x;
        P_.y = Rab(1, 2) * sep2 + Tab.y;
        P_.z = Rab(2, 2) * sep2 + Tab.z;
      } else {
        P_.x = -Rab(0, 2) * sep2 + Tab.x;
        P_.y = -Rab(1, 2) * sep2 + Tab.y;
        P_.z = -Rab(2, 2) * sep2 + Tab.z;
      }
      *P = P_;
      *Q = Q_;
    }
  }
  const S sep = (sep1 > sep2 ? sep1 : sep2);
  return (sep > 0 ? sep : (S)0);
}

// RSS-RSS distance under (R0,T0) (RSS-inl.h:1956-1974); axis = the node's box axes.
template <class S>
FCLG_HD S rss_distance(const M3<S>& R0, const V3<S>& T0, const M3<S>& A1, const V3<S>& To1, const S l1[2], S r1,
                       const M3<S>& A2, const V3<S>& To2, const S l2[2], S r2) {
  const M3<S> R0b2 = mul(R0, A2);
  const M3<S> R = mulT(A1, R0b2);
  const V3<S> Ttemp = (mulv(R0, To2) + T0) - To1;
  const V3<S> T = mulTv(A1, Ttemp);
  S dist = rect_distance<S>(R, T, l1, l2, (V3<S>*)nullptr, (V3<S>*)nullptr);
  dist -= (r1 + r2);
  return (dist < (S)0) ? (S)0 : dist;
}

// ---------------------------------------------------------------------------------
// Triangle distance (primitive_shape_algorithm/triangle_distance-inl.h:54-394)
// ---------------------------------------------------------------------------------
template <class S>
FCLG_HD void seg_points(const V3<S>& P, const V3<S>& A, const V3<S>& Q, const V3<S>& B, V3<S>& VEC, V3<S>& X,
                        V3<S>& Y) {
  V3<S> T = Q - P;
  const S A_dot_A = dot(A, A), B_dot_B = dot(B, B), A_dot_B = dot(A, B);
  const S A_dot_T = dot(A, T), B_dot_T = dot(B, T);
  const S denom = A_dot_A * B_dot_B - A_dot_B * A_dot_B;
  S t = (A_dot_T * B_dot_B - B_dot_T * A_dot_B) / denom;
  if ((t < 0) || isnan(t)) t = 0;
  else if (t > 1) t = 1;
  const S u = (t * A_dot_B - B_dot_T) / B_dot_B;
  if ((u <= 0) || isnan(u)) {
    Y = Q;
    t = A_dot_T / A_dot_A;
    if ((t <= 0) || isnan(t)) {
      X = P;
      VEC = Q - P;
    } else if (t >= 1) {
      X = P + A;
      VEC = Q - X;
    } else {
      X = P + A * t;
      VEC = cross(A, cross(T, A));
    }
  } else if (u >= 1) {
    Y = Q + B;
    t = (A_dot_B + A_dot_T) / A_dot_A;
    if ((t <= 0) || isnan(t)) {
      X = P;
      VEC = Y - P;
    } else if (t >= 1) {
      X = P + A;
      VEC = Y - X;
    } else {
      X = P + A * t;
      T = Y - P;
      VEC = cross(A, cross(T, A));
    }
  } else {
    Y = Q + B * u;
    if ((t <= 0) || isnan(t)) {
      X = P;
      VEC = cross(B, cross(T, B));
    } else if (t >= 1) {
      X = P + A;
      T = Q - X;
      VEC = cross(B, cross(T, B));
    } else {
      X = P + A * t;
      VEC = cross(A, B);
      if (dot(VEC, T) < 0) VEC = VEC * (S)(-1);
    }
  }
}

template <class S>
FCLG_HD S tri_distance(const V3<S> T1[3], const V3<S> T2[3], V3<S>& P, V3<S>& Q) {
  V3<S> Sv[3], Tv[3], VEC, V, Z;
  Sv[0] = T1[1] - T1[0];
  Sv[1] = T1[2] - T1[1];
  Sv[2] = T1[0] - T1[2];
  Tv[0] = T2[1] - T2[0];
  Tv[1] = T2[2] - T2[1];
  Tv[2] = T2[0] - T2[2];
  V3<S> minP = v3<S>(0, 0, 0), minQ = v3<S>(0, 0, 0);
  int shown_disjoint = 0;
  S mindd = sqnorm(T1[0] - T2[0]) + 1;
  for (int i = 0; i < 3; ++i) {
    for (int j = 0; j < 3; ++j) {
      seg_points<S>(T1[i], Sv[i], T2[j], Tv[j], VEC, P, Q);
      V = Q - P;
      const S dd = dot(V, V);
      if (dd <= mindd) {
        minP = P;
        minQ = Q;
        mindd = dd;
        Z = T1[(i + 2) % 3] - P;
        S a = dot(Z, VEC);
        Z = T2[(j + 2) % 3] - Q;
        S b = dot(Z, VEC);
        if ((a <= 0) && (b >= 0)) return sqrt(dd);
        const S p = dot(V, VEC);
        if (a < 0) a = 0;
        if (b > 0) b = 0;
        if ((p - a + b) > 0) shown_disjoint = 1;
      }
    }
  }
  const V3<S> Sn = cross(Sv[0], Sv[1]);
  const S Snl = dot(Sn, Sn);
  if (Snl > (S)1e-15) {
    S Tp[3];
    V = T1[0] - T2[0];
    Tp[0] = dot(V, Sn);
    V = T1[0] - T2[1];
    Tp[1] = dot(V, Sn);
    V = T1[0] - T2[2];
    Tp[2] = dot(V, Sn);
    int point = -1;
    if ((Tp[0] > 0) && (Tp[1] > 0) && (Tp[2] > 0)) {
      point = (Tp[0] < Tp[1]) ? 0 : 1;
      if (Tp[2] < Tp[point]) point = 2;
    } else if ((Tp[0] < 0) && (Tp[1] < 0) && (Tp[2] < 0)) {
      point = (Tp[0] > Tp[1]) ? 0 : 1;
      if (Tp[2] > Tp[point]) point = 2;
    }
    if (point >= 0) {
      shown_disjoint = 1;
      V = T2[point] - T1[0];
      Z = cross(Sn, Sv[0]);
      if (dot(V, Z) > 0) {
        V = T2[point] - T1[1];
        Z = cross(Sn, Sv[1]);
        if (dot(V, Z) > 0) {
          V = T2[point] - T1[2];
          Z = cross(Sn, Sv[2]);
          if (dot(V, Z) > 0) {
            P = T2[point] + Sn * (Tp[point] / Snl);
            Q = T2[point];
            return sqrt(sqnorm(P - Q));
          }
        }
      }
    }
  }
  const V3<S> Tn = cross(Tv[0], Tv[1]);
  const S Tnl = dot(Tn, Tn);
  if (Tnl > (S)1e-15) {
    S Sp[3];
    V = T2[0] - T1[0];
    Sp[0] = dot(V, Tn);
    V = T2[0] - T1[1];
    Sp[1] = dot(V, Tn);
    V = T2[0] - T1[2];
    Sp[2] = dot(V, Tn);
    int point = -1;
    if ((Sp[0] > 0) && (Sp[1] > 0) && (Sp[2] > 0)) {
      point = (Sp[0] < Sp[1]) ? 0 : 1;
      if (Sp[2] < Sp[point]) point = 2;
    } else if ((Sp[0] < 0) && (Sp[1] < 0) && (Sp[2] < 0)) {
      point = (Sp[0] > Sp[1]) ? 0 : 1;
      if (Sp[2] > Sp[point]) point = 2;
    }
    if (point >= 0) {
      shown_disjoint = 1;
      V = T1[point] - T2[0];
      Z = cross(Tn, Tv[0]);
      if (dot(V, Z) > 0) {
        V = T1[point] - T2[1];
        Z = cross(Tn, Tv[1]);
        if (dot(V, Z) > 0) {
          V = T1[point] - T2[2];
          Z = cross(Tn, Tv[2]);
          if (dot(V, Z) > 0) {
            P = T1[point];
            Q = T1[point] + Tn * (Sp[point] / Tnl);
            return sqrt(sqnorm(P - Q));
          }
        }
      }
    }
  }
  if (shown_disjoint) {
    P = minP;
    Q = minQ;
    return sqrt(mindd);
  }
  return 0;
}

// OBB::size() of node b (OBB-inl.h:205-209, extent.squaredNorm(), stored in FP64) as the
// bit pattern of the non-negative double: the integer order equals the FP64 order, so
// firstOverSecond's comparison runs on the integer pipes instead of the 1/64-rate FP64
// pipe.
FCLG_HD long long size_key(const DevMesh& m, int b) {
#if defined(__CUDA_ARCH__)
  return __ldg(reinterpret_cast<const long long*>(m.size64) + b);
#else
  long long k;
  memcpy(&k, m.size64 + b, sizeof(k));
  return k;
#endif
}

}  // namespace fclgpu
