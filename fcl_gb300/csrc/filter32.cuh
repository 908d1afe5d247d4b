// FP32 filtered predicates for the OBBRSS collide path.
//
// Each predicate evaluates FCL's FP64 test in FP32 together with a rigorous bound E
// on |margin_fp32 - margin_fp64| (margin = the difference the FP64 test compares
// with 0).  It returns CERTAIN_FALSE / CERTAIN_TRUE when |margin| > E settles the
// FP64 outcome, and UNCERTAIN otherwise; the caller then re-runs the exact FP64
// test.  Bounds are standard a-priori forward-error bounds (gamma_n = n u/(1-n u),
// u = 2^-24) plus the FP64 -> FP32 rounding of every input, with a 1.001 factor that
// absorbs the FP32 rounding of the bound itself and the (2^29 times smaller) error
// of the FP64 reference computation.  Derivations:
//
// OBB SAT (math/bv/OBB-inl.h:383-523).  R0 rotation, node axes orthonormal to 1e-12.
//   M = R0*A2:         |dM|  <= 5.1u
//   B = A1^T*M:        |dB|  <= 13u           (|B| <= 1.0003)
//   X = R0*To2+T0-To1: |dX|  <= 8.02u G,  G = C1 + 1.0001 C2 + sqrt3 tau
//   T = A1^T*X:        |dT|  <= 18u G -> eT = 20u G   (per query)
//   For all 15 axes, margin m = t - r with r >= 0 the right-hand side:
//   |dm| <= E0 + 5.1u r,  E0 = 2.01 eT + 16.1u Tn + 14.1u (sum a + sum b),
//   Tn = sum |T_i| + 3 eT.
//
// Triangle SAT (intersect-inl.h:727-798, 1085-1106).  Points are taken relative to
// P1 as in FCL.  P-side offsets P2-P1, P3-P1 are rounded from FP64 differences; the
// Q-side offset D = R0 Q1 + T0 - P1 is computed in float-float arithmetic (error
// <= u|D| + 32u^2 S, S = tau + V1 + sqrt3 V2 per query) and Q2, Q3 follow from
// R0 (Qk - Q1).  With l = max |coordinate| over all points and edge vectors:
//   every point/edge coordinate: |d| <= delta = 26u l + 32u^2 S + 32*2^-53 S
//   degree-2 axes (normals, edge x edge): |dax| <= e2 = 4 l delta + 2 delta^2 + 6u l^2,
//                                         |ax| <= L2 = 2 l^2 + e2
//   degree-3 axes (edge x normal):        |dax| <= e3 = 2(delta L2 + l e2 + delta e2) + 6u l L2,
//                                         |ax| <= L3 = 4 l^3 + e3
//   projection: |d(ax.v)| <= 3(eax l + Lax delta + eax delta) + 9.03u Lax l
//   margins mn1-mx2, mn2-mx1: E = 2.002 * projection bound.
#pragma once
#include <cuda_runtime.h>

#include "geom.cuh"

namespace fclgpu {

enum : int { F_FALSE = 0, F_TRUE = 1, F_UNSURE = 2 };

#define FCLG_U32 5.9604645e-08f  // 2^-24

// Per-query FP32 state for the collide traversal.
struct QueryF32 {
  float R[9];   // fl32(R0)
  float Rl[9];  // fl32(R0 - fl32(R0))
  float T[3];
  float Tl[3];
  float eT;     // 20u G (OBB tests)
  float dabs;   // 32u^2 S + 32*2^-53 S (leaf tests)
};

FCLG_HD void make_query_f32(const M3<double>& R, const V3<double>& T, double C1, double C2,
                                               double V1, double V2, QueryF32& q) {
#pragma unroll
  for (int i = 0; i < 9; ++i) {
    q.R[i] = (float)R.m[i];
    q.Rl[i] = (float)(R.m[i] - (double)q.R[i]);
  }
  const double tt[3] = {T.x, T.y, T.z};
  double tau = 0.0;
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    q.T[i] = (float)tt[i];
    q.Tl[i] = (float)(tt[i] - (double)q.T[i]);
    tau = fmax(tau, fabs(tt[i]));
  }
  const double G = C1 + 1.0001 * C2 + 1.7320509 * tau;
  q.eT = (float)(20.0 * 5.9604645e-08 * G * 1.001);
  const double S = tau + V1 + 1.7320509 * V2;
  q.dabs = (float)((32.0 * 5.9604645e-08 * 5.9604645e-08 + 32.0 * 1.1102230246251565e-16) * S * 1.001);
}

// ---------------------------------------------------------------------------------
// OBB SAT in FP32.  n1, n2: 4 float4 per node (axis col k + To[k]; extent + child).
// Returns F_FALSE (disjoint), F_TRUE (overlap) or F_UNSURE.
// ---------------------------------------------------------------------------------
FCLG_HD int obb_overlap_f32(const QueryF32& q, const float4 a0, const float4 a1,
                                               const float4 a2, const float4 ea, const float4 b0,
                                               const float4 b1, const float4 b2, const float4 eb) {
  const float* R = q.R;
  // M = R0 * A2 (columns of A2 are b0.xyz, b1.xyz, b2.xyz)
  float M[3][3];
  {
    const float4 bc[3] = {b0, b1, b2};
#pragma unroll
    for (int c = 0; c < 3; ++c)
#pragma unroll
      for (int r = 0; r < 3; ++r) M[r][c] = fmaf(R[3 * r], bc[c].x, fmaf(R[3 * r + 1], bc[c].y, R[3 * r + 2] * bc[c].z));
  }
  // B = A1^T * M: B[i][j] = (col i of A1) . (col j of M)
  float B[3][3];
  {
    const float4 ac[3] = {a0, a1, a2};
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) B[i][j] = fmaf(ac[i].x, M[0][j], fmaf(ac[i].y, M[1][j], ac[i].z * M[2][j]));
  }
  // X = R0*To2 + T0 - To1 ; T = A1^T X
  float X[3];
  {
    const float To1[3] = {a0.w, a1.w, a2.w};
#pragma unroll
    for (int r = 0; r < 3; ++r)
      X[r] = fmaf(R[3 * r], b0.w, fmaf(R[3 * r + 1], b1.w, fmaf(R[3 * r + 2], b2.w, q.T[r] - To1[r])));
  }
  float T[3];
  T[0] = fmaf(a0.x, X[0], fmaf(a0.y, X[1], a0.z * X[2]));
  T[1] = fmaf(a1.x, X[0], fmaf(a1.y, X[1], a1.z * X[2]));
  T[2] = fmaf(a2.x, X[0], fmaf(a2.y, X[1], a2.z * X[2]));

  const float a[3] = {ea.x, ea.y, ea.z};
  const float b[3] = {eb.x, eb.y, eb.z};
  float Bf[3][3];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) Bf[i][j] = fabsf(B[i][j]) + 1e-6f;

  const float eT = q.eT;
  const float Tn = fabsf(T[0]) + fabsf(T[1]) + fabsf(T[2]) + 3.f * eT;
  const float E0 = 2.01f * eT + (16.1f * FCLG_U32) * Tn + (14.1f * FCLG_U32) * ((a[0] + a[1] + a[2]) + (b[0] + b[1] + b[2]));
  const float kr = 5.1f * FCLG_U32;
  bool unsure = false;
#define FCLG_AXIS(tval, rval)                                  \
  {                                                            \
    const float t_ = (tval), r_ = (rval);                      \
    const float m_ = t_ - r_;                                  \
    const float E_ = fmaf(kr, r_, E0) * 1.001f;                \
    if (m_ > E_) return F_FALSE;                               \
    unsure |= (m_ >= -E_);                                     \
  }
  FCLG_AXIS(fabsf(T[0]), a[0] + fmaf(Bf[0][0], b[0], fmaf(Bf[0][1], b[1], Bf[0][2] * b[2])));
  FCLG_AXIS(fabsf(fmaf(B[0][0], T[0], fmaf(B[1][0], T[1], B[2][0] * T[2]))),
            b[0] + fmaf(Bf[0][0], a[0], fmaf(Bf[1][0], a[1], Bf[2][0] * a[2])));
  FCLG_AXIS(fabsf(T[1]), a[1] + fmaf(Bf[1][0], b[0], fmaf(Bf[1][1], b[1], Bf[1][2] * b[2])));
  FCLG_AXIS(fabsf(T[2]), a[2] + fmaf(Bf[2][0], b[0], fmaf(Bf[2][1], b[1], Bf[2][2] * b[2])));
  FCLG_AXIS(fabsf(fmaf(B[0][1], T[0], fmaf(B[1][1], T[1], B[2][1] * T[2]))),
            b[1] + fmaf(Bf[0][1], a[0], fmaf(Bf[1][1], a[1], Bf[2][1] * a[2])));
  FCLG_AXIS(fabsf(fmaf(B[0][2], T[0], fmaf(B[1][2], T[1], B[2][2] * T[2]))),
            b[2] + fmaf(Bf[0][2], a[0], fmaf(Bf[1][2], a[1], Bf[2][2] * a[2])));
  // edge x edge axes
  FCLG_AXIS(fabsf(fmaf(T[2], B[1][0], -T[1] * B[2][0])),
            fmaf(a[1], Bf[2][0], fmaf(a[2], Bf[1][0], fmaf(b[1], Bf[0][2], b[2] * Bf[0][1]))));
  FCLG_AXIS(fabsf(fmaf(T[2], B[1][1], -T[1] * B[2][1])),
            fmaf(a[1], Bf[2][1], fmaf(a[2], Bf[1][1], fmaf(b[0], Bf[0][2], b[2] * Bf[0][0]))));
  FCLG_AXIS(fabsf(fmaf(T[2], B[1][2], -T[1] * B[2][2])),
            fmaf(a[1], Bf[2][2], fmaf(a[2], Bf[1][2], fmaf(b[0], Bf[0][1], b[1] * Bf[0][0]))));
  FCLG_AXIS(fabsf(fmaf(T[0], B[2][0], -T[2] * B[0][0])),
            fmaf(a[0], Bf[2][0], fmaf(a[2], Bf[0][0], fmaf(b[1], Bf[1][2], b[2] * Bf[1][1]))));
  FCLG_AXIS(fabsf(fmaf(T[0], B[2][1], -T[2] * B[0][1])),
            fmaf(a[0], Bf[2][1], fmaf(a[2], Bf[0][1], fmaf(b[0], Bf[1][2], b[2] * Bf[1][0]))));
  FCLG_AXIS(fabsf(fmaf(T[0], B[2][2], -T[2] * B[0][2])),
            fmaf(a[0], Bf[2][2], fmaf(a[2], Bf[0][2], fmaf(b[0], Bf[1][1], b[1] * Bf[1][0]))));
  FCLG_AXIS(fabsf(fmaf(T[1], B[0][0], -T[0] * B[1][0])),
            fmaf(a[0], Bf[1][0], fmaf(a[1], Bf[0][0], fmaf(b[1], Bf[2][2], b[2] * Bf[2][1]))));
  FCLG_AXIS(fabsf(fmaf(T[1], B[0][1], -T[0] * B[1][1])),
            fmaf(a[0], Bf[1][1], fmaf(a[1], Bf[0][1], fmaf(b[0], Bf[2][2], b[2] * Bf[2][0]))));
  FCLG_AXIS(fabsf(fmaf(T[1], B[0][2], -T[0] * B[1][2])),
            fmaf(a[0], Bf[1][2], fmaf(a[1], Bf[0][2], fmaf(b[0], Bf[2][1], b[1] * Bf[2][0]))));
#undef FCLG_AXIS
  return unsure ? F_UNSURE : F_TRUE;
}

// ---------------------------------------------------------------------------------
// Triangle-triangle SAT in FP32.  t1, t2: 3 float4 per triangle (P1 hi, P1 lo, P2-P1,
// P3-P1).  Returns F_FALSE (disjoint), F_TRUE (intersecting) or F_UNSURE.
// ---------------------------------------------------------------------------------
FCLG_HD void two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

struct F3 {
  float x, y, z;
};
FCLG_HD F3 f3(float a, float b, float c) { return F3{a, b, c}; }
FCLG_HD F3 sub3(const F3& a, const F3& b) { return f3(a.x - b.x, a.y - b.y, a.z - b.z); }
FCLG_HD F3 add3(const F3& a, const F3& b) { return f3(a.x + b.x, a.y + b.y, a.z + b.z); }
FCLG_HD float dot3(const F3& a, const F3& b) { return fmaf(a.x, b.x, fmaf(a.y, b.y, a.z * b.z)); }
FCLG_HD F3 cross3(const F3& a, const F3& b) {
  return f3(fmaf(a.y, b.z, -a.z * b.y), fmaf(a.z, b.x, -a.x * b.z), fmaf(a.x, b.y, -a.y * b.x));
}
FCLG_HD float amax3(const F3& a) { return fmaxf(fabsf(a.x), fmaxf(fabsf(a.y), fabsf(a.z))); }
FCLG_HD F3 rot3(const float* R, const F3& v) {
  return f3(fmaf(R[0], v.x, fmaf(R[1], v.y, R[2] * v.z)), fmaf(R[3], v.x, fmaf(R[4], v.y, R[5] * v.z)),
            fmaf(R[6], v.x, fmaf(R[7], v.y, R[8] * v.z)));
}

// One separating-axis check with bound E.  Returns true if the axis certainly
// separates; sets unsure if it neither certainly separates nor certainly does not.
FCLG_HD bool sat_axis(const F3& ax, const F3& p2, const F3& p3, const F3& q1, const F3& q2,
                                         const F3& q3, float E, bool& unsure) {
  const float P2 = dot3(ax, p2), P3 = dot3(ax, p3);
  const float Q1 = dot3(ax, q1), Q2 = dot3(ax, q2), Q3 = dot3(ax, q3);
  const float mn1 = fminf(0.f, fminf(P2, P3)), mx1 = fmaxf(0.f, fmaxf(P2, P3));
  const float mn2 = fminf(Q1, fminf(Q2, Q3)), mx2 = fmaxf(Q1, fmaxf(Q2, Q3));
  const float s1 = mn1 - mx2, s2 = mn2 - mx1;
  if (s1 > E || s2 > E) return true;
  unsure |= (s1 >= -E) || (s2 >= -E);
  return false;
}

FCLG_HD int tri_intersect_f32(const QueryF32& q, const float4 x0, const float4 x1,
                                                 const float4 x2, const float4 y0, const float4 y1,
                                                 const float4 y2) {
  // triangle 1: P1 = hi + lo, p2 = P2 - P1, p3 = P3 - P1
  const F3 Ph = f3(x0.x, x0.y, x0.z), Pl = f3(x0.w, x1.x, x1.y);
  const F3 p2 = f3(x1.z, x1.w, x2.x), p3 = f3(x2.y, x2.z, x2.w);
  // triangle 2: Q1 = hi + lo, dQ2, dQ3
  const float Qh[3] = {y0.x, y0.y, y0.z}, Ql[3] = {y0.w, y1.x, y1.y};
  const F3 dQ2 = f3(y1.z, y1.w, y2.x), dQ3 = f3(y2.y, y2.z, y2.w);
  // D = R0 Q1 + T0 - P1 in float-float
  float D[3];
  {
    const float Pha[3] = {Ph.x, Ph.y, Ph.z}, Pla[3] = {Pl.x, Pl.y, Pl.z};
#pragma unroll
    for (int r = 0; r < 3; ++r) {
      float hi, lo;
      two_sum(q.T[r], -Pha[r], hi, lo);
      lo += q.Tl[r] - Pla[r];
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const float Rh = q.R[3 * r + k], Rlo = q.Rl[3 * r + k];
        const float p = Rh * Qh[k];
        const float pe = fmaf(Rh, Qh[k], -p) + fmaf(Rh, Ql[k], Rlo * Qh[k]);
        float s, e;
        two_sum(hi, p, s, e);
        hi = s;
        lo += e + pe;
      }
      D[r] = hi + lo;
    }
  }
  const F3 q1 = f3(D[0], D[1], D[2]);
  const F3 f1 = rot3(q.R, dQ2);                 // q2 - q1
  const F3 g3 = rot3(q.R, dQ3);                 // q3 - q1
  const F3 f2 = rot3(q.R, sub3(dQ3, dQ2));      // q3 - q2
  const F3 f3v = f3(-g3.x, -g3.y, -g3.z);       // q1 - q3
  const F3 q2 = add3(q1, f1), q3 = add3(q1, g3);
  const F3 e1 = p2, e2 = sub3(p3, p2), e3 = f3(-p3.x, -p3.y, -p3.z);

  float l = fmaxf(fmaxf(amax3(p2), amax3(p3)), fmaxf(amax3(q1), fmaxf(amax3(q2), amax3(q3))));
  l = fmaxf(l, fmaxf(amax3(e2), fmaxf(amax3(f1), fmaxf(amax3(f2), amax3(g3)))));
  l *= 1.0001f;
  const float u = FCLG_U32;
  const float delta = fmaf(26.f * u, l, q.dabs);
  const float e2b = fmaf(4.f * l, delta, fmaf(2.f * delta, delta, 6.f * u * l * l));
  const float L2 = fmaf(2.f * l, l, e2b);
  const float e3b = 2.f * (delta * L2 + l * e2b + delta * e2b) + 6.f * u * l * L2;
  const float L3 = fmaf(4.f * l * l, l, e3b);
  const float E2 = 2.002f * (3.f * (e2b * l + L2 * delta + e2b * delta) + 9.03f * u * L2 * l);
  const float E3 = 2.002f * (3.f * (e3b * l + L3 * delta + e3b * delta) + 9.03f * u * L3 * l);

  bool unsure = false;
  const F3 n1 = cross3(e1, e2);
  if (sat_axis(n1, p2, p3, q1, q2, q3, E2, unsure)) return F_FALSE;
  const F3 m1 = cross3(f1, f2);
  if (sat_axis(m1, p2, p3, q1, q2, q3, E2, unsure)) return F_FALSE;
  if (sat_axis(cross3(e1, f1), p2, p3, q1, q2, q3, E2, unsure)) return F_FALSE;
  if (sat_axis(cross3(e1, f2), p2, p3, q1, q2, q3, E2, unsure)) return F_FALSE;
  if (sat_axis(cross3(e1, f3v), p2, p3, q1, q2, q3, E2, unsure)) return F_FALSE;
  if (sat_axis(cross3(e2, f1), p2, p3, q1, q2, q3, E2, unsure)) return F_FALSE;
  if (sat_axis(cross3(e2, f2), p2, p3, q1, q2, q3, E2, unsure)) return F_FALSE;
  if (sat_axis(cross3(e2, f3v), p2, p3, q1, q2, q3, E2, unsure)) return F_FALSE;
  if (sat_axis(cross3(e3, f1), p2, p3, q1, q2, q3, E2, unsure)) return F_FALSE;
  if (sat_axis(cross3(e3, f2), p2, p3, q1, q2, q3, E2, unsure)) return F_FALSE;
  if (sat_axis(cross3(e3, f3v), p2, p3, q1, q2, q3, E2, unsure)) return F_FALSE;
  if (sat_axis(cross3(e1, n1), p2, p3, q1, q2, q3, E3, unsure)) return F_FALSE;
  if (sat_axis(cross3(e2, n1), p2, p3, q1, q2, q3, E3, unsure)) return F_FALSE;
  if (sat_axis(cross3(e3, n1), p2, p3, q1, q2, q3, E3, unsure)) return F_FALSE;
  if (sat_axis(cross3(f1, m1), p2, p3, q1, q2, q3, E3, unsure)) return F_FALSE;
  if (sat_axis(cross3(f2, m1), p2, p3, q1, q2, q3, E3, unsure)) return F_FALSE;
  if (sat_axis(cross3(f3v, m1), p2, p3, q1, q2, q3, E3, unsure)) return F_FALSE;
  return unsure ? F_UNSURE : F_TRUE;
}

}  // namespace fclgpu
