// Certified FP32 distance traversal for BVHModel<OBBRSS> pairs (host and device).
//
// FCL's distance traversal (traversal_recurse-inl.h:257-316) prunes a BV pair when
// its RSS distance (RSS-inl.h:1956-1974, rectDistance :512-1224) is not below the
// best distance so far, and updates the best with DistanceResult's strict "<"
// (distance_result-inl.h:84-105).  rectDistance picks one of many branches (edge-pair
// Voronoi tests, then plane separations); an FP32 evaluation can take another branch
// than the FP64 one, so its error has no useful a-priori bound.  This traversal does
// not evaluate it.  It prunes with a different lower bound that has one:
//
//   for every direction n != 0 and convex sets X, Y:
//       dist(X, Y) >= (min_{y in Y} n.y - max_{x in X} n.x) / |n|.
//
// The support function of an RSS (rectangle To + s a0 + t a1, s in [0,l0], t in
// [0,l1], swept by a ball of radius r) is n.To + l0 max(0, n.a0) + l1 max(0, n.a1)
// + r|n|, and B's volumes are moved by (R0, T0): min over B = m.To + n.T0 +
// l0 min(0, m.a0) + l1 min(0, m.a1) - r|m| with m = R0^T n.  The bound holds for any
// direction, so the direction only affects how tight it is.  The traversal uses the
// direction between the witness points of the best pair found so far (initially the
// direction between the two root boxes' centres); near the minimum this is the
// separating direction and the bound is close to the RSS distance itself.
//
// Forward error of the FP32 evaluation (u = 2^-24; inputs are the FP64 node data
// rounded to FP32; n is an exact FP32 vector of norm 1 +- 2u; m and n.T0 are the
// FP64 values R0^T n, n.T0 rounded to FP32; |To| <= rmax of its mesh):
//   A side  n.To + l0 max(0,n.a0) + l1 max(0,n.a1) + r:
//           <= 7.1u rmaxA + 9.2u (l0 + l1) + 5.1u r
//   B side  m.To + n.T0 + l0 min(0,m.a0) + l1 min(0,m.a1) - r:
//           <= 9.2u rmaxB + 5.1u |n.T0| + 11.3u (l0 + l1) + 6.2u r
//   (3-term FMA dot products err by gamma_3 times the sum of |terms|, bounded by
//   Cauchy-Schwarz with |n|, |m| <= 1 + 3u and unit-length axes; the radius term
//   carries |n| - 1 and |R0^T n| - |n| <= 1e-9 for the checked rotations.)
//   difference: + u (|A side| + |B side|).
//   Together E <= 12.5u (rmaxA + rmaxB + |n.T0| + l0A + l1A + rA + l0B + l1B + rB),
//   used with a factor 1.01 that covers the rounding of E itself.  The certified
//   lower bound is L = (gap - E)(1 - 8u) (the factor covers the division by |n| and
//   the two roundings).
//   Triangles along n (P1 in FP32, P2-P1 and P3-P1 rounded from FP64 differences,
//   |coordinates| <= vmax): E_tri <= 40u (vmaxA + vmaxB + |n.T0|).
//   Triangles along their own FP32 witness direction w (points relative to P1, every
//   coordinate within delta of the exact one, delta as in filter32.cuh):
//   E_w <= |w|_1 (2 delta + 8.1u l), L_w = (gap_w - E_w)(1 - 8u) / |w|.
//
// So every pruned BV pair and every skipped triangle pair is, in exact arithmetic,
// farther apart than L > best.  Two FP64 effects are covered by a margin
// m64 = 2^-36 S (S = the query's coordinate scale): FCL's FP64 RSS fit contains its
// triangles up to rounding, and FCL's FP64 triDistance is within rounding of the
// exact distance.  For the second, the traversal also evaluates in FP64 every pair
// whose certified bound is below 2^-6 of the pair's triangle size, where triDistance
// switches to its overlap branch.  Hence a pair that is skipped can never pass
// DistanceResult's strict "<" test, and the reported distance is the smallest FP64
// triDistance over all triangle pairs, its triangle ids and witness points those of
// the first such pair in this traversal's order.  FCL's own result is the same pair
// unless several pairs tie exactly in FP64 (shared vertices), where the first in
// FCL's visit order wins; FCL reports the same distance and, at a shared vertex, the
// same witness points.
#pragma once
#include <string.h>

#include "filter32.cuh"
#include "geom.cuh"
#include "kernels.h"

#if defined(__CUDACC__)
#define FCLG_NOINLINE __host__ __device__ __noinline__
#else
#define FCLG_NOINLINE __attribute__((noinline))
#endif

namespace fclgpu {

FCLG_HD int f2i_hd(float x) {
#if defined(__CUDA_ARCH__)
  return __float_as_int(x);
#else
  int i;
  memcpy(&i, &x, 4);
  return i;
#endif
}

template <class T>
FCLG_HD T ldro(const T* p) {
#if defined(__CUDA_ARCH__)
  return __ldg(p);
#else
  return *p;
#endif
}
FCLG_HD float rsqrt_hd(float x) {
#if defined(__CUDA_ARCH__)
  return rsqrtf(x);  // at most 2 ulp from 1/sqrt(x)
#else
  return 1.f / sqrtf(x);
#endif
}
FCLG_HD float4 ld4(const void* base, long long i) { return ldro(reinterpret_cast<const float4*>(base) + i); }

struct DistOut {
  double d;
  int id1, id2;
  V3<double> P, Q;  // first mesh's frame
  long long nbv, nleaf, nrc;
  unsigned status;
};

// Exact FP64 triangle distance of triangle p1 (mesh A) and p2 (mesh B moved by R,T);
// points in A's frame (triangle_distance-inl.h:425-436).
FCLG_NOINLINE double leaf_distance64_hd(const DevMesh& A, const DevMesh& B, int p1, int p2, const M3<double>& R,
                                  const V3<double>& T, V3<double>& P, V3<double>& Q) {
  const int* ta = A.tris + 3 * (long long)p1;
  const int* tb = B.tris + 3 * (long long)p2;
  V3<double> T1[3], T2[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const double* pa = A.verts64 + 3 * (long long)ldro(ta + k);
    const double* pb = B.verts64 + 3 * (long long)ldro(tb + k);
    T1[k] = v3(ldro(pa), ldro(pa + 1), ldro(pa + 2));
    T2[k] = mulv(R, v3(ldro(pb), ldro(pb + 1), ldro(pb + 2))) + T;
  }
  return tri_distance<double>(T1, T2, P, Q);
}

// Search direction of one query and the error terms that depend on it.
struct DistDir {
  float n[3];  // A's frame, |n| = 1 +- 2u
  float m[3];  // fl32(R0^T n), B's frame
  float nT;    // fl32(n . T0)
  float Eq;    // RSS gap error, query part: 1.01 * 12.5u (rmaxA + rmaxB + |nT|)
  float Et;    // triangle gap error: 1.01 * 40u (vmaxA + vmaxB + |nT|)
};

// Sets the direction to (x, y, z) normalised (FP64, then rounded); false when the
// vector has no usable length (the direction is then left unchanged).
FCLG_HD bool set_dist_dir(const DevMesh& A, const DevMesh& B, const M3<double>& R, const V3<double>& T, double x,
                          double y, double z, DistDir& d) {
  const double s2 = (x * x + y * y) + z * z;
  if (!(s2 > 1e-200) || !(s2 < 1e200)) return false;
  const double is = 1.0 / sqrt(s2);
  d.n[0] = (float)(x * is);
  d.n[1] = (float)(y * is);
  d.n[2] = (float)(z * is);
  const double n0 = d.n[0], n1 = d.n[1], n2 = d.n[2];
  d.m[0] = (float)((R(0, 0) * n0 + R(1, 0) * n1) + R(2, 0) * n2);
  d.m[1] = (float)((R(0, 1) * n0 + R(1, 1) * n1) + R(2, 1) * n2);
  d.m[2] = (float)((R(0, 2) * n0 + R(1, 2) * n1) + R(2, 2) * n2);
  const double nt = (n0 * T.x + n1 * T.y) + n2 * T.z;
  d.nT = (float)nt;
  const double u = 5.9604644775390625e-08;
  d.Eq = (float)(1.01 * 12.5 * u * ((A.rmax + B.rmax) + fabs(nt)) + 1e-30);
  d.Et = (float)(1.01 * 40.0 * u * ((A.vmax + B.vmax) + fabs(nt)) + 1e-30);
  return true;
}

// Certified lower bound of the distance between the two RSS from their supports.
FCLG_HD float rss_gap_bound(float lo_b, float hi_a, float sz_a, float sz_b, const DistDir& d) {
  const float E = fmaf(1.01f * 12.5f * FCLG_U32, sz_a + sz_b, d.Eq);
  return ((lo_b - hi_a) - E) * (1.f - 8.f * FCLG_U32);
}

struct RssF {
  float4 o, l, c0, c1;  // (To, r), (l0, l1, -, -), first two axis columns
};
FCLG_HD RssF load_rss(const DevMesh& M, int b) {
  RssF r;
  r.o = ld4(M.rss32, 5 * (long long)b);
  r.l = ld4(M.rss32, 5 * (long long)b + 1);
  r.c0 = ld4(M.rss32, 5 * (long long)b + 2);
  r.c1 = ld4(M.rss32, 5 * (long long)b + 3);
  return r;
}

// Certified lower bound of the distance of two RSS: the larger of the gaps along
// the query direction n and along the pair's own centre-to-centre direction c.
// For c (normalised in FP32, |c| = 1 +- 8u; m_c = R0^T c and c.T0 evaluated in FP32
// from fl32(R0), fl32(T0), so each carries 4.1u |c|_1 more):
//   E_c <= 20u (rmaxA + rmaxB) + 14u tau + 20u (l0A + l1A + rA + l0B + l1B + rB),
// tau = max |T0_i|, with the factor 1.01, and L_c = (gap_c - E_c)(1 - 14u).
FCLG_HD float rss_pair_bound(const RssF& a, const RssF& b, const DistDir& d, const QueryF32& q, float Ec0) {
  const float sa = (a.l.x + a.l.y) + a.o.w, sb = (b.l.x + b.l.y) + b.o.w;
  // along n
  float Ln;
  {
    const float p0 = fmaf(d.n[0], a.c0.x, fmaf(d.n[1], a.c0.y, d.n[2] * a.c0.z));
    const float p1 = fmaf(d.n[0], a.c1.x, fmaf(d.n[1], a.c1.y, d.n[2] * a.c1.z));
    const float hi = fmaf(d.n[0], a.o.x, fmaf(d.n[1], a.o.y, d.n[2] * a.o.z)) +
                     fmaf(a.l.x, fmaxf(p0, 0.f), fmaf(a.l.y, fmaxf(p1, 0.f), a.o.w));
    const float q0 = fmaf(d.m[0], b.c0.x, fmaf(d.m[1], b.c0.y, d.m[2] * b.c0.z));
    const float q1 = fmaf(d.m[0], b.c1.x, fmaf(d.m[1], b.c1.y, d.m[2] * b.c1.z));
    const float lo = (fmaf(d.m[0], b.o.x, fmaf(d.m[1], b.o.y, d.m[2] * b.o.z)) + d.nT) +
                     fmaf(b.l.x, fminf(q0, 0.f), fmaf(b.l.y, fminf(q1, 0.f), -b.o.w));
    Ln = rss_gap_bound(lo, hi, sa, sb, d);
  }
  // along the centre-to-centre direction
  float Lc;
  {
    const float ha0 = 0.5f * a.l.x, ha1 = 0.5f * a.l.y, hb0 = 0.5f * b.l.x, hb1 = 0.5f * b.l.y;
    const F3 ca = f3(fmaf(ha0, a.c0.x, fmaf(ha1, a.c1.x, a.o.x)), fmaf(ha0, a.c0.y, fmaf(ha1, a.c1.y, a.o.y)),
                     fmaf(ha0, a.c0.z, fmaf(ha1, a.c1.z, a.o.z)));
    const F3 cbl = f3(fmaf(hb0, b.c0.x, fmaf(hb1, b.c1.x, b.o.x)), fmaf(hb0, b.c0.y, fmaf(hb1, b.c1.y, b.o.y)),
                      fmaf(hb0, b.c0.z, fmaf(hb1, b.c1.z, b.o.z)));
    const F3 cb = rot3(q.R, cbl);
    F3 c = f3((cb.x + q.T[0]) - ca.x, (cb.y + q.T[1]) - ca.y, (cb.z + q.T[2]) - ca.z);
    const float c2 = dot3(c, c);
    const float ic = c2 > 1e-30f ? rsqrt_hd(c2) : 0.f;
    c = f3(c.x * ic, c.y * ic, c.z * ic);
    const F3 mc = f3(fmaf(q.R[0], c.x, fmaf(q.R[3], c.y, q.R[6] * c.z)), fmaf(q.R[1], c.x, fmaf(q.R[4], c.y, q.R[7] * c.z)),
                     fmaf(q.R[2], c.x, fmaf(q.R[5], c.y, q.R[8] * c.z)));
    const float p0 = dot3(c, f3(a.c0.x, a.c0.y, a.c0.z)), p1 = dot3(c, f3(a.c1.x, a.c1.y, a.c1.z));
    const float hi = dot3(c, f3(a.o.x, a.o.y, a.o.z)) + fmaf(a.l.x, fmaxf(p0, 0.f), fmaf(a.l.y, fmaxf(p1, 0.f), a.o.w));
    const float q0 = dot3(mc, f3(b.c0.x, b.c0.y, b.c0.z)), q1 = dot3(mc, f3(b.c1.x, b.c1.y, b.c1.z));
    const float cT = dot3(c, f3(q.T[0], q.T[1], q.T[2]));
    const float lo = (dot3(mc, f3(b.o.x, b.o.y, b.o.z)) + cT) +
                     fmaf(b.l.x, fminf(q0, 0.f), fmaf(b.l.y, fminf(q1, 0.f), -b.o.w));
    const float E = fmaf(1.01f * 20.f * FCLG_U32, sa + sb, Ec0);
    Lc = ic > 0.f ? ((lo - hi) - E) * (1.f - 14.f * FCLG_U32) : -1.f;
  }
  return fmaxf(Ln, Lc);
}

// Certified lower bound of the distance of triangle p1 (A) and p2 (B moved) along n;
// tsize = the larger triangle's largest edge-offset coordinate.
FCLG_HD float tri_gap_bound(const DevMesh& A, const DevMesh& B, int p1, int p2, const DistDir& d, float& tsize) {
  const float4 x0 = ld4(A.tri32, 3 * (long long)p1), x1 = ld4(A.tri32, 3 * (long long)p1 + 1),
               x2 = ld4(A.tri32, 3 * (long long)p1 + 2);
  const float4 y0 = ld4(B.tri32, 3 * (long long)p2), y1 = ld4(B.tri32, 3 * (long long)p2 + 1),
               y2 = ld4(B.tri32, 3 * (long long)p2 + 2);
  const float a1 = fmaf(d.n[0], x0.x, fmaf(d.n[1], x0.y, d.n[2] * x0.z));
  const float a2 = fmaf(d.n[0], x1.z, fmaf(d.n[1], x1.w, d.n[2] * x2.x));
  const float a3 = fmaf(d.n[0], x2.y, fmaf(d.n[1], x2.z, d.n[2] * x2.w));
  const float b1 = fmaf(d.m[0], y0.x, fmaf(d.m[1], y0.y, d.m[2] * y0.z));
  const float b2 = fmaf(d.m[0], y1.z, fmaf(d.m[1], y1.w, d.m[2] * y2.x));
  const float b3 = fmaf(d.m[0], y2.y, fmaf(d.m[1], y2.z, d.m[2] * y2.w));
  const float hA = a1 + fmaxf(0.f, fmaxf(a2, a3));
  const float gB = (b1 + d.nT) + fminf(0.f, fminf(b2, b3));
  tsize = fmaxf(fmaxf(fmaxf(fabsf(x1.z), fabsf(x1.w)), fmaxf(fabsf(x2.x), fabsf(x2.y))),
                fmaxf(fmaxf(fabsf(x2.z), fabsf(x2.w)), fmaxf(fmaxf(fabsf(y1.z), fabsf(y1.w)),
                                                            fmaxf(fmaxf(fabsf(y2.x), fabsf(y2.y)),
                                                                  fmaxf(fabsf(y2.z), fabsf(y2.w))))));
  return ((gB - hA) - d.Et) * (1.f - 8.f * FCLG_U32);
}

// FP32 triangle distance with a certified lower bound along its own witness
// direction.  Points relative to triangle 1's first vertex (the Q offset in
// float-float, as the collide filter does); returns L_w, sets w = Q - P and l.
FCLG_NOINLINE float tri_witness_bound(const QueryF32& q, const DevMesh& A, const DevMesh& B, int t1, int t2, float* w,
                                float& l_out) {
  const float4 x0 = ld4(A.tri32, 3 * (long long)t1), x1 = ld4(A.tri32, 3 * (long long)t1 + 1),
               x2 = ld4(A.tri32, 3 * (long long)t1 + 2);
  const float4 y0 = ld4(B.tri32, 3 * (long long)t2), y1 = ld4(B.tri32, 3 * (long long)t2 + 1),
               y2 = ld4(B.tri32, 3 * (long long)t2 + 2);
  const float Ph[3] = {x0.x, x0.y, x0.z}, Pl[3] = {x0.w, x1.x, x1.y};
  const float Qh[3] = {y0.x, y0.y, y0.z}, Ql[3] = {y0.w, y1.x, y1.y};
  float D[3];
#pragma unroll
  for (int r = 0; r < 3; ++r) {
    float hi, lo;
    two_sum(q.T[r], -Ph[r], hi, lo);
    lo += q.Tl[r] - Pl[r];
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
  const F3 q1 = f3(D[0], D[1], D[2]);
  const F3 f1 = rot3(q.R, f3(y1.z, y1.w, y2.x));
  const F3 g3 = rot3(q.R, f3(y2.y, y2.z, y2.w));
  const F3 q2 = add3(q1, f1), q3 = add3(q1, g3);
  const F3 p2 = f3(x1.z, x1.w, x2.x), p3 = f3(x2.y, x2.z, x2.w);
  float l = fmaxf(fmaxf(amax3(p2), amax3(p3)), fmaxf(amax3(q1), fmaxf(amax3(q2), amax3(q3))));
  l = fmaxf(l, fmaxf(amax3(f1), amax3(g3))) * 1.0001f;
  l_out = l;
  V3<float> T1[3], T2[3], P, Q;
  T1[0] = v3(0.f, 0.f, 0.f);
  T1[1] = v3(p2.x, p2.y, p2.z);
  T1[2] = v3(p3.x, p3.y, p3.z);
  T2[0] = v3(q1.x, q1.y, q1.z);
  T2[1] = v3(q2.x, q2.y, q2.z);
  T2[2] = v3(q3.x, q3.y, q3.z);
  tri_distance<float>(T1, T2, P, Q);
  const F3 wv = f3(Q.x - P.x, Q.y - P.y, Q.z - P.z);
  w[0] = wv.x;
  w[1] = wv.y;
  w[2] = wv.z;
  const float gq = fminf(dot3(wv, q1), fminf(dot3(wv, q2), dot3(wv, q3)));
  const float hp = fmaxf(0.f, fmaxf(dot3(wv, p2), dot3(wv, p3)));
  const float delta = fmaf(26.f * FCLG_U32, l, q.dabs);
  const float w1 = fabsf(wv.x) + fabsf(wv.y) + fabsf(wv.z);
  const float E = 1.01f * w1 * fmaf(2.f, delta, 8.1f * FCLG_U32 * l);
  const float nw = sqrtf(dot3(wv, wv));
  return ((gq - hp) - E) * (1.f - 8.f * FCLG_U32) / nw;  // NaN or -inf when w = 0: never skips
}

// FP64 support gap of triangle p1 (A) and p2 (B moved by R0, T0) along the FP32
// witness direction w, then along the direction between the two supporting
// vertices u (A) and v (B) it selects.  Returns a certified lower bound of the
// exact distance; sets u, v and vv = true when the gap along v - u proves that the
// pair's distance is |v - u| itself (a vertex-vertex configuration, the usual
// closest features of two tessellated convex surfaces).  Forward error (u64 = 2^-53;
// B's vertices moved in FP64 with 3-term sums, each coordinate within
// u64 (4.01 sqrt3 vmaxB + tau) of the exact one; 3-term dot products; one
// subtraction): below |w|_1 16 u64 (vmaxA + vmaxB + tau).
FCLG_NOINLINE double tri_gap64(const DevMesh& A, const DevMesh& B, int p1, int p2, const M3<double>& R,
                               const V3<double>& T, const float* w, double tau, V3<double>& u, V3<double>& v,
                               bool& vv) {
  const int* ta = A.tris + 3 * (long long)p1;
  const int* tb = B.tris + 3 * (long long)p2;
  V3<double> P[3], Q[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const double* pa = A.verts64 + 3 * (long long)ldro(ta + k);
    const double* pb = B.verts64 + 3 * (long long)ldro(tb + k);
    P[k] = v3(ldro(pa), ldro(pa + 1), ldro(pa + 2));
    Q[k] = mulv(R, v3(ldro(pb), ldro(pb + 1), ldro(pb + 2))) + T;
  }
  const double scale = (A.vmax + B.vmax) + tau;
  double best = -1.7976931348623157e308;
  vv = false;
#pragma unroll
  for (int pass = 0; pass < 2; ++pass) {
    const V3<double> d = pass == 0 ? v3((double)w[0], (double)w[1], (double)w[2]) : v - u;
    double hi = -1.7976931348623157e308, lo = 1.7976931348623157e308;
    int ih = 0, il = 0;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const double a = dot(d, P[k]), b = dot(d, Q[k]);
      if (a > hi) { hi = a; ih = k; }
      if (b < lo) { lo = b; il = k; }
    }
    const double d1 = (fabs(d.x) + fabs(d.y)) + fabs(d.z);
    const double E = d1 * 1.7763568394002505e-15 * scale;  // 16 u64
    const double nd = sqrt(sqnorm(d));
    if (!(nd > 0.0)) break;
    const double L = ((lo - hi) - E) / nd * (1.0 - 8.881784197001252e-16);
    best = L > best ? L : best;
    if (pass == 0) {
      u = P[ih];
      v = Q[il];
    } else {
      // |v - u| computed, rounded up; the gap along v - u proves the distance is |v - u|
      vv = L >= nd * (1.0 - 1.7763568394002505e-15) - 2.0 * E / nd;
    }
  }
  return best;
}

FCLG_HD bool same_point(const V3<double>& a, const V3<double>& b, double tol) {
  return fabs(a.x - b.x) <= tol && fabs(a.y - b.y) <= tol && fabs(a.z - b.z) <= tol;
}

struct DStackC {
  int b1, b2;
  float L;    // certified lower bound when pushed
  int epoch;  // direction it was computed with
};

// One query in the certified FP32 form as a resumable state machine.  init() sets the
// query up (false: it must run in the exact FP64 form instead -- a rotation that is
// not orthonormal to 1e-9, or a mesh whose bounds were refitted: FCL's merged volumes
// need not contain their triangles, so FCL's own result depends on its visit order
// and only its traversal reproduces it).  Then the query moves through phases:
//   TRAVERSE  visit one BV pair (bound both children, descend or pop), or reach a
//             triangle pair and run its cheap gap test along the query direction;
//   WITNESS   the triangle pair's FP32 distance, its certified bound along its own
//             witness direction and, near the best, the FP64 gap;
//   EXACT     FCL's FP64 triDistance and the strict "<" update;
//   DONE.
// A query's pairs are handled strictly in its own visit order; the GPU kernel only
// chooses which phase a warp runs next, so that lanes in the same phase execute
// together (the FP64 pipe of this GPU runs a warp instruction at the same cost
// whether one lane or 32 use it).
enum : int { DC_TRAVERSE = 0, DC_WITNESS = 1, DC_EXACT = 2, DC_DONE = 3 };

template <int STACK>
struct DistCert {
  const DevMesh* A;
  const DevMesh* B;
  M3<double> R;
  V3<double> T;
  QueryF32 qf;
  double tau, not_better, vtol;
  float m64, Ec0, best_up, tsize;
  DistDir dir;
  int epoch, sp, b1, b2, p1, p2, phase;
  DistOut o;
  DStackC stk[STACK];

  FCLG_HD bool init(const DevMesh* A_, const DevMesh* B_, const M3<double>& R_, const V3<double>& T_) {
    A = A_;
    B = B_;
    R = R_;
    T = T_;
    if (A->refitted || B->refitted) return false;
    double e = 0.0;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        const double g = (R(0, i) * R(0, j) + R(1, i) * R(1, j)) + R(2, i) * R(2, j);
        e = fmax(e, fabs(g - (i == j ? 1.0 : 0.0)));
      }
    if (!(e <= 1e-9)) return false;
    make_query_f32(R, T, A->rmax, B->rmax, A->vmax, B->vmax, qf);
    tau = fmax(fabs(T.x), fmax(fabs(T.y), fabs(T.z)));
    m64 = (float)(1.4551915228366852e-11 * ((tau + A->vmax) + 1.7320509 * B->vmax));  // 2^-36 S
    Ec0 = (float)(1.01 * 5.9604644775390625e-08 * (20.0 * (A->rmax + B->rmax) + 14.0 * tau) + 1e-30);
    vtol = 1.4210854715202004e-14 * ((tau + A->vmax) + 1.7320509 * B->vmax);  // 2^-46 S
    o.d = 1.7976931348623157e308;
    o.id1 = o.id2 = 0;
    o.P = o.Q = v3(0.0, 0.0, 0.0);
    o.nbv = o.nleaf = o.nrc = 0;
    o.status = 0;
    best_up = 3.0e38f;  // >= best + m64, as a float
    // a triangle pair whose certified lower bound exceeds best + m64 cannot pass the
    // strict "<" update: it is not evaluated in FP64
    not_better = 1.7976931348623157e308;
    // first direction: between the root boxes' centres
    const double* ca = A->nodes64[0].To;
    const double* cb = B->nodes64[0].To;
    const V3<double> c2 = mulv(R, v3(ldro(cb), ldro(cb + 1), ldro(cb + 2))) + T;
    if (!set_dist_dir(*A, *B, R, T, c2.x - ldro(ca), c2.y - ldro(ca + 1), c2.z - ldro(ca + 2), dir))
      set_dist_dir(*A, *B, R, T, 1.0, 0.0, 0.0, dir);
    epoch = 0;
    sp = 0;
    b1 = b2 = 0;
    phase = DC_TRAVERSE;
    return true;
  }

  // Next pair from the stack (phase TRAVERSE), or DONE when none is left.
  FCLG_HD void pop() {
    while (sp > 0) {
      const DStackC e = stk[--sp];
      if (e.L > best_up) continue;
      if (e.epoch != epoch) {  // the direction has changed since: re-bound with the new one
        if (rss_pair_bound(load_rss(*A, e.b1), load_rss(*B, e.b2), dir, qf, Ec0) > best_up) continue;
      }
      b1 = e.b1;
      b2 = e.b2;
      phase = DC_TRAVERSE;
      return;
    }
    phase = DC_DONE;
  }

  // TRAVERSE: one BV pair, or a triangle pair's gap test along the query direction.
  FCLG_HD void traverse() {
    const int c1 = f2i_hd(ld4(A->nodes32, 4 * (long long)b1 + 3).w);
    const int c2 = f2i_hd(ld4(B->nodes32, 4 * (long long)b2 + 3).w);
    const bool l1 = c1 < 0, l2 = c2 < 0;
    if (l1 && l2) {
      ++o.nleaf;
      p1 = -(c1 + 1);
      p2 = -(c2 + 1);
      const float Lg = tri_gap_bound(*A, *B, p1, p2, dir, tsize);
      if (Lg > fmaxf(best_up, 0.015625f * tsize)) {
        pop();
        return;
      }
      phase = DC_WITNESS;
      return;
    }
    int a1, a2, e1, e2;
    const bool fos = l2 ? true : (l1 ? false : size_key(*A, b1) > size_key(*B, b2));
    float L1, L2;
    if (fos) {
      a1 = c1; a2 = b2; e1 = c1 + 1; e2 = b2;
      const RssF rb = load_rss(*B, b2);
      L1 = rss_pair_bound(load_rss(*A, a1), rb, dir, qf, Ec0);
      L2 = rss_pair_bound(load_rss(*A, e1), rb, dir, qf, Ec0);
    } else {
      a1 = b1; a2 = c2; e1 = b1; e2 = c2 + 1;
      const RssF ra = load_rss(*A, b1);
      L1 = rss_pair_bound(ra, load_rss(*B, a2), dir, qf, Ec0);
      L2 = rss_pair_bound(ra, load_rss(*B, e2), dir, qf, Ec0);
    }
    o.nbv += 2;
    int f1, f2, g1, g2;
    float fd, gd;
    if (L2 < L1) {
      f1 = e1; f2 = e2; fd = L2; g1 = a1; g2 = a2; gd = L1;
    } else {
      f1 = a1; f2 = a2; fd = L1; g1 = e1; g2 = e2; gd = L2;
    }
    if (!(gd > best_up)) {
      if (sp >= STACK) {
        o.status |= DEV_ERR_STACK;
        phase = DC_DONE;
        return;
      }
      stk[sp++] = DStackC{g1, g2, gd, epoch};
    }
    if (!(fd > best_up)) {
      b1 = f1;
      b2 = f2;
      return;
    }
    pop();
  }

  // WITNESS: FP32 triangle distance with its certified bound, then the FP64 gap near
  // the best; EXACT when the pair may still pass the strict "<" update.
  FCLG_HD void witness() {
    const float near = 0.015625f * tsize;
    float w[3], l;
    const float Lw = tri_witness_bound(qf, *A, *B, p1, p2, w, l);
    bool eval = !((double)Lw > not_better) || !(Lw > near);
    if (eval && Lw > near && o.d < 1.7976931348623157e308) {
      // the FP64 gap decides pairs near the best: skipped when certainly not better,
      // or when their distance is the same vertex-vertex distance as the best's (same
      // two vertices as the best's witness points)
      V3<double> pu, pv;
      bool vv;
      const double L64 = tri_gap64(*A, *B, p1, p2, R, T, w, tau, pu, pv, vv);
      if (L64 > not_better) eval = false;
      else if (vv && same_point(pu, o.P, vtol) && same_point(pv, o.Q, vtol)) eval = false;
    }
    if (eval)
      phase = DC_EXACT;
    else
      pop();
  }

  // EXACT: FCL's FP64 triangle distance and DistanceResult's strict "<" update.
  FCLG_HD void exact() {
    const float u = FCLG_U32;
    ++o.nrc;
    V3<double> P, Q;
    const double d64 = leaf_distance64_hd(*A, *B, p1, p2, R, T, P, Q);
    if (o.d > d64) {
      o.d = d64;
      o.id1 = p1;
      o.id2 = p2;
      o.P = P;
      o.Q = Q;
      if (d64 == 0.0) {  // nothing passes a strict "<" against 0
        phase = DC_DONE;
        return;
      }
      best_up = (float)d64 * (1.f + 2.f * u) + m64;
      not_better = d64 + (double)m64;
      if (set_dist_dir(*A, *B, R, T, Q.x - P.x, Q.y - P.y, Q.z - P.z, dir)) ++epoch;
    }
    pop();
  }

  FCLG_HD void run_phase(int ph) {
    if (ph == DC_TRAVERSE)
      traverse();
    else if (ph == DC_WITNESS)
      witness();
    else if (ph == DC_EXACT)
      exact();
  }
};

// The whole query at once (host emulation and tests).
template <int STACK>
FCLG_HD bool distance_query_cert(const DevMesh& A, const DevMesh& B, const M3<double>& R, const V3<double>& T,
                                 DistOut& o) {
  DistCert<STACK> c;
  if (!c.init(&A, &B, R, T)) return false;
  while (c.phase != DC_DONE) c.run_phase(c.phase);
  o = c.o;
  return true;
}

}  // namespace fclgpu
