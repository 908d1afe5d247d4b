// FP32 GJK pre-pass for convex pairs, with an FP32 separation certificate that carries
// a rigorous error bound.
//
// FP64 arithmetic runs at 1/64 of the FP32 rate on GB300, and FCL's GJK/EPA
// (GJKSolver_indep, narrowphase/detail/convexity_based_algorithm/gjk-inl.h) is FP64 from
// the first iteration.  This pass runs GJK in FP32 -- Gilbert, Johnson and Keerthi's
// iteration with the closest-point-on-simplex case analysis of Ericson, "Real-Time
// Collision Detection" (2005), 5.1.2-5.1.6 -- to find a separating direction, then
// certifies it: for the world direction D (an FP32 vector, taken as exact),
//   gap = min over A of D.a - max over B of D.b
//       = D.ta - h_A(-Ra^T D) - D.tb - h_B(Rb^T D),   h_S(u) = max over S of u.s,
// is evaluated in FP32 from the FP64 poses rounded to FP32.  Every step's error is
// bounded by u ||D||_1 times the shapes' radii and the translations (u = 2^-24): the
// rotated directions (4u per component, each moving a support value by at most that
// times the shape's radius), the support values (under 10u relative), the translation
// terms and the final sums -- under 40u ||D||_1 S in all, S = 1 + rho_A + rho_B + |ta|
// + |tb|.  The pair is certified disjoint when the computed gap exceeds 64u ||D||_1 S:
// the true gap along the unit direction then exceeds 24u S, every point of A lies beyond
// every point of B, and FCL's GJK cannot end Inside (its simplex stays inside the
// Minkowski difference; the gap is far above its rounding).  GJK also ends Inside once
// its ray is shorter than its absolute tolerance (2^-45.5 by default, 1e-6 through
// fcl::collide), so the threshold adds 1.01 times that tolerance times ||D||_1.  Only
// pairs without a certificate run the FP64 solver.
#pragma once
#include "gjk_epa.cuh"

namespace fclgpu {

struct G3f {
  float x, y, z;
};
FCLG_HD G3f g3f(float a, float b, float c) { return G3f{a, b, c}; }
FCLG_HD G3f operator+(const G3f& a, const G3f& b) { return g3f(a.x + b.x, a.y + b.y, a.z + b.z); }
FCLG_HD G3f operator-(const G3f& a, const G3f& b) { return g3f(a.x - b.x, a.y - b.y, a.z - b.z); }
FCLG_HD G3f operator*(const G3f& a, float s) { return g3f(a.x * s, a.y * s, a.z * s); }
FCLG_HD float gdot(const G3f& a, const G3f& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
FCLG_HD G3f gcross(const G3f& a, const G3f& b) {
  return g3f(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}

// support of a shape in its own frame, FP32 (any point of the shape is acceptable for
// the certificate; these are the usual support points)
FCLG_HD G3f support32(const ShapeRef& sh, const G3f& d) {
  const DevShape& s = sh.s;
  switch (s.type) {
    case SHAPE_BOX:
      return g3f(d.x > 0 ? (float)(s.p[0] * 0.5) : (float)(-s.p[0] * 0.5),
                d.y > 0 ? (float)(s.p[1] * 0.5) : (float)(-s.p[1] * 0.5),
                d.z > 0 ? (float)(s.p[2] * 0.5) : (float)(-s.p[2] * 0.5));
    case SHAPE_SPHERE: {
      const float n = sqrtf(gdot(d, d));
      return n > 0 ? d * ((float)s.p[0] / n) : g3f(0.f, 0.f, 0.f);
    }
    case SHAPE_CAPSULE: {
      const float n = sqrtf(gdot(d, d));
      const G3f r = n > 0 ? d * ((float)s.p[0] / n) : g3f(0.f, 0.f, 0.f);
      return g3f(r.x, r.y, r.z + (d.z > 0 ? (float)(s.p[1] * 0.5) : (float)(-s.p[1] * 0.5)));
    }
    case SHAPE_CYLINDER: {
      const float zd = sqrtf(d.x * d.x + d.y * d.y);
      const float hz = d.z > 0 ? (float)(s.p[1] * 0.5) : (float)(-s.p[1] * 0.5);
      if (zd == 0.f) return g3f(0.f, 0.f, hz);
      const float k = (float)s.p[0] / zd;
      return g3f(d.x * k, d.y * k, hz);
    }
    case SHAPE_CONE: {
      const float r = (float)s.p[0], hh = (float)(s.p[1] * 0.5);
      const float zd = sqrtf(d.x * d.x + d.y * d.y);
      // apex (0,0,hh) or a point of the base rim: the larger projection
      const G3f rim = zd > 0 ? g3f(d.x * (r / zd), d.y * (r / zd), -hh) : g3f(0.f, 0.f, -hh);
      return (d.z * hh > gdot(d, rim)) ? g3f(0.f, 0.f, hh) : rim;
    }
    case SHAPE_CONVEX:
      if (const float4* V32 = convex_v32(sh)) {
        G3f best = g3f(V32[0].x, V32[0].y, V32[0].z);
        float bd = gdot(d, best);
        for (int i = 1; i < s.vcnt; ++i) {
          const G3f p = g3f(V32[i].x, V32[i].y, V32[i].z);
          const float t = gdot(d, p);
          if (t > bd) {
            bd = t;
            best = p;
          }
        }
        return best;
      }
      // fall through: FP64 pool only
    case SHAPE_TRIANGLE: {
      const double* V = sh.verts + 3 * (long long)s.voff;
      const int n = s.type == SHAPE_TRIANGLE ? 3 : s.vcnt;
      G3f best = g3f((float)V[0], (float)V[1], (float)V[2]);
      float bd = gdot(d, best);
      for (int i = 1; i < n; ++i) {
        const G3f p = g3f((float)V[3 * i], (float)V[3 * i + 1], (float)V[3 * i + 2]);
        const float t = gdot(d, p);
        if (t > bd) {
          bd = t;
          best = p;
        }
      }
      return best;
    }
  }
  return g3f(0.f, 0.f, 0.f);
}

// A shape's support data rounded to FP32 once: the same values support32 rounds from
// the FP64 parameters on every call, so supports (and every decision built on them)
// are identical; leaf loops that take many supports of one shape or triangle use it
// to keep FP64 conversions out of the FP32 iteration.
struct Shape32 {
  int type, n;
  float h0, h1;       // box: half sides x, y (h2 z); round shapes: radius, half height
  float h2;
  const float4* v32;  // convex: FP32 vertices, or null
  const double* v64;  // convex without FP32 vertices: the FP64 pool
  float tv[9];        // triangle vertices
};
FCLG_HD void shape32(const ShapeRef& sh, Shape32& o) {
  const DevShape& s = sh.s;
  o.type = s.type;
  o.n = s.vcnt;
  o.h0 = o.h1 = o.h2 = 0.f;
  o.v32 = nullptr;
  o.v64 = nullptr;
  switch (s.type) {
    case SHAPE_BOX:
      o.h0 = (float)(s.p[0] * 0.5);
      o.h1 = (float)(s.p[1] * 0.5);
      o.h2 = (float)(s.p[2] * 0.5);
      break;
    case SHAPE_SPHERE:
      o.h0 = (float)s.p[0];
      break;
    case SHAPE_CAPSULE:
    case SHAPE_CYLINDER:
    case SHAPE_CONE:
      o.h0 = (float)s.p[0];
      o.h1 = (float)(s.p[1] * 0.5);
      break;
    case SHAPE_CONVEX:
      o.v32 = convex_v32(sh);
      o.v64 = sh.verts + 3 * (long long)s.voff;
      break;
    default: {  // triangle
      const double* V = sh.verts + 3 * (long long)s.voff;
      o.n = 3;
      for (int k = 0; k < 9; ++k) o.tv[k] = (float)V[k];
    }
  }
}
FCLG_HD G3f support32(const Shape32& s, const G3f& d) {
  switch (s.type) {
    case SHAPE_BOX:
      return g3f(d.x > 0 ? s.h0 : -s.h0, d.y > 0 ? s.h1 : -s.h1, d.z > 0 ? s.h2 : -s.h2);
    case SHAPE_SPHERE: {
      const float n = sqrtf(gdot(d, d));
      return n > 0 ? d * (s.h0 / n) : g3f(0.f, 0.f, 0.f);
    }
    case SHAPE_CAPSULE: {
      const float n = sqrtf(gdot(d, d));
      const G3f r = n > 0 ? d * (s.h0 / n) : g3f(0.f, 0.f, 0.f);
      return g3f(r.x, r.y, r.z + (d.z > 0 ? s.h1 : -s.h1));
    }
    case SHAPE_CYLINDER: {
      const float zd = sqrtf(d.x * d.x + d.y * d.y);
      const float hz = d.z > 0 ? s.h1 : -s.h1;
      if (zd == 0.f) return g3f(0.f, 0.f, hz);
      const float k = s.h0 / zd;
      return g3f(d.x * k, d.y * k, hz);
    }
    case SHAPE_CONE: {
      const float r = s.h0, hh = s.h1;
      const float zd = sqrtf(d.x * d.x + d.y * d.y);
      const G3f rim = zd > 0 ? g3f(d.x * (r / zd), d.y * (r / zd), -hh) : g3f(0.f, 0.f, -hh);
      return (d.z * hh > gdot(d, rim)) ? g3f(0.f, 0.f, hh) : rim;
    }
    case SHAPE_CONVEX: {
      if (s.v32) {
        G3f best = g3f(s.v32[0].x, s.v32[0].y, s.v32[0].z);
        float bd = gdot(d, best);
        for (int i = 1; i < s.n; ++i) {
          const G3f p = g3f(s.v32[i].x, s.v32[i].y, s.v32[i].z);
          const float t = gdot(d, p);
          if (t > bd) {
            bd = t;
            best = p;
          }
        }
        return best;
      }
      const double* V = s.v64;
      G3f best = g3f((float)V[0], (float)V[1], (float)V[2]);
      float bd = gdot(d, best);
      for (int i = 1; i < s.n; ++i) {
        const G3f p = g3f((float)V[3 * i], (float)V[3 * i + 1], (float)V[3 * i + 2]);
        const float t = gdot(d, p);
        if (t > bd) {
          bd = t;
          best = p;
        }
      }
      return best;
    }
    default: {  // triangle
      G3f best = g3f(s.tv[0], s.tv[1], s.tv[2]);
      float bd = gdot(d, best);
      for (int i = 1; i < 3; ++i) {
        const G3f p = g3f(s.tv[3 * i], s.tv[3 * i + 1], s.tv[3 * i + 2]);
        const float t = gdot(d, p);
        if (t > bd) {
          bd = t;
          best = p;
        }
      }
      return best;
    }
  }
}

// A and B as posed: Minkowski difference A - B in A's frame
template <class SH>
struct Mink32T {
  SH a, b;
  float R1[9];  // A-frame direction -> B-frame direction (R_B^T R_A)
  float R0[9];  // B-frame point -> A frame (R_A^T R_B)
  G3f t0;        // (A^-1 B) translation
  FCLG_HD G3f sup(const G3f& d) const {
    const G3f db = g3f(R1[0] * d.x + R1[1] * d.y + R1[2] * d.z, R1[3] * d.x + R1[4] * d.y + R1[5] * d.z,
                     R1[6] * d.x + R1[7] * d.y + R1[8] * d.z);
    const G3f pb = support32(b, g3f(-db.x, -db.y, -db.z));
    const G3f pa = support32(a, d);
    const G3f wb = g3f(R0[0] * pb.x + R0[1] * pb.y + R0[2] * pb.z, R0[3] * pb.x + R0[4] * pb.y + R0[5] * pb.z,
                     R0[6] * pb.x + R0[7] * pb.y + R0[8] * pb.z) +
                  t0;
    return pa - wb;
  }
};
using Mink32 = Mink32T<ShapeRef>;
using Mink32P = Mink32T<Shape32>;


// closest point to the origin on the triangle W[0..3) (Ericson 5.1.5 with p = origin);
// reduces W to the supporting vertex / edge / face
FCLG_HD void closest_on_triangle(G3f* W, int& n, G3f& v) {
  const G3f a = W[0], b = W[1], c = W[2];
  const G3f ab = b - a, ac = c - a, ap = g3f(-a.x, -a.y, -a.z);
  const float d1 = gdot(ab, ap), d2 = gdot(ac, ap);
  if (d1 <= 0.f && d2 <= 0.f) {
    n = 1;
    v = a;
    return;
  }
  const G3f bp = g3f(-b.x, -b.y, -b.z);
  const float d3 = gdot(ab, bp), d4 = gdot(ac, bp);
  if (d3 >= 0.f && d4 <= d3) {
    W[0] = b;
    n = 1;
    v = b;
    return;
  }
  const float vc = d1 * d4 - d3 * d2;
  if (vc <= 0.f && d1 >= 0.f && d3 <= 0.f) {
    n = 2;  // a, b
    v = a + ab * (d1 / (d1 - d3));
    return;
  }
  const G3f cp = g3f(-c.x, -c.y, -c.z);
  const float d5 = gdot(ab, cp), d6 = gdot(ac, cp);
  if (d6 >= 0.f && d5 <= d6) {
    W[0] = c;
    n = 1;
    v = c;
    return;
  }
  const float vb = d5 * d2 - d1 * d6;
  if (vb <= 0.f && d2 >= 0.f && d6 <= 0.f) {
    W[1] = c;
    n = 2;  // a, c
    v = a + ac * (d2 / (d2 - d6));
    return;
  }
  const float va = d3 * d6 - d5 * d4;
  if (va <= 0.f && (d4 - d3) >= 0.f && (d5 - d6) >= 0.f) {
    W[0] = b;
    W[1] = c;
    n = 2;  // b, c
    v = b + (c - b) * ((d4 - d3) / ((d4 - d3) + (d5 - d6)));
    return;
  }
  const float den = 1.f / (va + vb + vc);
  v = a + ab * (vb * den) + ac * (vc * den);
}

// closest point to the origin on the simplex W[0..n), reducing W to the supporting
// feature.  Returns false when the origin is inside the tetrahedron (n = 4) or the
// tetrahedron is too flat to tell.
FCLG_HD bool closest_on_simplex(G3f* W, int& n, G3f& v) {
  if (n == 1) {
    v = W[0];
    return true;
  }
  if (n == 2) {
    const G3f a = W[0], b = W[1], ab = b - a;
    const float den = gdot(ab, ab);
    const float t = den > 0 ? -gdot(a, ab) / den : 0.f;
    if (t <= 0.f) {
      n = 1;
      v = a;
    } else if (t >= 1.f) {
      W[0] = b;
      n = 1;
      v = b;
    } else {
      v = a + ab * t;
    }
    return true;
  }
  if (n == 3) {
    closest_on_triangle(W, n, v);
    return true;
  }
  // tetrahedron: the faces that have the origin on the far side from the fourth vertex
  const int face[4][4] = {{0, 1, 2, 3}, {0, 3, 1, 2}, {0, 2, 3, 1}, {1, 3, 2, 0}};
  float best = 3.4e38f;
  G3f bestv = g3f(0.f, 0.f, 0.f);
  G3f bestW[3];
  int bestn = 0;
  for (int f = 0; f < 4; ++f) {
    const G3f a = W[face[f][0]], b = W[face[f][1]], c = W[face[f][2]], d = W[face[f][3]];
    const G3f nrm = gcross(b - a, c - a);
    const float so = -gdot(a, nrm), sd = gdot(d - a, nrm);
    if (so * sd < 0.f) {
      G3f T[3] = {a, b, c};
      int tn = 3;
      G3f tv;
      closest_on_triangle(T, tn, tv);
      const float dd = gdot(tv, tv);
      if (dd < best) {
        best = dd;
        bestv = tv;
        bestn = tn;
        for (int k = 0; k < tn; ++k) bestW[k] = T[k];
      }
    }
  }
  if (bestn == 0) return false;
  for (int k = 0; k < bestn; ++k) W[k] = bestW[k];
  n = bestn;
  v = bestv;
  return true;
}

enum : int { G32_SEPARATED = 0, G32_UNKNOWN = 1 };

// Stops at the first direction v whose support gap v.w exceeds target |v| (or when the
// distance estimate converges, relative 2^-16); G32_SEPARATED when v.w > 0 at the end.
template <class MK>
FCLG_HD int gjk32(const MK& m, float target, G3f& v_out, float scale) {
  G3f W[4];
  int n = 0;
  G3f v = m.sup(g3f(1.f, 0.f, 0.f));
  W[n++] = v;
  const float eps_zero = 1e-12f * scale * scale;
  bool separated = false;
  for (int it = 0; it < 64; ++it) {
    const float vv = gdot(v, v);
    if (vv <= eps_zero) break;  // touching or inside: no certificate
    const G3f w = m.sup(g3f(-v.x, -v.y, -v.z));
    const float vw = gdot(v, w);
    if (vw > 0.f) {
      separated = true;
      if (vw * vw > target * target * vv) break;
    }
    if (vv - vw <= 1.5e-5f * vv) break;  // converged
    W[n++] = w;
    if (!closest_on_simplex(W, n, v)) {
      separated = false;
      break;
    }
  }
  v_out = v;
  return separated ? G32_SEPARATED : G32_UNKNOWN;
}

// an upper bound of the distance from a shape's frame origin to its points
FCLG_HD float shape_radius32(const ShapeRef& sh) {
  const DevShape& s = sh.s;
  float r;
  switch (s.type) {
    case SHAPE_BOX: r = 0.5f * ((fabsf((float)s.p[0]) + fabsf((float)s.p[1])) + fabsf((float)s.p[2])); break;
    case SHAPE_SPHERE: r = fabsf((float)s.p[0]); break;
    case SHAPE_CAPSULE:
    case SHAPE_CYLINDER:
    case SHAPE_CONE: r = fabsf((float)s.p[0]) + 0.5f * fabsf((float)s.p[1]); break;
    case SHAPE_CONVEX: r = (float)s.p[0]; break;  // the vertex pool's radius, set at upload
    default: {  // triangle: the largest L1 norm of its vertices
      const double* V = sh.verts + 3 * (long long)s.voff;
      r = 0.f;
      for (int i = 0; i < 3; ++i)
        r = fmaxf(r, (fabsf((float)V[3 * i]) + fabsf((float)V[3 * i + 1])) + fabsf((float)V[3 * i + 2]));
    }
  }
  return r * 1.0001f;
}

struct Pose32 {
  float R[9];  // row-major
  float t[3];
};
FCLG_HD void pose32(const M3<double>& R, const D3v& t, Pose32& p) {
  for (int i = 0; i < 9; ++i) p.R[i] = (float)R.m[i];
  p.t[0] = (float)t.x;
  p.t[1] = (float)t.y;
  p.t[2] = (float)t.z;
}
FCLG_HD G3f rot32(const float* R, const G3f& v) {
  return g3f(R[0] * v.x + R[1] * v.y + R[2] * v.z, R[3] * v.x + R[4] * v.y + R[5] * v.z,
             R[6] * v.x + R[7] * v.y + R[8] * v.z);
}
FCLG_HD G3f rot32T(const float* R, const G3f& v) {
  return g3f(R[0] * v.x + R[3] * v.y + R[6] * v.z, R[1] * v.x + R[4] * v.y + R[7] * v.z,
             R[2] * v.x + R[5] * v.y + R[8] * v.z);
}

// the Minkowski difference of A and B posed by a and b, in A's frame, in FP32
template <class SH>
FCLG_HD void make_mink32(const SH& A, const Pose32& a, const SH& B, const Pose32& b, Mink32T<SH>& m) {
  m.a = A;
  m.b = B;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      // R1 = Rb^T Ra, R0 = Ra^T Rb
      m.R1[3 * i + j] = b.R[i] * a.R[j] + b.R[3 + i] * a.R[3 + j] + b.R[6 + i] * a.R[6 + j];
      m.R0[3 * i + j] = a.R[i] * b.R[j] + a.R[3 + i] * b.R[3 + j] + a.R[6 + i] * b.R[6 + j];
    }
  m.t0 = rot32T(a.R, g3f(b.t[0] - a.t[0], b.t[1] - a.t[1], b.t[2] - a.t[2]));
}

// the FP32 certificate along the world direction D = Ra dA
template <class SH>
FCLG_HD bool certify_separated32(const SH& A, const Pose32& a, const SH& B, const Pose32& b, const G3f& dA, float S,
                                 float tol) {
  const G3f D = rot32(a.R, dA);
  const float n1 = (fabsf(D.x) + fabsf(D.y)) + fabsf(D.z);
  if (!(n1 > 0.f)) return false;
  const G3f uA = rot32T(a.R, g3f(-D.x, -D.y, -D.z)), uB = rot32T(b.R, D);
  const float hA = gdot(uA, support32(A, uA)), hB = gdot(uB, support32(B, uB));
  const G3f ta = g3f(a.t[0], a.t[1], a.t[2]), tb = g3f(b.t[0], b.t[1], b.t[2]);
  const float gap = (gdot(D, ta) - hA) - (gdot(D, tb) + hB);
  // 64u ||D||_1 S, plus the GJK tolerance (tol = 1.01 gjk_tolerance): FCL's GJK ends
  // Inside once its ray is shorter than gjk_tolerance, so a certified pair is also
  // farther apart than that
  return gap > (3.81469727e-06f * S + tol) * n1;
}

// FP32 GJK, then the FP32 certificate: true when FCL's GJK on this pair cannot end
// Inside, i.e. when GJKSolver_indep::shapeIntersect is certainly false
FCLG_HD bool certified_disjoint(const ShapeRef& A, const M3<double>& Ra, const D3v& ta, const ShapeRef& B,
                                const M3<double>& Rb, const D3v& tb) {
  Pose32 a, b;
  pose32(Ra, ta, a);
  pose32(Rb, tb, b);
  const float S = 1.f + shape_radius32(A) + shape_radius32(B) +
                  fmaxf(fabsf(a.t[0]), fmaxf(fabsf(a.t[1]), fabsf(a.t[2]))) +
                  fmaxf(fabsf(b.t[0]), fmaxf(fabsf(b.t[1]), fabsf(b.t[2])));
  if (!(S < 1e30f)) return false;
  Mink32 m;
  make_mink32(A, a, B, b, m);
  G3f v;
  // a direction whose gap clears the certificate's threshold with room to spare
  if (gjk32(m, 1.32e-5f * S, v, S) != G32_SEPARATED) return false;
  return certify_separated32(A, a, B, b, v, S, (float)solver_params().gjk_tolerance * 1.01f);
}

// One posed shape against many triangles of one posed mesh: certified_disjoint and a
// certified distance lower bound with the per-pair work done once (poses, the shape's
// FP32 supports, the relative rotations) and every triangle's supports rounded once.
// Same values, hence the same decisions, as the per-call forms.
struct LeafCert32 {
  Mink32P m;  // m.a: the shape; m.b: the current triangle
  Pose32 a, b;
  float s1;   // 1 + the shape's radius
  float ta, tb;
  float tol;  // 1.01 gjk_tolerance
};
FCLG_HD void leaf_cert_init(const ShapeRef& A, const M3<double>& Ra, const D3v& ta, const M3<double>& Rb,
                            const D3v& tb, LeafCert32& c) {
  pose32(Ra, ta, c.a);
  pose32(Rb, tb, c.b);
  Shape32 A32;
  shape32(A, A32);
  c.m.b = A32;  // replaced per triangle
  make_mink32(A32, c.a, A32, c.b, c.m);
  c.s1 = 1.f + shape_radius32(A);
  c.ta = fmaxf(fabsf(c.a.t[0]), fmaxf(fabsf(c.a.t[1]), fabsf(c.a.t[2])));
  c.tb = fmaxf(fabsf(c.b.t[0]), fmaxf(fabsf(c.b.t[1]), fabsf(c.b.t[2])));
  c.tol = (float)solver_params().gjk_tolerance * 1.01f;
}
// the triangle P (mesh frame, FP64) becomes c.m.b; returns the scale S of certified_disjoint
FCLG_HD float leaf_cert_triangle(LeafCert32& c, const double* P) {
  Shape32& t = c.m.b;
  t.type = SHAPE_TRIANGLE;
  t.n = 3;
  float r = 0.f;
  for (int i = 0; i < 3; ++i) {
    t.tv[3 * i] = (float)P[3 * i];
    t.tv[3 * i + 1] = (float)P[3 * i + 1];
    t.tv[3 * i + 2] = (float)P[3 * i + 2];
    r = fmaxf(r, (fabsf(t.tv[3 * i]) + fabsf(t.tv[3 * i + 1])) + fabsf(t.tv[3 * i + 2]));
  }
  return ((c.s1 + r * 1.0001f) + c.ta) + c.tb;
}
// == certified_disjoint(A, Ra, ta, triangle_ref(P), Rb, tb)
FCLG_HD bool leaf_cert_disjoint(LeafCert32& c, const double* P) {
  const float S = leaf_cert_triangle(c, P);
  if (!(S < 1e30f)) return false;
  G3f v;
  if (gjk32(c.m, 1.32e-5f * S, v, S) != G32_SEPARATED) return false;
  return certify_separated32(c.m.a, c.a, c.m.b, c.b, v, S, c.tol);
}
// A lower bound of the exact shape-triangle distance (-infinity when none): FP32 GJK to
// convergence, then the support gap along its direction D with the certificate's error
// bound (under 40u ||D||_1 S; 64u is subtracted), divided by |D| and scaled by 1 - 8u
// for the division and the norm; dirA = the direction in the shape's frame.
FCLG_HD float leaf_cert_lb(LeafCert32& c, const double* P, G3f& dirA) {
  const float S = leaf_cert_triangle(c, P);
  if (!(S < 1e30f)) return -INFINITY;
  G3f v;
  if (gjk32(c.m, INFINITY, v, S) != G32_SEPARATED) return -INFINITY;
  const G3f D = rot32(c.a.R, v);
  const float n1 = (fabsf(D.x) + fabsf(D.y)) + fabsf(D.z);
  const float nn = sqrtf(gdot(D, D));
  if (!(nn > 0.f)) return -INFINITY;
  const G3f uA = rot32T(c.a.R, g3f(-D.x, -D.y, -D.z)), uB = rot32T(c.b.R, D);
  const float hA = gdot(uA, support32(c.m.a, uA)), hB = gdot(uB, support32(c.m.b, uB));
  const G3f ta = g3f(c.a.t[0], c.a.t[1], c.a.t[2]), tb = g3f(c.b.t[0], c.b.t[1], c.b.t[2]);
  const float gap = (gdot(D, ta) - hA) - (gdot(D, tb) + hB);
  const float g = gap - 3.81469727e-06f * S * n1;
  if (!(g > 0.f)) return -INFINITY;
  dirA = v;
  return g * (1.f - 4.76837158e-07f) / nn;
}

}  // namespace fclgpu
