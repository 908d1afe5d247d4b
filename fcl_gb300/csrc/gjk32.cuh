// FP32 GJK pre-pass for convex pairs, certified in FP64.
//
// FP64 arithmetic runs at 1/64 of the FP32 rate on GB300, and FCL's GJK/EPA
// (GJKSolver_indep, narrowphase/detail/convexity_based_algorithm/gjk-inl.h) is FP64 from
// the first iteration.  This pass runs GJK in FP32 -- Gilbert, Johnson and Keerthi's
// iteration with the closest-point-on-simplex case analysis of Ericson, "Real-Time
// Collision Detection" (2005), 5.1.2-5.1.6 -- to find a separating direction d.  The
// pair is then certified separated in FP64: with pA the support point of shape A
// toward -d and pB that of B toward d (FP64 support functions of
// minkowski_diff-inl.h:65-265), d.pA - d.pB > 0 means every point of A lies beyond every
// point of B along d, so the shapes are disjoint and FCL's GJK/EPA, whose simplices
// stay inside the Minkowski difference, cannot report an intersection.  Only pairs
// without a certificate run the FP64 solver.  The certificate asks for a gap of 2^-24
// of the coordinate scale: far above the FP64 rounding of the support points and dot
// products (2^-52 of the scale) and of FCL's absolute GJK tolerance (2^-45.5), so
// that the FP64 solver's own rounding cannot place the origin inside its simplex, and
// below what the FP32 pass can resolve anyway (coordinates rounded to 2^-24).
//
// The pass also returns its last closest point v, a good start for FCL's GJK distance
// iteration (its guess argument) when the caller wants the distance.
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

// A and B as posed: Minkowski difference A - B in A's frame
struct Mink32 {
  ShapeRef a, b;
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

FCLG_HD void make_mink32(const ShapeRef& A, const M3<double>& Ra, const D3v& ta, const ShapeRef& B,
                         const M3<double>& Rb, const D3v& tb, Mink32& m) {
  m.a = A;
  m.b = B;
  const M3<double> R1 = mulT(Rb, Ra);  // Rb^T Ra
  const M3<double> R0 = mulT(Ra, Rb);  // Ra^T Rb
  for (int i = 0; i < 9; ++i) {
    m.R1[i] = (float)R1.m[i];
    m.R0[i] = (float)R0.m[i];
  }
  const D3v dt = mulTv(Ra, tb - ta);
  m.t0 = g3f((float)dt.x, (float)dt.y, (float)dt.z);
}

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

// want_distance = false stops at the first separating direction; true iterates until
// the distance estimate converges (relative 2^-16) so that v is close to the closest
// point of the Minkowski difference.
FCLG_HD int gjk32(const Mink32& m, bool want_distance, G3f& v_out, float scale) {
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
      if (!want_distance) break;
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

// FP64 certificate along d (A-frame direction): world supports of A toward -d and of B
// toward d, both FCL's FP64 support functions on the unit direction.
FCLG_HD bool certify_separated(const ShapeRef& A, const M3<double>& Ra, const D3v& ta, const ShapeRef& B,
                               const M3<double>& Rb, const D3v& tb, const G3f& dA, double scale) {
  D3v d = mulv(Ra, v3((double)dA.x, (double)dA.y, (double)dA.z));  // world direction
  const double len = d3norm(d);
  if (!(len > 0)) return false;
  d = d3scale(d, 1.0 / len);
  const D3v pa = mulv(Ra, shape_support(A, mulTv(Ra, d3neg(d)))) + ta;
  const D3v pb = mulv(Rb, shape_support(B, mulTv(Rb, d))) + tb;
  return dot(d, pa) - dot(d, pb) > 5.9604644775390625e-08 * scale;  // 2^-24 of the scale
}

// bound on the coordinates: the translations plus each shape's extent
FCLG_HD double pair_scale(const ShapeRef& A, const D3v& ta, const ShapeRef& B, const D3v& tb) {
  auto ext = [](const ShapeRef& s) {
    switch (s.s.type) {
      case SHAPE_BOX: return 0.5 * (fabs(s.s.p[0]) + fabs(s.s.p[1]) + fabs(s.s.p[2]));
      case SHAPE_SPHERE: return fabs(s.s.p[0]);
      case SHAPE_CAPSULE: return fabs(s.s.p[0]) + 0.5 * fabs(s.s.p[1]);
      case SHAPE_CYLINDER:
      case SHAPE_CONE: return fabs(s.s.p[0]) + 0.5 * fabs(s.s.p[1]);
      default: {
        double r = 0;
        const double* V = s.verts + 3 * (long long)s.s.voff;
        const int n = s.s.type == SHAPE_TRIANGLE ? 3 : s.s.vcnt;
        for (int i = 0; i < 3 * n; ++i) r = fmax(r, fabs(V[i]));
        return 1.7320508075688772 * r;
      }
    }
  };
  return 1.0 + fmax(fabs(ta.x), fmax(fabs(ta.y), fabs(ta.z))) + fmax(fabs(tb.x), fmax(fabs(tb.y), fabs(tb.z))) +
         ext(A) + ext(B);
}

// FP32 GJK, then the FP64 certificate: true when FCL's GJK on this pair cannot end
// Inside, i.e. when GJKSolver_indep::shapeIntersect is certainly false
FCLG_HD bool certified_disjoint(const ShapeRef& A, const M3<double>& Ra, const D3v& ta, const ShapeRef& B,
                                const M3<double>& Rb, const D3v& tb) {
  Mink32 m;
  make_mink32(A, Ra, ta, B, Rb, tb, m);
  const double scale = pair_scale(A, ta, B, tb);
  G3f v;
  if (gjk32(m, false, v, (float)scale) != G32_SEPARATED) return false;
  return certify_separated(A, Ra, ta, B, Rb, tb, v, scale);
}

}  // namespace fclgpu
