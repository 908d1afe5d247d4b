// Per-pair convex shape query (collide with contact, then distance when separated),
// shared by the GPU kernel and the test-only host build.  See shape_batch.cu.
#pragma once
#include <math.h>

#include "box_box.cuh"
#include "gjk32.cuh"
#include "gjk_epa.cuh"

#if !defined(FCLG_LDG)
#if defined(__CUDA_ARCH__)
#define FCLG_LDG(p) __ldg(p)
#else
#define FCLG_LDG(p) (*(p))
#endif
#endif

namespace fclgpu {

constexpr double kGjkTol = kSolverDefaultTol;  // std::pow(eps, 7/8) = 2^-45.5 (math/constants.h:164-167)

struct PairOut {
  int hit;
  D3v normal, point;
  double depth;
  double dist;
  D3v p1, p2;
  int gstat, estat;
};

FCLG_HD D3v tf_apply(const M3<double>& R, const D3v& t, const D3v& p) { return mulv(R, p) + t; }
// point of world frame expressed in frame (R,t): R^T p + (-(R^T t))
FCLG_HD D3v tf_inv_apply(const M3<double>& R, const D3v& t, const D3v& p) {
  M3<double> Ri;
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) Ri(r, c) = R(c, r);
  const D3v ti = d3neg(mulv(Ri, t));
  return mulv(Ri, p) + ti;
}

// ---- closed forms (primitive_shape_algorithm/*-inl.h) --------------------------------
FCLG_HD bool sphere_sphere_intersect(double r1, const D3v& t1, double r2, const D3v& t2, PairOut& o) {
  const D3v diff = t2 - t1;
  const double len = d3norm(diff);
  if (len > r1 + r2) return false;
  o.normal = len > 0 ? v3(diff.x / len, diff.y / len, diff.z / len) : diff;
  const D3v t = d3scale(diff, r1);
  const double den = r1 + r2;
  o.point = t1 + v3(t.x / den, t.y / den, t.z / den);
  o.depth = r1 + r2 - len;
  return true;
}
FCLG_HD void sphere_sphere_distance(double r1, const D3v& o1, double r2, const D3v& o2, PairOut& o) {
  const D3v diff = o1 - o2;
  const double len = d3norm(diff);
  if (len > r1 + r2) {
    o.dist = len - (r1 + r2);
    o.p1 = o1 - d3scale(diff, r1 / len);
    o.p2 = o2 + d3scale(diff, r2 / len);
    return;
  }
  o.dist = -1;
}

FCLG_HD void segment_closest(const D3v& p, const D3v& s1, const D3v& s2, D3v& sp) {
  const D3v v = s2 - s1;
  const D3v w = p - s1;
  const double c1 = dot(w, v);
  const double c2 = dot(v, v);
  if (c1 <= 0)
    sp = s1;
  else if (c2 <= c1)
    sp = s2;
  else
    sp = s1 + d3scale(v, c1 / c2);
}
FCLG_HD bool sphere_capsule_intersect(double rs, const D3v& ts, double rc, double lz, const M3<double>& Rc,
                                         const D3v& tc, PairOut& o) {
  const D3v pos1 = v3(0., 0., 0.5 * lz), pos2 = v3(0., 0., -0.5 * lz);
  const D3v s_c = tf_inv_apply(Rc, tc, ts);
  D3v sp;
  segment_closest(s_c, pos1, pos2, sp);
  const D3v diff = s_c - sp;
  const double distance = d3norm(diff) - rs - rc;
  if (distance > 0) return false;
  const D3v ln = d3neg(d3normalized(diff));
  o.normal = mulv(Rc, ln);
  o.point = tf_apply(Rc, tc, sp + d3scale(ln, distance));
  o.depth = -distance;
  return true;
}
FCLG_HD void sphere_capsule_distance(double rs, const D3v& ts, double rc, double lz, const M3<double>& Rc,
                                        const D3v& tc, D3v& ps, D3v& pc, double& dist) {
  const D3v pos1 = v3(0., 0., 0.5 * lz), pos2 = v3(0., 0., -0.5 * lz);
  const D3v s_c = tf_inv_apply(Rc, tc, ts);
  D3v sp;
  segment_closest(s_c, pos1, pos2, sp);
  D3v diff = s_c - sp;
  const double distance = d3norm(diff) - rs - rc;
  if (distance <= 0) {
    dist = -1;
    return;
  }
  dist = distance;
  diff = d3normalized(diff);
  ps = tf_apply(Rc, tc, s_c - d3scale(diff, rs));
  pc = tf_apply(Rc, tc, sp + d3scale(diff, rc));
}

FCLG_HD bool nearest_in_box(const double* side, const D3v& p, D3v& n) {
  const double h[3] = {side[0] / 2, side[1] / 2, side[2] / 2};
  const double pa[3] = {p.x, p.y, p.z};
  double na[3];
  bool clamped = false;
  for (int i = 0; i < 3; ++i) {
    na[i] = pa[i];
    if (pa[i] < -h[i]) {
      clamped = true;
      na[i] = -h[i];
    }
    if (pa[i] > h[i]) {
      clamped = true;
      na[i] = h[i];
    }
  }
  n = v3(na[0], na[1], na[2]);
  return clamped;
}
FCLG_HD bool sphere_box_intersect(double r, const D3v& ts, const double* side, const M3<double>& Rb,
                                     const D3v& tb, PairOut& o) {
  const D3v p_BC = tf_inv_apply(Rb, tb, ts);
  D3v p_BN;
  const bool N_is_not_C = nearest_in_box(side, p_BC, p_BN);
  const D3v p_CN_B = p_BN - p_BC;
  const double sq = sqnorm(p_CN_B);
  if (sq > r * r) return false;
  const double eps = 16 * 2.220446049250313e-16;
  D3v n, p;
  double depth;
  if (N_is_not_C && sq > eps * eps) {
    const double distance = sqrt(sq);
    n = v3(p_CN_B.x / distance, p_CN_B.y / distance, p_CN_B.z / distance);
    depth = r - distance;
    p = p_BN + d3scale(n, depth * 0.5);
  } else {
    const double h[3] = {side[0] / 2, side[1] / 2, side[2] / 2};
    const double pc[3] = {p_BC.x, p_BC.y, p_BC.z};
    double min_distance = (double)INFINITY;
    int min_axis = -1;
    for (int i = 0; i < 3; ++i) {
      const double dist = pc[i] >= 0 ? h[i] - pc[i] : pc[i] + h[i];
      if (dist + eps < min_distance) {
        min_distance = dist;
        min_axis = i;
      }
    }
    double na[3] = {0, 0, 0};
    na[min_axis] = pc[min_axis] >= 0 ? -1 : 1;
    n = v3(na[0], na[1], na[2]);
    depth = min_distance + r;
    p = p_BC + d3scale(n, (r - min_distance) / 2);
  }
  o.normal = mulv(Rb, n);
  o.point = tf_apply(Rb, tb, p);
  o.depth = depth;
  return true;
}
FCLG_HD void sphere_box_distance(double r, const D3v& ts, const double* side, const M3<double>& Rb, const D3v& tb,
                                    D3v& ps, D3v& pb, double& dist) {
  const D3v p_BC = tf_inv_apply(Rb, tb, ts);
  D3v p_BN;
  if (nearest_in_box(side, p_BC, p_BN)) {
    const D3v p_NC = p_BC - p_BN;
    const double sq = sqnorm(p_NC);
    if (sq > r * r) {
      const double d = sqrt(sq);
      dist = d - r;
      pb = tf_apply(Rb, tb, p_BN);
      const D3v u = v3(p_NC.x / d, p_NC.y / d, p_NC.z / d);
      ps = tf_apply(Rb, tb, d3scale(u, d - r) + p_BN);
      return;
    }
  }
  dist = -1;
}

FCLG_HD bool nearest_in_cylinder(double height, double radius, const D3v& q, D3v& n) {
  n = q;
  bool clamped = false;
  const double hh = height / 2;
  if (q.z > hh) {
    clamped = true;
    n.z = hh;
  } else if (q.z < -hh) {
    clamped = true;
    n.z = -hh;
  }
  double rx = q.x, ry = q.y;
  const double sq = rx * rx + ry * ry;
  if (sq > radius * radius) {
    clamped = true;
    const double k = radius / sqrt(sq);
    rx *= k;
    ry *= k;
    n.x = rx;
    n.y = ry;
  }
  return clamped;
}
FCLG_HD bool sphere_cylinder_intersect(double rs, const D3v& ts, double rc, double lz, const M3<double>& Rc,
                                          const D3v& tc, PairOut& o) {
  const D3v p_CS = tf_inv_apply(Rc, tc, ts);
  D3v p_CN;
  const bool outside = nearest_in_cylinder(lz, rc, p_CS, p_CN);
  const D3v p_SN = p_CN - p_CS;
  const double sq = sqnorm(p_SN);
  if (sq > rs * rs) return false;
  const double eps = 16 * 2.220446049250313e-16;
  D3v n, p;
  double depth;
  if (outside && sq > eps * eps) {
    const double d = sqrt(sq);
    n = v3(p_SN.x / d, p_SN.y / d, p_SN.z / d);
    depth = rs - d;
    p = p_CN + d3scale(n, depth * 0.5);
  } else {
    const double face_distance = p_CS.z >= 0 ? lz / 2 - p_CS.z : p_CS.z + lz / 2;
    const double dxy = sqrt(p_CS.x * p_CS.x + p_CS.y * p_CS.y);
    const double barrel = rc - dxy;
    if (barrel < face_distance - eps) {
      if (dxy > eps) {
        n = v3(-p_CS.x / dxy, -p_CS.y / dxy, 0.0);
        depth = rs + barrel;
        p = p_CS + d3scale(n, (rs - barrel) / 2);
      } else {
        n = v3(-1.0, 0.0, 0.0);
        depth = rs + rc;
        p = p_CS + d3scale(n, (rs - barrel) / 2);
      }
    } else {
      n = v3(0.0, 0.0, p_CS.z >= 0 ? -1.0 : 1.0);
      depth = face_distance + rs;
      p = p_CS + d3scale(n, (rs - face_distance) / 2);
    }
  }
  o.normal = mulv(Rc, n);
  o.point = tf_apply(Rc, tc, p);
  o.depth = depth;
  return true;
}
FCLG_HD void sphere_cylinder_distance(double rs, const D3v& ts, double rc, double lz, const M3<double>& Rc,
                                         const D3v& tc, D3v& ps, D3v& pc, double& dist) {
  const D3v p_CS = tf_inv_apply(Rc, tc, ts);
  D3v p_CN;
  if (nearest_in_cylinder(lz, rc, p_CS, p_CN)) {
    const D3v p_NS = p_CS - p_CN;
    const double sq = sqnorm(p_NS);
    if (sq > rs * rs) {
      const double d = sqrt(sq);
      dist = d - rs;
      pc = tf_apply(Rc, tc, p_CN);
      const D3v t = d3scale(p_NS, rs);
      ps = tf_apply(Rc, tc, p_CS - v3(t.x / d, t.y / d, t.z / d));
      return;
    }
  }
  dist = -1;
}

FCLG_HD double clampd(double n, double lo, double hi) { return n < lo ? lo : (n > hi ? hi : n); }
FCLG_HD void capsule_capsule_distance(double r1, double lz1, const M3<double>& R1, const D3v& t1, double r2,
                                         double lz2, const M3<double>& R2, const D3v& t2, PairOut& o) {
  const double kEps = kGjkTol, kEps2 = kEps * kEps;
  const D3v z1 = v3(R1(0, 2), R1(1, 2), R1(2, 2)), z2 = v3(R2(0, 2), R2(1, 2), R2(2, 2));
  const D3v arm1 = d3scale(z1, lz1 / 2), arm2 = d3scale(z2, lz2 / 2);
  const D3v P1 = t1 + arm1, Q1 = t1 - arm1, P2 = t2 + arm2, Q2 = t2 - arm2;
  const D3v d1 = Q1 - P1, d2 = Q2 - P2, r = P1 - P2;
  const double a = dot(d1, d1), e = dot(d2, d2), f = dot(d2, r);
  double s, t;
  if (a <= kEps2 && e <= kEps2) {
    s = t = 0.0;
  } else if (a <= kEps2) {
    s = 0.0;
    t = clampd(f / e, 0.0, 1.0);
  } else {
    const double c = dot(d1, r);
    if (e <= kEps2) {
      t = 0.0;
      s = clampd(-c / a, 0.0, 1.0);
    } else {
      const double b = dot(d1, d2);
      const double denom = fmax(0.0, a * e - b * b);
      s = denom > kEps2 ? clampd((b * f - c * e) / denom, 0.0, 1.0) : 0.0;
      t = (b * s + f) / e;
      if (t < 0.0) {
        t = 0.0;
        s = clampd(-c / a, 0.0, 1.0);
      } else if (t > 1.0) {
        t = 1.0;
        s = clampd((b - c) / a, 0.0, 1.0);
      }
    }
  }
  D3v n1, n2;
  if (a <= kEps2 && e <= kEps2) {
    n1 = P1;
    n2 = P2;
  } else {
    n1 = P1 + d3scale(d1, s);
    n2 = P2 + d3scale(d2, t);
  }
  const double seg = sqrt(sqnorm(n1 - n2));
  o.dist = seg - r1 - r2;
  D3v vhat;
  if (seg > kEps) {
    const D3v dd = n2 - n1;
    vhat = v3(dd.x / seg, dd.y / seg, dd.z / seg);
  } else if (fabs(dot(z1, z2)) < 1 - kEps) {
    vhat = d3normalized(cross(z1, z2));
  } else {
    vhat = v3(R1(0, 0), R1(1, 0), R1(2, 0));
  }
  o.p1 = n1 + d3scale(vhat, r1);
  o.p2 = n2 - d3scale(vhat, r2);
}

FCLG_HD void load_tf(const double* p, M3<double>& R, D3v& t) {
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) R(r, c) = FCLG_LDG(p + 4 * r + c);
  t = v3(FCLG_LDG(p + 3), FCLG_LDG(p + 7), FCLG_LDG(p + 11));
}

// the contact of an EPA that ended with status es (gjk_solver_indep-inl.h:130-154)
FCLG_HD void epa_contact(const GjkState& g, const EpaState& epa, const M3<double>& R1, const D3v& t1, int es,
                         PairOut& o) {
  o.estat = es;
  if (es == EPA_FAILED) return;
  const SimplexVert* V = g.V;
  D3v w0 = v3(0.0, 0.0, 0.0);
  for (int i = 0; i < epa.res_rank; ++i) w0 = w0 + d3scale(g.shape.support(V[epa.res_c[i]].d, 0), epa.res_p[i]);
  o.normal = epa.normal;
  o.point = tf_apply(R1, t1, w0 - d3scale(epa.normal, epa.depth * 0.5));
  o.depth = -epa.depth;  // ContactPoint depth of GST_INDEP
  o.hit = 1;
}

// GJKSolver_indep::shapeIntersect through GJK (+ EPA for the contact).  epa == nullptr
// asks for the answer only: GJK Inside decides it, since EPA::evaluate never returns
// Failed (epa-inl.h sets Failed only in initialize, :118), so FCL's EPA never turns
// an Inside into "no intersection".
FCLG_HD void gjk_intersect(const ShapeRef& A, const M3<double>& R1, const D3v& t1, const ShapeRef& B,
                              const M3<double>& R2, const D3v& t2, SimplexVert* V, EpaState* epa, PairOut& o) {
  const D3v guess = v3(1.0, 0.0, 0.0);
  const SolverParams sp = solver_params();
  o.estat = -1;
  o.hit = 0;
  // FCL's GJK ends Valid on a certified pair: no intersection (with fewer iterations
  // than the default it may end Failed instead, so the status needs the FP64 run)
  if (sp.gjk_max_iterations >= 128 && certified_disjoint(A, R1, t1, B, R2, t2)) {
    o.gstat = GJK_VALID;
    return;
  }
  GjkState g;
  make_minkowski(A, R1, t1, B, R2, t2, g.shape);
  g.V = V;
  g.tolerance = sp.gjk_tolerance;
  const int gs = g.evaluate(d3neg(guess), sp.gjk_max_iterations);
  o.gstat = gs;
  if (gs != GJK_INSIDE) return;
  if (!epa) {
    o.hit = 1;
    return;
  }
  epa->tolerance = sp.epa_tolerance;
  epa->init();
  const int es = epa->evaluate(g, d3neg(guess), sp.epa_max_iterations);
  epa_contact(g, *epa, R1, t1, es, o);
}

// GJKSolver_indep::shapeDistance through GJK (gjk_solver_indep-inl.h:593-645): the
// solver's setup, then (after the GJK loop) the witness points and the distance
FCLG_HD void gjk_distance_begin(const ShapeRef& A, const M3<double>& R1, const D3v& t1, const ShapeRef& B,
                                const M3<double>& R2, const D3v& t2, SimplexVert* V, GjkState& g) {
  const D3v guess = v3(1.0, 0.0, 0.0);
  const SolverParams sp = solver_params();
  make_minkowski(A, R1, t1, B, R2, t2, g.shape);
  g.V = V;
  g.tolerance = sp.gjk_tolerance;
  g.begin(d3neg(guess), sp.gjk_max_iterations);
}
FCLG_HD void gjk_distance_end(GjkState& g, const M3<double>& R1, const D3v& t1, PairOut& o) {
  const SimplexVert* V = g.V;
  const int gs = g.finish();
  o.gstat = gs;
  if (gs == GJK_VALID) {
    D3v w0 = v3(0.0, 0.0, 0.0), w1 = v3(0.0, 0.0, 0.0);
    const Simplex& s = g.simplices[g.current];
    for (int i = 0; i < s.rank; ++i) {
      const double p = s.p[i];
      w0 = w0 + d3scale(g.shape.support(V[s.c[i]].d, 0), p);
      w1 = w1 + d3scale(g.shape.support(d3neg(V[s.c[i]].d), 1), p);
    }
    o.dist = d3norm(w0 - w1);
    o.p1 = tf_apply(R1, t1, w0);
    o.p2 = tf_apply(R1, t1, w1);
  } else {
    o.dist = -1;
  }
}
FCLG_HD void gjk_distance(const ShapeRef& A, const M3<double>& R1, const D3v& t1, const ShapeRef& B,
                             const M3<double>& R2, const D3v& t2, SimplexVert* V, PairOut& o) {
  GjkState g;
  gjk_distance_begin(A, R1, t1, B, R2, t2, V, g);
  while (!g.step()) {
  }
  gjk_distance_end(g, R1, t1, o);
}

// true when fcl::distance on this ordered type pair runs GJK (no closed form is
// registered for it in GJKSolver_indep, gjk_solver_indep-inl.h:686-708)
FCLG_HD bool distance_uses_gjk(int a, int b) {
  if (a == SHAPE_SPHERE && (b == SHAPE_SPHERE || b == SHAPE_CAPSULE || b == SHAPE_BOX || b == SHAPE_CYLINDER))
    return false;
  if (b == SHAPE_SPHERE && (a == SHAPE_CAPSULE || a == SHAPE_BOX || a == SHAPE_CYLINDER)) return false;
  return !(a == SHAPE_CAPSULE && b == SHAPE_CAPSULE);
}

// One pair: shapes a, b (with the vertex pool) at tf1, tf2 (3x4 row-major).
enum { PAIR_INTERSECT = 1, PAIR_DISTANCE = 2, PAIR_BOTH = 3, PAIR_NO_CONTACT = 4, PAIR_DEFER_EPA = 8 };
// estat of a pair whose GJK ended Inside under PAIR_DEFER_EPA: the contact (EPA) is
// still to be computed by a full PAIR_INTERSECT query
constexpr int kEpaPending = -2;

// mode PAIR_INTERSECT: fcl::collide only; PAIR_DISTANCE: fcl::distance only (dist = -1
// when the distance dispatch finds the pair intersecting); PAIR_BOTH: collide, then
// distance when the pair does not collide.  PAIR_DEFER_EPA: a GJK pair that ends
// Inside is reported hit with estat = kEpaPending and no contact (EPA is run later,
// apart from the GJK pairs).  PAIR_NO_CONTACT: collide without contact
// information (CollisionRequest::enable_contact = false); it changes only the box-box
// case in which the reference's face clipping keeps no point, which then collides
// (box_box-inl.h:747, 775) while collide() with contacts adds no contact and reports
// no collision.
FCLG_HD void shape_pair_query(const DevShape& sa, const DevShape& sb, const double* verts, const double* tf1p,
                              const double* tf2p, PairOut& o, int mode = PAIR_BOTH) {
  ShapeRef A, B;
  A.s = sa;
  B.s = sb;
  A.verts = B.verts = verts;
  M3<double> R1, R2;
  D3v t1, t2;
  load_tf(tf1p, R1, t1);
  load_tf(tf2p, R2, t2);
  o.hit = 0;
  o.normal = o.point = o.p1 = o.p2 = v3(0.0, 0.0, 0.0);
  o.depth = 0;
  o.dist = -1;
  o.gstat = o.estat = -1;
  SimplexVert V[kSimplexSlots];
  const int a = A.s.type, b = B.s.type;
  bool hit = false;
  if (!(mode & PAIR_INTERSECT)) {
  } else if (a == SHAPE_BOX && b == SHAPE_BOX) {
    BoxBoxOut bb;
    box_box_contact(A.s.p, R1, t1, B.s.p, R2, t2, bb);
    hit = (mode & PAIR_NO_CONTACT) ? bb.code != 0 : bb.num_points > 0;
    if (bb.num_points > 0) {
      o.normal = bb.normal;
      o.point = bb.point;
      o.depth = bb.depth;
    }
  } else if (a == SHAPE_SPHERE && b == SHAPE_SPHERE) {
    hit = sphere_sphere_intersect(A.s.p[0], t1, B.s.p[0], t2, o);
  } else if (a == SHAPE_SPHERE && b == SHAPE_CAPSULE) {
    hit = sphere_capsule_intersect(A.s.p[0], t1, B.s.p[0], B.s.p[1], R2, t2, o);
  } else if (a == SHAPE_CAPSULE && b == SHAPE_SPHERE) {
    hit = sphere_capsule_intersect(B.s.p[0], t2, A.s.p[0], A.s.p[1], R1, t1, o);
    if (hit) o.normal = d3neg(o.normal);
  } else if (a == SHAPE_SPHERE && b == SHAPE_BOX) {
    hit = sphere_box_intersect(A.s.p[0], t1, B.s.p, R2, t2, o);
  } else if (a == SHAPE_BOX && b == SHAPE_SPHERE) {
    hit = sphere_box_intersect(B.s.p[0], t2, A.s.p, R1, t1, o);
    if (hit) o.normal = d3neg(o.normal);
  } else if (a == SHAPE_SPHERE && b == SHAPE_CYLINDER) {
    hit = sphere_cylinder_intersect(A.s.p[0], t1, B.s.p[0], B.s.p[1], R2, t2, o);
  } else if (a == SHAPE_CYLINDER && b == SHAPE_SPHERE) {
    hit = sphere_cylinder_intersect(B.s.p[0], t2, A.s.p[0], A.s.p[1], R1, t1, o);
    if (hit) o.normal = d3neg(o.normal);
  } else if (mode & (PAIR_NO_CONTACT | PAIR_DEFER_EPA)) {
    gjk_intersect(A, R1, t1, B, R2, t2, V, nullptr, o);
    hit = o.hit != 0;
    if (hit && (mode & PAIR_DEFER_EPA)) o.estat = kEpaPending;
  } else {
    EpaState epa;
    gjk_intersect(A, R1, t1, B, R2, t2, V, &epa, o);
    hit = o.hit != 0;
  }
  o.hit = hit ? 1 : 0;
  if (!hit && (mode & PAIR_DISTANCE)) {
    if (a == SHAPE_SPHERE && b == SHAPE_SPHERE) {
      sphere_sphere_distance(A.s.p[0], t1, B.s.p[0], t2, o);
    } else if (a == SHAPE_SPHERE && b == SHAPE_CAPSULE) {
      sphere_capsule_distance(A.s.p[0], t1, B.s.p[0], B.s.p[1], R2, t2, o.p1, o.p2, o.dist);
    } else if (a == SHAPE_CAPSULE && b == SHAPE_SPHERE) {
      sphere_capsule_distance(B.s.p[0], t2, A.s.p[0], A.s.p[1], R1, t1, o.p2, o.p1, o.dist);
    } else if (a == SHAPE_SPHERE && b == SHAPE_BOX) {
      sphere_box_distance(A.s.p[0], t1, B.s.p, R2, t2, o.p1, o.p2, o.dist);
    } else if (a == SHAPE_BOX && b == SHAPE_SPHERE) {
      sphere_box_distance(B.s.p[0], t2, A.s.p, R1, t1, o.p2, o.p1, o.dist);
    } else if (a == SHAPE_SPHERE && b == SHAPE_CYLINDER) {
      sphere_cylinder_distance(A.s.p[0], t1, B.s.p[0], B.s.p[1], R2, t2, o.p1, o.p2, o.dist);
    } else if (a == SHAPE_CYLINDER && b == SHAPE_SPHERE) {
      sphere_cylinder_distance(B.s.p[0], t2, A.s.p[0], A.s.p[1], R1, t1, o.p2, o.p1, o.dist);
    } else if (a == SHAPE_CAPSULE && b == SHAPE_CAPSULE) {
      capsule_capsule_distance(A.s.p[0], A.s.p[1], R1, t1, B.s.p[0], B.s.p[1], R2, t2, o);
    } else {
      gjk_distance(A, R1, t1, B, R2, t2, V, o);
    }
  }
}

}  // namespace fclgpu
