// Continuous collision of mesh pairs for the oracle (test infrastructure only):
// continuousCollideNaive (narrowphase/continuous_collision-inl.h:134-171) with
// TranslationMotion (math/motion/translation_motion-inl.h: the start rotation is held as
// a quaternion and turned back into a matrix at each step; translation start + range t),
// InterpMotion (interp_motion-inl.h) or ScrewMotion (screw_motion-inl.h).
#include <algorithm>
#include <cmath>
#include <limits>
#include <vector>

#include "oracle_mesh.h"

namespace oracle {

void quat_from_matrix(const M3& m, double q[4]);  // oracle_refit.cpp (Eigen's Quaternion(Matrix3))
M3 matrix_from_quat(const double q[4]);           // oracle_refit.cpp (toRotationMatrix)

namespace {

// TranslationMotion(tf_beg, tf_end).integrate(dt) + getCurrentTransform
Tf translation_motion_at(const Tf& beg, const Tf& end, double dt) {
  if (dt > 1) dt = 1;
  double q[4];
  quat_from_matrix(beg.R, q);
  Tf f;
  f.R = matrix_from_quat(q);
  const V3 range = sub(end.t, beg.t);
  f.t = add(beg.t, scale(range, dt));
  return f;
}

// --- Eigen's rotation algebra (published formulas), as FCL's motions use it ---------
struct Q4 {
  double x, y, z, w;
};

Q4 quat_of(const M3& R) {
  double q[4];
  quat_from_matrix(R, q);
  return Q4{q[0], q[1], q[2], q[3]};
}

M3 rot_of(const Q4& q) {
  const double c[4] = {q.x, q.y, q.z, q.w};
  return matrix_from_quat(c);
}

// Hamilton product (Eigen's generic quat_product)
Q4 qmul(const Q4& a, const Q4& b) {
  return Q4{((a.w * b.x + a.x * b.w) + a.y * b.z) - a.z * b.y, ((a.w * b.y + a.y * b.w) + a.z * b.x) - a.x * b.z,
            ((a.w * b.z + a.z * b.w) + a.x * b.y) - a.y * b.x, ((a.w * b.w - a.x * b.x) - a.y * b.y) - a.z * b.z};
}

// Quaternion(AngleAxis(angle, axis))
Q4 qangle(double angle, const V3& axis) {
  double ha = 0.5 * angle;
  double s = std::sin(ha);
  return Q4{s * axis[0], s * axis[1], s * axis[2], std::cos(ha)};
}

// AngleAxis(Quaternion) (Eigen 3.3+; the norm where Eigen takes stableNorm below epsilon)
void angle_axis(const Q4& q, double& angle, V3& axis) {
  double n = std::sqrt((q.x * q.x + q.y * q.y) + q.z * q.z);
  if (n != 0.0) {
    angle = 2.0 * std::atan2(n, std::fabs(q.w));
    if (q.w < 0.0) n = -n;
    axis = mk(q.x / n, q.y / n, q.z / n);
  } else {
    angle = 0.0;
    axis = mk(1, 0, 0);
  }
}

// q * v: v + w uv + qv x uv, uv = 2 (qv x v) (Eigen's _transformVector)
V3 qrotate(const Q4& q, const V3& v) {
  V3 qv = mk(q.x, q.y, q.z);
  V3 uv = cross(qv, v);
  uv = add(uv, uv);
  return add(add(v, scale(uv, q.w)), cross(qv, uv));
}

// AngleAxis(R2 R1^T) with a non-negative angle (InterpMotion::computeVelocity,
// ScrewMotion::computeScrewParameter)
void relative_rotation(const Tf& beg, const Tf& end, double& angle, V3& axis) {
  M3 Rr = mul(end.R, transpose(beg.R));
  angle_axis(quat_of(Rr), angle, axis);
  if (angle < 0) {
    angle = -angle;
    axis = neg(axis);
  }
}

// InterpMotion(tf_beg, tf_end).integrate(dt), reference point at the origin
// (math/motion/interp_motion-inl.h)
Tf linear_motion_at(const Tf& beg, const Tf& end, double dt) {
  if (dt > 1) dt = 1;
  double angle;
  V3 axis;
  relative_rotation(beg, end, angle, axis);
  V3 p = mk(0, 0, 0);
  V3 tf1p = apply(beg, p), tf2p = apply(end, p);
  V3 linear_vel = sub(tf2p, tf1p);
  Tf f;
  f.R = rot_of(qmul(qangle(dt * angle, axis), quat_of(beg.R)));
  f.t = sub(add(scale(linear_vel, dt), tf1p), mulv(f.R, p));
  return f;
}

// ScrewMotion(tf_beg, tf_end).integrate(dt) (math/motion/screw_motion-inl.h)
Tf screw_motion_at(const Tf& beg, const Tf& end, double dt) {
  if (dt > 1) dt = 1;
  double angle;
  V3 axis;
  relative_rotation(beg, end, angle, axis);
  V3 p;
  double linear_vel;
  if (angle < 1e-10) {
    angle = 0;
    axis = sub(end.t, beg.t);
    linear_vel = norm(axis);
    p = beg.t;
  } else {
    V3 o = sub(end.t, beg.t);
    p = scale(add(add(beg.t, end.t), scale(cross(axis, o), 1.0 / std::tan(angle / 2.0))), 0.5);
    linear_vel = dot(o, axis);
  }
  Q4 dq = qangle(dt * angle, axis);
  Tf f;
  f.R = rot_of(qmul(dq, quat_of(beg.R)));
  f.t = add(add(p, scale(axis, dt * linear_vel)), qrotate(dq, sub(beg.t, p)));
  return f;
}

Tf motion_at(int type, const Tf& beg, const Tf& end, double dt) {
  if (type == 1) return linear_motion_at(beg, end, dt);
  if (type == 2) return screw_motion_at(beg, end, dt);
  return translation_motion_at(beg, end, dt);
}

// --- conservative advancement ------------------------------------------------------
// A motion with the state its bound visitors read (getVelocity, getAngularAxis, ...) and
// its current transform (the constructor's tf1 until the first integrate).
struct MotionO {
  int type;
  Tf beg, end, cur;
  V3 vel;      // translation: trans_range; linear: linear_vel
  V3 axis;     // linear: angular_axis; screw: axis
  double ang;  // angular velocity
  double lin;  // screw: linear velocity along the axis
  V3 p;        // screw: axis origin
};

void motion_init(MotionO& m, int type, const Tf& beg, const Tf& end) {
  m.type = type;
  m.beg = beg;
  m.end = end;
  m.cur = beg;
  m.ang = m.lin = 0;
  m.vel = m.axis = m.p = mk(0, 0, 0);
  if (type == 0) {
    m.vel = sub(end.t, beg.t);  // translation_motion-inl.h: trans_range
  } else if (type == 1) {       // InterpMotion::computeVelocity, reference point at the origin
    relative_rotation(beg, end, m.ang, m.axis);
    const V3 o = mk(0, 0, 0);
    m.vel = sub(apply(end, o), apply(beg, o));
  } else {  // ScrewMotion::computeScrewParameter
    relative_rotation(beg, end, m.ang, m.axis);
    if (m.ang < 1e-10) {
      m.ang = 0;
      m.axis = sub(end.t, beg.t);
      m.lin = norm(m.axis);
      m.p = beg.t;
    } else {
      const V3 o = sub(end.t, beg.t);
      m.p = scale(add(add(beg.t, end.t), scale(cross(m.axis, o), 1.0 / std::tan(m.ang / 2.0))), 0.5);
      m.lin = dot(o, m.axis);
    }
  }
}

// TriangleMotionBoundVisitor::visit (math/motion/triangle_motion_bound_visitor-inl.h)
double tri_motion_bound(const MotionO& m, const V3& a, const V3& b, const V3& c, const V3& n) {
  if (m.type == 0) return dot(m.vel, n);
  const V3 v[3] = {a, b, c};
  double pm = 0;
  for (int k = 0; k < 3; ++k) {
    // linear: tf.linear() (v - reference_p) x axis; screw: (tf.linear() v + t - p) x axis
    const V3 w = m.type == 1 ? mulv(m.cur.R, sub(v[k], mk(0, 0, 0))) : sub(add(mulv(m.cur.R, v[k]), m.cur.t), m.p);
    const double s = sqnorm(cross(w, m.axis));
    if (k == 0 || s > pm) pm = s;
  }
  pm = std::sqrt(pm);
  const double v_dot_n = m.type == 1 ? dot(m.vel, n) : dot(m.axis, n) * m.lin;
  const double w_cross_n = norm(cross(m.axis, n)) * m.ang;
  return v_dot_n + w_cross_n * pm;
}

struct CaCtx {
  const Mesh* m1;
  const Mesh* m2;
  M3 R;
  V3 T;
  Q4 R0;  // motion1's current rotation
  const MotionO* mo1;
  const MotionO* mo2;
  double min_distance;
  double delta_t;
  int64_t nbv, nleaf;
};

// meshConservativeAdvancementOrientedNodeLeafTesting
// (mesh_conservative_advancement_traversal_node-inl.h:663-747)
void ca_leaf(CaCtx& c, int b1, int b2) {
  c.nleaf++;
  const int p1 = -(c.m1->nodes[b1].first_child + 1);
  const int p2 = -(c.m2->nodes[b2].first_child + 1);
  const Tri& t1 = c.m1->tris[p1];
  const Tri& t2 = c.m2->tris[p2];
  const V3 A[3] = {c.m1->verts[t1.v[0]], c.m1->verts[t1.v[1]], c.m1->verts[t1.v[2]]};
  const V3 Bl[3] = {c.m2->verts[t2.v[0]], c.m2->verts[t2.v[1]], c.m2->verts[t2.v[2]]};
  V3 B[3];
  for (int k = 0; k < 3; ++k) B[k] = add(mulv(c.R, Bl[k]), c.T);
  V3 P, Q;
  const double d = tri_distance(A, B, P, Q);
  if (d < c.min_distance) c.min_distance = d;
  // n from object 1 to object 2 in object 1's frame, turned into the world frame by the
  // current rotation of motion 1 (Quaternion * vector), then normalize()
  V3 n = qrotate(c.R0, sub(Q, P));
  const double z = sqnorm(n);
  if (z > 0) {
    const double s = std::sqrt(z);
    n = mk(n[0] / s, n[1] / s, n[2] / s);
  }
  const double bound = tri_motion_bound(*c.mo1, A[0], A[1], A[2], n) + tri_motion_bound(*c.mo2, Bl[0], Bl[1], Bl[2], neg(n));
  const double cur = (bound <= d) ? 1.0 : d / bound;
  if (cur < c.delta_t) c.delta_t = cur;
}

// canStop with w = 1 and rel_err = abs_err = 0 (meshConservativeAdvancementOrientedNodeCanStop,
// :580-661): the OBBRSS node's BV motion bound is 0 (TBVMotionBoundVisitor has visits
// for RSS only, tbv_motion_bound_visitor-inl.h), so its delta_t update never lowers it
bool ca_can_stop(const CaCtx& c, double v) { return (v >= c.min_distance) && (v >= c.min_distance); }

bool ca_first_over_second(const CaCtx& c, int b1, int b2) {
  const bool l1 = c.m1->nodes[b1].first_child < 0, l2 = c.m2->nodes[b2].first_child < 0;
  return l2 || (!l1 && (obb_size(c.m1->nodes[b1].obb) > obb_size(c.m2->nodes[b2].obb)));
}

// distanceRecurse (traversal_recurse-inl.h:257-316) on the CA node; BVTesting is the RSS
// distance under (R, T) (mesh_conservative_advancement_traversal_node.h:169-186)
void ca_recurse(CaCtx& c, int b1, int b2) {
  const bool l1 = c.m1->nodes[b1].first_child < 0, l2 = c.m2->nodes[b2].first_child < 0;
  if (l1 && l2) {
    ca_leaf(c, b1, b2);
    return;
  }
  int a1, a2, e1, e2;
  if (ca_first_over_second(c, b1, b2)) {
    a1 = c.m1->nodes[b1].first_child;
    a2 = b2;
    e1 = a1 + 1;
    e2 = b2;
  } else {
    a1 = b1;
    a2 = c.m2->nodes[b2].first_child;
    e1 = b1;
    e2 = a2 + 1;
  }
  c.nbv += 2;
  const double d1 = rss_distance(c.R, c.T, c.m1->nodes[a1].rss, c.m2->nodes[a2].rss, nullptr, nullptr);
  const double d2 = rss_distance(c.R, c.T, c.m1->nodes[e1].rss, c.m2->nodes[e2].rss, nullptr, nullptr);
  if (d2 < d1) {
    if (!ca_can_stop(c, d2)) ca_recurse(c, e1, e2);
    if (!ca_can_stop(c, d1)) ca_recurse(c, a1, a2);
  } else {
    if (!ca_can_stop(c, d1)) ca_recurse(c, a1, a2);
    if (!ca_can_stop(c, d2)) ca_recurse(c, e1, e2);
  }
}

}  // namespace

bool continuous_collide_ca(const Mesh& m1, const Tf& a0, const Tf& a1, const Mesh& m2, const Tf& b0, const Tf& b1,
                           int motion, double& toc, Tf& ca, Tf& cb, int64_t* iterations) {
  MotionO mo1, mo2;
  motion_init(mo1, motion, a0, a1);
  motion_init(mo2, motion, b0, b1);
  int64_t it = 0;
  std::vector<int> contacts;
  bool hit;
  if (collide_mesh(m1, mo1.cur, m2, mo2.cur, 1, contacts, nullptr) > 0) {
    toc = 0;
    hit = true;
  } else {
    double t = 0;
    for (;;) {
      ++it;
      CaCtx c;
      c.m1 = &m1;
      c.m2 = &m2;
      // tf = tf1.inverse(Isometry) * tf2
      const M3 Ri = transpose(mo1.cur.R);
      c.R = mul(Ri, mo2.cur.R);
      c.T = add(mulv(Ri, mo2.cur.t), neg(mulv(Ri, mo1.cur.t)));
      c.R0 = quat_of(mo1.cur.R);
      c.mo1 = &mo1;
      c.mo2 = &mo2;
      c.min_distance = std::numeric_limits<double>::max();
      c.delta_t = 1;
      c.nbv = c.nleaf = 0;
      ca_recurse(c, 0, 0);
      if (c.delta_t <= 0.00001) break;  // t_err
      t += c.delta_t;
      if (t > 1) {
        t = 1;
        break;
      }
      mo1.cur = motion_at(motion, a0, a1, t);
      mo2.cur = motion_at(motion, b0, b1, t);
    }
    toc = t;
    hit = t < 1;
  }
  if (hit) {  // continuousCollideConservativeAdvancement: integrate(toc), then the transforms
    ca = motion_at(motion, a0, a1, toc);
    cb = motion_at(motion, b0, b1, toc);
  }
  if (iterations) *iterations = it;
  return hit;
}

bool continuous_collide_naive(const Mesh& m1, const Tf& a0, const Tf& a1, const Mesh& m2, const Tf& b0,
                              const Tf& b1, size_t num_max_iterations, double toc_err, int motion, double& toc,
                              Tf& ca, Tf& cb) {
  size_t n_iter = std::min(num_max_iterations, (size_t)std::ceil(1 / toc_err));
  for (size_t i = 0; i < n_iter; ++i) {
    double t = i / (double)(n_iter - 1);
    Tf ta = motion_at(motion, a0, a1, t);
    Tf tb = motion_at(motion, b0, b1, t);
    std::vector<int> c;
    if (collide_mesh(m1, ta, m2, tb, 1, c, nullptr)) {
      toc = t;
      ca = ta;
      cb = tb;
      return true;
    }
  }
  toc = 1.0;
  return false;
}

}  // namespace oracle

extern "C" {
// a motion (0 translation, 1 linear, 2 screw) at n times (test access to the oracle's motions)
void orc_motion(int type, int64_t n, const double* beg, const double* end, const double* t, double* out) {
  using namespace oracle;
  for (int64_t i = 0; i < n; ++i) {
    Tf a, b;
    for (int r = 0; r < 3; ++r) {
      for (int c = 0; c < 3; ++c) {
        a.R(r, c) = beg[12 * i + 4 * r + c];
        b.R(r, c) = end[12 * i + 4 * r + c];
      }
      a.t[r] = beg[12 * i + 4 * r + 3];
      b.t[r] = end[12 * i + 4 * r + 3];
    }
    Tf f = motion_at(type, a, b, t[i]);
    for (int r = 0; r < 3; ++r) {
      for (int c = 0; c < 3; ++c) out[12 * i + 4 * r + c] = f.R(r, c);
      out[12 * i + 4 * r + 3] = f.t[r];
    }
  }
}
}
