// Continuous collision of mesh pairs for the oracle (test infrastructure only):
// continuousCollideNaive (narrowphase/continuous_collision-inl.h:134-171) with
// TranslationMotion (math/motion/translation_motion-inl.h: the start rotation is held as
// a quaternion and turned back into a matrix at each step; translation start + range t),
// InterpMotion (interp_motion-inl.h) or ScrewMotion (screw_motion-inl.h).
#include <algorithm>
#include <cmath>
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

}  // namespace

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
