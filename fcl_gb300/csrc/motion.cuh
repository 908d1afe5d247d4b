// Motions of continuous collision (math/motion/), FP64 in the reference's operation
// order, shared by the device kernels and the test-only host build.  The rotation
// algebra follows Eigen's published formulas: Quaternion(Matrix3) (trace / largest
// diagonal cases), toRotationMatrix(), the Hamilton product, Quaternion(AngleAxis)
// (w = cos(a/2), v = sin(a/2) axis), AngleAxis(Quaternion) (angle = 2 atan2(|v|, |w|),
// axis = v / +-|v|, (0, (1,0,0)) for v = 0) and the rotation of a vector by a
// quaternion (v + w uv + v x uv with uv = 2 (q.v x v)).
//
// The linear and screw motions call sin, cos, tan and atan2; CUDA's and the host's
// implementations of those differ in the last bits, so on the device their sampled poses
// agree with an FP64 host evaluation to rounding, not bit for bit.  The translation
// motion uses only +, -, x, / and sqrt and is bit-exact.
#pragma once
#include "refit.cuh"

namespace fclgpu {

enum : int { MOTION_TRANS = 0, MOTION_LINEAR = 1, MOTION_SCREW = 2 };

struct Quat {
  double x, y, z, w;
};

FCLG_HD Quat quat_of_rotation(const double R[9]) {
  double q[4];
  quat_from_matrix(R, q);
  return Quat{q[0], q[1], q[2], q[3]};
}

FCLG_HD void rotation_of_quat(const Quat& q, double R[9]) {
  const double c[4] = {q.x, q.y, q.z, q.w};
  matrix_from_quat(c, R);
}

// a * b (Hamilton product, Eigen's generic quat_product)
FCLG_HD Quat quat_mul(const Quat& a, const Quat& b) {
  Quat r;
  r.w = ((a.w * b.w - a.x * b.x) - a.y * b.y) - a.z * b.z;
  r.x = ((a.w * b.x + a.x * b.w) + a.y * b.z) - a.z * b.y;
  r.y = ((a.w * b.y + a.y * b.w) + a.z * b.x) - a.x * b.z;
  r.z = ((a.w * b.z + a.z * b.w) + a.x * b.y) - a.y * b.x;
  return r;
}

FCLG_HD Quat quat_of_angle_axis(double angle, const D3v& axis) {
  const double ha = 0.5 * angle;
  const double s = sin(ha);
  return Quat{s * axis.x, s * axis.y, s * axis.z, cos(ha)};
}

FCLG_HD void angle_axis_of_quat(const Quat& q, double& angle, D3v& axis) {
  double n = sqrt((q.x * q.x + q.y * q.y) + q.z * q.z);
  if (n != 0.0) {
    angle = 2.0 * atan2(n, fabs(q.w));
    if (q.w < 0.0) n = -n;
    axis = v3(q.x / n, q.y / n, q.z / n);
  } else {
    angle = 0.0;
    axis = v3(1.0, 0.0, 0.0);
  }
}

// q * v for a unit quaternion
FCLG_HD D3v quat_rotate(const Quat& q, const D3v& v) {
  const D3v qv = v3(q.x, q.y, q.z);
  D3v uv = cross(qv, v);
  uv = uv + uv;
  return (v + d3scale(uv, q.w)) + cross(qv, uv);
}

// C = A * B^T (row-major 3x3)
FCLG_HD void mul_transpose(const double* A, const double* B, double C[9]) {
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j)
      C[3 * i + j] = (A[3 * i] * B[3 * j] + A[3 * i + 1] * B[3 * j + 1]) + A[3 * i + 2] * B[3 * j + 2];
}

FCLG_HD void rot_of_tf(const double* tf, double R[9]) {
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) R[3 * r + c] = tf[4 * r + c];
}

FCLG_HD D3v trans_of_tf(const double* tf) { return v3(tf[3], tf[7], tf[11]); }

FCLG_HD void write_tf(const double R[9], const D3v& t, double* out) {
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) out[4 * r + c] = R[3 * r + c];
  out[3] = t.x;
  out[7] = t.y;
  out[11] = t.z;
}

// TranslationMotion(tf_beg, tf_end).integrate(t) + getCurrentTransform
// (translation_motion-inl.h): the start rotation through a quaternion, start + range t
FCLG_HD void translation_motion_at(const double* beg, const double* end, double t, double* out) {
  if (t > 1) t = 1;
  double R[9], q[4], Rq[9];
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) R[3 * r + c] = beg[4 * r + c];
  quat_from_matrix(R, q);
  matrix_from_quat(q, Rq);
  for (int r = 0; r < 3; ++r) {
    for (int c = 0; c < 3; ++c) out[4 * r + c] = Rq[3 * r + c];
    const double start = beg[4 * r + 3];
    const double range = end[4 * r + 3] - start;
    out[4 * r + 3] = start + range * t;
  }
}

// the relative rotation R2 R1^T as an angle >= 0 and a unit axis
FCLG_HD void relative_angle_axis(const double* beg, const double* end, double& angle, D3v& axis) {
  double R1[9], R2[9], Rr[9];
  rot_of_tf(beg, R1);
  rot_of_tf(end, R2);
  mul_transpose(R2, R1, Rr);
  angle_axis_of_quat(quat_of_rotation(Rr), angle, axis);
  if (angle < 0) {
    angle = -angle;
    axis = v3(-axis.x, -axis.y, -axis.z);
  }
}

// InterpMotion(tf_beg, tf_end).integrate(t) (interp_motion-inl.h): rotation
// Quaternion(AngleAxis(t w, axis)) * Quaternion(R1) about the reference point, which this
// constructor leaves unset in FCL and is the origin here; translation
// (linear_vel t + tf1 p) - R(t) p with linear_vel = tf2 p - tf1 p.
FCLG_HD void linear_motion_at(const double* beg, const double* end, double t, double* out) {
  if (t > 1) t = 1;
  double angle;
  D3v axis;
  relative_angle_axis(beg, end, angle, axis);
  const D3v p = v3(0.0, 0.0, 0.0);
  double R1[9], R2[9];
  rot_of_tf(beg, R1);
  rot_of_tf(end, R2);
  M3<double> M1, M2;
  for (int k = 0; k < 9; ++k) {
    M1.m[k] = R1[k];
    M2.m[k] = R2[k];
  }
  const D3v tf1p = mulv(M1, p) + trans_of_tf(beg);
  const D3v tf2p = mulv(M2, p) + trans_of_tf(end);
  const D3v linear_vel = tf2p - tf1p;
  const Quat dq = quat_of_angle_axis(t * angle, axis);
  const Quat aq = quat_mul(dq, quat_of_rotation(R1));
  double R[9];
  rotation_of_quat(aq, R);
  M3<double> MR;
  for (int k = 0; k < 9; ++k) MR.m[k] = R[k];
  const D3v T = (d3scale(linear_vel, t) + tf1p) - mulv(MR, p);
  write_tf(R, T, out);
}

// ScrewMotion(tf_beg, tf_end).integrate(t) (screw_motion-inl.h, computeScrewParameter):
// rotation as the linear motion's; translation (p + axis (t v)) + dq (t1 - p).  For an
// angle below 1e-10 FCL takes axis = t2 - t1 unnormalised and v = |t2 - t1|, kept here.
FCLG_HD void screw_motion_at(const double* beg, const double* end, double t, double* out) {
  if (t > 1) t = 1;
  double angle;
  D3v axis;
  relative_angle_axis(beg, end, angle, axis);
  const D3v t1 = trans_of_tf(beg), t2 = trans_of_tf(end);
  D3v p;
  double linear_vel;
  if (angle < 1e-10) {
    angle = 0.0;
    axis = t2 - t1;
    linear_vel = sqrt(sqnorm(axis));
    p = t1;
  } else {
    const D3v o = t2 - t1;
    p = d3scale((t1 + t2) + d3scale(cross(axis, o), 1.0 / tan(angle / 2.0)), 0.5);
    linear_vel = dot(o, axis);
  }
  double R1[9];
  rot_of_tf(beg, R1);
  const Quat dq = quat_of_angle_axis(t * angle, axis);
  const Quat aq = quat_mul(dq, quat_of_rotation(R1));
  double R[9];
  rotation_of_quat(aq, R);
  const D3v T = (p + d3scale(axis, t * linear_vel)) + quat_rotate(dq, t1 - p);
  write_tf(R, T, out);
}

FCLG_HD void motion_at(int type, const double* beg, const double* end, double t, double* out) {
  if (type == MOTION_LINEAR)
    linear_motion_at(beg, end, t, out);
  else if (type == MOTION_SCREW)
    screw_motion_at(beg, end, t, out);
  else
    translation_motion_at(beg, end, t, out);
}

}  // namespace fclgpu
