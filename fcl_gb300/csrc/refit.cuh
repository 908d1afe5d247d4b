// Bottom-up refit of a BVHModel<OBBRSS> after its vertices moved
// (geometry/bvh/BVH_model-inl.h:961-1027, recursiveRefitTree_bottomup, reached by
// endUpdateModel(refit = true, bottomup = true)), FP64 in the reference's operation order.
//
//   leaf:     fit<OBBRSS> of the triangle in the previous and the current frame (six
//             points: fitn, math/bv/utility-inl.h:516-523);
//   internal: left + right (OBBRSS operator+ = OBB::operator+, OBB-inl.h:161-173, and
//             RSS::operator+, RSS-inl.h).
//
// OBB::operator+ takes merge_largedist (OBB-inl.h:254-313) when the centres are farther
// apart than twice the sum of the largest half-extents, else merge_smalldist (:316-375),
// which averages the two rotations as quaternions; the quaternion conversions are
// Eigen's published formulas (matrix -> quaternion by the trace / largest-diagonal case
// split; quaternion -> matrix from the doubled products).  Both merges keep FCL's
// details: RSS::operator+ takes columns of eigen_old's matrix, whose rows are the
// eigenvectors, and builds its third axis from the first operand's axes;
// merge_smalldist updates the lower bound of a projection only when the upper bound did
// not change (`else if`).
#pragma once
#include "mesh_shape.cuh"

namespace fclgpu {

// computeVertices (OBB-inl.h:233-250)
FCLG_HD void obb_corners(const NodeD& b, D3v v[8]) {
  const D3v a0 = v3(b.axis[0], b.axis[3], b.axis[6]), a1 = v3(b.axis[1], b.axis[4], b.axis[7]),
            a2 = v3(b.axis[2], b.axis[5], b.axis[8]);
  const D3v e0 = d3scale(a0, b.ext[0]), e1 = d3scale(a1, b.ext[1]), e2 = d3scale(a2, b.ext[2]);
  const D3v T = v3(b.To[0], b.To[1], b.To[2]);
  v[0] = ((T - e0) - e1) - e2;
  v[1] = ((T + e0) - e1) - e2;
  v[2] = ((T + e0) + e1) - e2;
  v[3] = ((T - e0) + e1) - e2;
  v[4] = ((T - e0) - e1) + e2;
  v[5] = ((T + e0) - e1) + e2;
  v[6] = ((T + e0) + e1) + e2;
  v[7] = ((T - e0) + e1) + e2;
}

FCLG_HD D3v axis_col(const double a9[9], int k) { return v3(a9[k], a9[3 + k], a9[6 + k]); }

// rotation matrix (row-major) -> quaternion (x, y, z, w)
FCLG_HD void quat_from_matrix(const double m[9], double q[4]) {
  const double t = (m[0] + m[4]) + m[8];
  if (t > 0) {
    double r = sqrt(t + 1.0);
    q[3] = 0.5 * r;
    r = 0.5 / r;
    q[0] = (m[7] - m[5]) * r;
    q[1] = (m[2] - m[6]) * r;
    q[2] = (m[3] - m[1]) * r;
  } else {
    int i = 0;
    if (m[4] > m[0]) i = 1;
    if (m[8] > m[4 * i]) i = 2;
    const int j = (i + 1) % 3, k = (j + 1) % 3;
    double r = sqrt(((m[4 * i] - m[4 * j]) - m[4 * k]) + 1.0);
    q[i] = 0.5 * r;
    r = 0.5 / r;
    q[3] = (m[3 * k + j] - m[3 * j + k]) * r;
    q[j] = (m[3 * j + i] + m[3 * i + j]) * r;
    q[k] = (m[3 * k + i] + m[3 * i + k]) * r;
  }
}

// quaternion (x, y, z, w) -> rotation matrix (row-major)
FCLG_HD void matrix_from_quat(const double q[4], double r[9]) {
  const double x = q[0], y = q[1], z = q[2], w = q[3];
  const double tx = 2 * x, ty = 2 * y, tz = 2 * z;
  const double twx = tx * w, twy = ty * w, twz = tz * w;
  const double txx = tx * x, txy = ty * x, txz = tz * x;
  const double tyy = ty * y, tyz = tz * y, tzz = tz * z;
  r[0] = 1 - (tyy + tzz);
  r[1] = txy - twz;
  r[2] = txz + twy;
  r[3] = txy + twz;
  r[4] = 1 - (txx + tzz);
  r[5] = tyz - twx;
  r[6] = txz - twy;
  r[7] = tyz + twx;
  r[8] = 1 - (txx + tyy);
}

FCLG_HD NodeD obb_merge_largedist(const NodeD& b1, const NodeD& b2) {
  D3v vertex[16];
  obb_corners(b1, vertex);
  obb_corners(b2, vertex + 8);
  const D3v c = v3(b1.To[0] - b2.To[0], b1.To[1] - b2.To[1], b1.To[2] - b2.To[2]);
  const double cn = sqrt(sqnorm(c));
  const D3v a0 = cn > 0 ? v3(c.x / cn, c.y / cn, c.z / cn) : c;
  auto proj = [&](int i) { return vertex[i] - d3scale(a0, dot(vertex[i], a0)); };
  double C[3][3];
  covariance_of(proj, 16, C);
  double evals[3], evecs[3][3];
  jacobi3(C, evals, evecs);
  int lo, mid, hi;
  order3(evals, lo, mid, hi);
  // rows max / mid of eigen_old's matrix: its eigenvectors (evecs[k] = row k)
  const D3v ax[3] = {a0, v3(evecs[hi][0], evecs[hi][1], evecs[hi][2]), v3(evecs[mid][0], evecs[mid][1], evecs[mid][2])};
  NodeD b;
  set_axis9(b.axis, ax);
  auto pts = [&](int i) { return vertex[i]; };
  extent_center_of(pts, 16, ax, b.To, b.ext);
  b.child = 0;
  b.pad = 0;
  return b;
}

FCLG_HD NodeD obb_merge_smalldist(const NodeD& b1, const NodeD& b2) {
  NodeD b;
  D3v To = v3((b1.To[0] + b2.To[0]) * 0.5, (b1.To[1] + b2.To[1]) * 0.5, (b1.To[2] + b2.To[2]) * 0.5);
  double q0[4], q1[4];
  quat_from_matrix(b1.axis, q0);
  quat_from_matrix(b2.axis, q1);
  const double d01 = ((q0[0] * q1[0] + q0[1] * q1[1]) + q0[2] * q1[2]) + q0[3] * q1[3];
  if (d01 < 0)
    for (int k = 0; k < 4; ++k) q1[k] = -q1[k];
  double q[4];
  for (int k = 0; k < 4; ++k) q[k] = q0[k] + q1[k];
  const double qn = sqrt(((q[0] * q[0] + q[1] * q[1]) + q[2] * q[2]) + q[3] * q[3]);
  if (qn > 0)
    for (int k = 0; k < 4; ++k) q[k] /= qn;
  matrix_from_quat(q, b.axis);
  double pmin[3] = {DBL_MAX, DBL_MAX, DBL_MAX}, pmax[3] = {-DBL_MAX, -DBL_MAX, -DBL_MAX};
  D3v vertex[8];
  for (int pass = 0; pass < 2; ++pass) {
    obb_corners(pass == 0 ? b1 : b2, vertex);
    for (int i = 0; i < 8; ++i) {
      const D3v diff = vertex[i] - To;
      for (int j = 0; j < 3; ++j) {
        const double d = dot(diff, axis_col(b.axis, j));
        if (d > pmax[j])
          pmax[j] = d;
        else if (d < pmin[j])
          pmin[j] = d;
      }
    }
  }
  for (int j = 0; j < 3; ++j) {
    To = To + d3scale(axis_col(b.axis, j), 0.5 * (pmax[j] + pmin[j]));
    b.ext[j] = 0.5 * (pmax[j] - pmin[j]);
  }
  b.To[0] = To.x;
  b.To[1] = To.y;
  b.To[2] = To.z;
  b.child = 0;
  b.pad = 0;
  return b;
}

// Eigen's normalized(): v / |v| when |v|^2 > 0, else v
FCLG_HD D3v eigen_normalized(const D3v& v) {
  const double z = sqnorm(v);
  if (z > 0) {
    const double n = sqrt(z);
    return v3(v.x / n, v.y / n, v.z / n);
  }
  return v;
}

// fit<OBBRSS>(ps, 3) of a leaf refitted without a previous frame (after
// beginReplaceModel): OBB fit3 and RSS fit3 (math/bv/utility-inl.h:92-119, 208-233) share
// the axes (third = normalised e0 x e1, first = the longest edge normalised, second =
// third x first); then the extent / centre and the RSS rectangle of the three points.
FCLG_HD void fit3_obbrss(const D3v p[3], NodeD& obb, RssD& rss) {
  const D3v e[3] = {p[0] - p[1], p[1] - p[2], p[2] - p[0]};
  const double len[3] = {sqnorm(e[0]), sqnorm(e[1]), sqnorm(e[2])};
  int imax = 0;
  if (len[1] > len[0]) imax = 1;
  if (len[2] > len[imax]) imax = 2;
  const D3v a2 = eigen_normalized(cross(e[0], e[1]));
  const D3v a0 = eigen_normalized(e[imax]);
  const D3v ax[3] = {a0, cross(a2, a0), a2};
  set_axis9(obb.axis, ax);
  auto pts = [&](int i) { return p[i]; };
  extent_center_of(pts, 3, ax, obb.To, obb.ext);
  for (int k = 0; k < 9; ++k) rss.axis[k] = obb.axis[k];
  rss_fit_of(pts, 3, ax, rss.To, rss.l, rss.r);
}

// OBB::operator+
FCLG_HD NodeD obb_merge(const NodeD& a, const NodeD& b) {
  const D3v cd = v3(a.To[0] - b.To[0], a.To[1] - b.To[1], a.To[2] - b.To[2]);
  const double me1 = fmax(fmax(a.ext[0], a.ext[1]), a.ext[2]);
  const double me2 = fmax(fmax(b.ext[0], b.ext[1]), b.ext[2]);
  if (sqrt(sqnorm(cd)) > 2 * (me1 + me2)) return obb_merge_largedist(a, b);
  return obb_merge_smalldist(a, b);
}

// the 8 corners of an RSS's rectangle swept by its radius (RSS::operator+)
FCLG_HD void rss_corners(const RssD& s, D3v* out) {
  const D3v c0 = axis_col(s.axis, 0), c1 = axis_col(s.axis, 1), c2 = axis_col(s.axis, 2);
  const D3v d0p = d3scale(c0, s.l[0] + s.r), d1p = d3scale(c1, s.l[1] + s.r);
  const D3v d0n = d3scale(c0, -s.r), d1n = d3scale(c1, -s.r);
  const D3v d2p = d3scale(c2, s.r), d2n = d3scale(c2, -s.r);
  const D3v T = v3(s.To[0], s.To[1], s.To[2]);
  out[0] = ((T + d0p) + d1p) + d2p;
  out[1] = ((T + d0p) + d1p) + d2n;
  out[2] = ((T + d0p) + d1n) + d2p;
  out[3] = ((T + d0p) + d1n) + d2n;
  out[4] = ((T + d0n) + d1p) + d2p;
  out[5] = ((T + d0n) + d1p) + d2n;
  out[6] = ((T + d0n) + d1n) + d2p;
  out[7] = ((T + d0n) + d1n) + d2n;
}

// RSS::operator+ (self + other)
FCLG_HD RssD rss_merge(const RssD& self, const RssD& other) {
  D3v v[16];
  rss_corners(other, v);
  rss_corners(self, v + 8);
  auto pts = [&](int i) { return v[i]; };
  double C[3][3];
  covariance_of(pts, 16, C);
  double evals[3], evecs[3][3];
  jacobi3(C, evals, evecs);
  int lo, mid, hi;
  order3(evals, lo, mid, hi);
  // columns max / mid of eigen_old's matrix (whose rows are the eigenvectors), as FCL
  // takes them here
  const D3v ax[3] = {v3(evecs[0][hi], evecs[1][hi], evecs[2][hi]), v3(evecs[0][mid], evecs[1][mid], evecs[2][mid]),
                     cross(axis_col(self.axis, 0), axis_col(self.axis, 1))};
  RssD bv;
  set_axis9(bv.axis, ax);
  rss_fit_of(pts, 16, ax, bv.To, bv.l, bv.r);
  return bv;
}

}  // namespace fclgpu
