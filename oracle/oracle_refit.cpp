// FP64 CPU restatement of BVHModel<OBBRSS>::beginUpdateModel / updateVertex /
// endUpdateModel(refit = true, bottomup = true).  TEST INFRASTRUCTURE ONLY.
//
// Follows geometry/bvh/BVH_model-inl.h:624-727 (update protocol) and :961-1027
// (recursiveRefitTree_bottomup): a leaf is refitted to its triangle in the previous and
// the current frame (six points, fit<OBBRSS> = fitn, math/bv/utility-inl.h:516-523), an
// internal node is the OBBRSS sum of its two children, left + right
// (OBBRSS-inl.h operator+: OBB::operator+, OBB-inl.h:161-173, merge_largedist :254-313,
// merge_smalldist :316-375; RSS::operator+, RSS-inl.h).  Quaternion conversions follow
// Eigen's published formulas (rotation matrix -> quaternion by the trace / largest
// diagonal case split, quaternion -> matrix by the 2x products), reductions left to
// right; Eigen's own evaluation order is not pinned.
#include <cmath>
#include <limits>

#include "oracle_mesh.h"

namespace oracle {

// getCovariance over a point set (math/geometry-inl.h:1383-1421, point branch)
void covariance_points(const V3* ps, int n, M3& M) {
  V3 S1 = mk(0, 0, 0);
  double S2[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
  for (int i = 0; i < n; ++i) {
    const V3& p = ps[i];
    S1 = add(S1, p);
    S2[0][0] += (p[0] * p[0]);
    S2[1][1] += (p[1] * p[1]);
    S2[2][2] += (p[2] * p[2]);
    S2[0][1] += (p[0] * p[1]);
    S2[0][2] += (p[0] * p[2]);
    S2[1][2] += (p[1] * p[2]);
  }
  M(0, 0) = S2[0][0] - S1[0] * S1[0] / n;
  M(1, 1) = S2[1][1] - S1[1] * S1[1] / n;
  M(2, 2) = S2[2][2] - S1[2] * S1[2] / n;
  M(0, 1) = S2[0][1] - S1[0] * S1[1] / n;
  M(1, 2) = S2[1][2] - S1[1] * S1[2] / n;
  M(0, 2) = S2[0][2] - S1[0] * S1[2] / n;
  M(1, 0) = M(0, 1);
  M(2, 0) = M(0, 2);
  M(2, 1) = M(1, 2);
}

// getExtentAndCenter over a point set (math/geometry-inl.h:229-287); P gets the
// projections onto the axes
void extent_center_points(const V3* ps, int n, const M3& axis, V3& center, V3& extent, std::vector<V3>* P) {
  const double real_max = std::numeric_limits<double>::max();
  V3 mn = mk(real_max, real_max, real_max), mx = mk(-real_max, -real_max, -real_max);
  if (P) P->resize(n);
  for (int i = 0; i < n; ++i) {
    const V3 proj = mk(dot(col(axis, 0), ps[i]), dot(col(axis, 1), ps[i]), dot(col(axis, 2), ps[i]));
    if (P) (*P)[i] = proj;
    for (int j = 0; j < 3; ++j) {
      if (proj[j] > mx[j]) mx[j] = proj[j];
      if (proj[j] < mn[j]) mn[j] = proj[j];
    }
  }
  const V3 o = mk((mx[0] + mn[0]) / 2, (mx[1] + mn[1]) / 2, (mx[2] + mn[2]) / 2);
  center = mulv(axis, o);
  extent = mk((mx[0] - mn[0]) * 0.5, (mx[1] - mn[1]) * 0.5, (mx[2] - mn[2]) * 0.5);
}

// projections of a point set onto the columns of axis
static std::vector<V3> project_points(const V3* ps, int n, const M3& axis) {
  std::vector<V3> P(n);
  for (int i = 0; i < n; ++i)
    P[i] = mk(dot(col(axis, 0), ps[i]), dot(col(axis, 1), ps[i]), dot(col(axis, 2), ps[i]));
  return P;
}

// fit<OBBRSS> of n >= 4 points: OBB fitn and RSS fitn, which compute the same
// covariance, eigen decomposition and axes (math/bv/utility-inl.h:133-145, 247-259)
void fit_points_obbrss(const V3* ps, int n, OBB& obb, RSS& rss) {
  M3 M;
  covariance_points(ps, n, M);
  M3 E = ident();
  V3 sv = mk(0, 0, 0);
  eigen_old(M, sv, E);
  axis_from_eigen(E, sv, obb.axis);
  rss.axis = obb.axis;
  std::vector<V3> P;
  extent_center_points(ps, n, obb.axis, obb.To, obb.extent, &P);
  rss_from_projected(P, rss.axis, rss.To, rss.l, rss.r);
}

namespace {

// computeVertices (OBB-inl.h:233-250)
void obb_vertices(const OBB& b, V3 v[8]) {
  const V3 e0 = scale(col(b.axis, 0), b.extent[0]);
  const V3 e1 = scale(col(b.axis, 1), b.extent[1]);
  const V3 e2 = scale(col(b.axis, 2), b.extent[2]);
  v[0] = sub(sub(sub(b.To, e0), e1), e2);
  v[1] = sub(sub(add(b.To, e0), e1), e2);
  v[2] = sub(add(add(b.To, e0), e1), e2);
  v[3] = sub(add(sub(b.To, e0), e1), e2);
  v[4] = add(sub(sub(b.To, e0), e1), e2);
  v[5] = add(sub(add(b.To, e0), e1), e2);
  v[6] = add(add(add(b.To, e0), e1), e2);
  v[7] = add(add(sub(b.To, e0), e1), e2);
}

// the (min, mid, max) selection of OBB/RSS merges on eigenvalues s
void order3(const V3& s, int& mn, int& mid, int& mx) {
  if (s[0] > s[1]) {
    mx = 0;
    mn = 1;
  } else {
    mn = 0;
    mx = 1;
  }
  if (s[2] < s[mn]) {
    mid = mn;
    mn = 2;
  } else if (s[2] > s[mx]) {
    mid = mx;
    mx = 2;
  } else {
    mid = 2;
  }
}

V3 normalized(const V3& v) {
  const double n = norm(v);
  return n > 0 ? mk(v[0] / n, v[1] / n, v[2] / n) : v;
}

OBB merge_largedist(const OBB& b1, const OBB& b2) {
  V3 vertex[16];
  obb_vertices(b1, vertex);
  obb_vertices(b2, vertex + 8);
  OBB b;
  const V3 a0 = normalized(sub(b1.To, b2.To));
  V3 vproj[16];
  for (int i = 0; i < 16; ++i) vproj[i] = sub(vertex[i], scale(a0, dot(vertex[i], a0)));
  M3 M;
  covariance_points(vproj, 16, M);
  M3 E = ident();
  V3 s = mk(0, 0, 0);
  eigen_old(M, s, E);
  int mn, mid, mx;
  order3(s, mn, mid, mx);
  setcol(b.axis, 0, a0);
  // rows max / mid of eigen_old's matrix: its eigenvectors
  setcol(b.axis, 1, mk(E(mx, 0), E(mx, 1), E(mx, 2)));
  setcol(b.axis, 2, mk(E(mid, 0), E(mid, 1), E(mid, 2)));
  extent_center_points(vertex, 16, b.axis, b.To, b.extent, nullptr);
  return b;
}

}  // namespace

// Eigen's rotation matrix -> quaternion (x, y, z, w)
void quat_from_matrix(const M3& m, double q[4]) {
  const double t = (m(0, 0) + m(1, 1)) + m(2, 2);
  if (t > 0) {
    double r = std::sqrt(t + 1.0);
    q[3] = 0.5 * r;
    r = 0.5 / r;
    q[0] = (m(2, 1) - m(1, 2)) * r;
    q[1] = (m(0, 2) - m(2, 0)) * r;
    q[2] = (m(1, 0) - m(0, 1)) * r;
  } else {
    int i = 0;
    if (m(1, 1) > m(0, 0)) i = 1;
    if (m(2, 2) > m(i, i)) i = 2;
    const int j = (i + 1) % 3, k = (j + 1) % 3;
    double r = std::sqrt(((m(i, i) - m(j, j)) - m(k, k)) + 1.0);
    q[i] = 0.5 * r;
    r = 0.5 / r;
    q[3] = (m(k, j) - m(j, k)) * r;
    q[j] = (m(j, i) + m(i, j)) * r;
    q[k] = (m(k, i) + m(i, k)) * r;
  }
}

// Eigen's quaternion -> rotation matrix
M3 matrix_from_quat(const double q[4]) {
  const double x = q[0], y = q[1], z = q[2], w = q[3];
  const double tx = 2 * x, ty = 2 * y, tz = 2 * z;
  const double twx = tx * w, twy = ty * w, twz = tz * w;
  const double txx = tx * x, txy = ty * x, txz = tz * x;
  const double tyy = ty * y, tyz = tz * y, tzz = tz * z;
  M3 r;
  r(0, 0) = 1 - (tyy + tzz);
  r(0, 1) = txy - twz;
  r(0, 2) = txz + twy;
  r(1, 0) = txy + twz;
  r(1, 1) = 1 - (txx + tzz);
  r(1, 2) = tyz - twx;
  r(2, 0) = txz - twy;
  r(2, 1) = tyz + twx;
  r(2, 2) = 1 - (txx + tyy);
  return r;
}

namespace {

OBB merge_smalldist(const OBB& b1, const OBB& b2) {
  OBB b;
  b.To = scale(add(b1.To, b2.To), 0.5);
  double q0[4], q1[4];
  quat_from_matrix(b1.axis, q0);
  quat_from_matrix(b2.axis, q1);
  const double d01 = ((q0[0] * q1[0] + q0[1] * q1[1]) + q0[2] * q1[2]) + q0[3] * q1[3];
  if (d01 < 0)
    for (int k = 0; k < 4; ++k) q1[k] = -q1[k];
  double q[4];
  for (int k = 0; k < 4; ++k) q[k] = q0[k] + q1[k];
  const double qn = std::sqrt(((q[0] * q[0] + q[1] * q[1]) + q[2] * q[2]) + q[3] * q[3]);
  if (qn > 0)
    for (int k = 0; k < 4; ++k) q[k] /= qn;
  b.axis = matrix_from_quat(q);
  const double real_max = std::numeric_limits<double>::max();
  V3 pmin = mk(real_max, real_max, real_max), pmax = mk(-real_max, -real_max, -real_max);
  V3 vertex[8];
  for (int pass = 0; pass < 2; ++pass) {
    obb_vertices(pass == 0 ? b1 : b2, vertex);
    for (int i = 0; i < 8; ++i) {
      const V3 diff = sub(vertex[i], b.To);
      for (int j = 0; j < 3; ++j) {
        const double d = dot(diff, col(b.axis, j));
        if (d > pmax[j])
          pmax[j] = d;
        else if (d < pmin[j])
          pmin[j] = d;
      }
    }
  }
  for (int j = 0; j < 3; ++j) {
    b.To = add(b.To, scale(col(b.axis, j), 0.5 * (pmax[j] + pmin[j])));
    b.extent[j] = 0.5 * (pmax[j] - pmin[j]);
  }
  return b;
}

}  // namespace

// OBB::operator+ (OBB-inl.h:161-173)
OBB obb_merge(const OBB& a, const OBB& b) {
  const V3 cd = sub(a.To, b.To);
  const double me1 = std::max(std::max(a.extent[0], a.extent[1]), a.extent[2]);
  const double me2 = std::max(std::max(b.extent[0], b.extent[1]), b.extent[2]);
  if (norm(cd) > 2 * (me1 + me2)) return merge_largedist(a, b);
  return merge_smalldist(a, b);
}

// RSS::operator+ (RSS-inl.h): 8 corner points of each rectangle swept by r, other's
// first, covariance, eigen; axes = eigenvectors (max, mid), third axis from this's axes
RSS rss_merge(const RSS& self, const RSS& other) {
  V3 v[16];
  auto corners = [&](const RSS& s, V3* out) {
    const V3 d0p = scale(col(s.axis, 0), s.l[0] + s.r), d1p = scale(col(s.axis, 1), s.l[1] + s.r);
    const V3 d0n = scale(col(s.axis, 0), -s.r), d1n = scale(col(s.axis, 1), -s.r);
    const V3 d2p = scale(col(s.axis, 2), s.r), d2n = scale(col(s.axis, 2), -s.r);
    out[0] = add(add(add(s.To, d0p), d1p), d2p);
    out[1] = add(add(add(s.To, d0p), d1p), d2n);
    out[2] = add(add(add(s.To, d0p), d1n), d2p);
    out[3] = add(add(add(s.To, d0p), d1n), d2n);
    out[4] = add(add(add(s.To, d0n), d1p), d2p);
    out[5] = add(add(add(s.To, d0n), d1p), d2n);
    out[6] = add(add(add(s.To, d0n), d1n), d2p);
    out[7] = add(add(add(s.To, d0n), d1n), d2n);
  };
  corners(other, v);
  corners(self, v + 8);
  M3 M;
  covariance_points(v, 16, M);
  M3 E = ident();
  V3 s = mk(0, 0, 0);
  eigen_old(M, s, E);
  int mn, mid, mx;
  order3(s, mn, mid, mx);
  RSS bv;
  // columns max / mid of eigen_old's matrix (whose rows are the eigenvectors), as FCL
  // takes them here
  setcol(bv.axis, 0, col(E, mx));
  setcol(bv.axis, 1, col(E, mid));
  setcol(bv.axis, 2, cross(col(self.axis, 0), col(self.axis, 1)));
  rss_from_projected(project_points(v, 16, bv.axis), bv.axis, bv.To, bv.l, bv.r);
  return bv;
}

// recursiveRefitTree_bottomup (BVH_model-inl.h:961-1027), triangles with a previous frame
static void refit_node(Mesh& m, const std::vector<V3>& prev, int id) {
  Node& nd = m.nodes[id];
  if (nd.first_child < 0) {
    const Tri& t = m.tris[-(nd.first_child + 1)];
    V3 v[6];
    for (int i = 0; i < 3; ++i) {
      v[i] = prev[t.v[i]];
      v[i + 3] = m.verts[t.v[i]];
    }
    fit_points_obbrss(v, 6, nd.obb, nd.rss);
    return;
  }
  refit_node(m, prev, nd.first_child);
  refit_node(m, prev, nd.first_child + 1);
  const Node& l = m.nodes[nd.first_child];
  const Node& r = m.nodes[nd.first_child + 1];
  Node& me = m.nodes[id];
  me.obb = obb_merge(l.obb, r.obb);
  me.rss = rss_merge(l.rss, r.rss);
}

// beginUpdateModel + updateVertex (all vertices) + endUpdateModel(true, true): the
// previous frame becomes the vertices before this update
// Eigen's normalized(): v / |v| when |v|^2 > 0, else v
static V3 eigen_normalized(const V3& v) {
  double z = sqnorm(v);
  if (z > 0) {
    double n = std::sqrt(z);
    return mk(v[0] / n, v[1] / n, v[2] / n);
  }
  return v;
}

// fit<OBBRSS>(ps, 3): OBB fit3 + RSS fit3 (math/bv/utility-inl.h:92-119, 208-233, 507-511)
void fit3_obbrss(const V3 ps[3], OBB& obb, RSS& rss) {
  V3 e[3] = {sub(ps[0], ps[1]), sub(ps[1], ps[2]), sub(ps[2], ps[0])};
  double len[3] = {sqnorm(e[0]), sqnorm(e[1]), sqnorm(e[2])};
  int imax = 0;
  if (len[1] > len[0]) imax = 1;
  if (len[2] > len[imax]) imax = 2;
  setcol(obb.axis, 2, eigen_normalized(cross(e[0], e[1])));
  setcol(obb.axis, 0, eigen_normalized(e[imax]));
  setcol(obb.axis, 1, cross(col(obb.axis, 2), col(obb.axis, 0)));
  rss.axis = obb.axis;
  std::vector<V3> P;
  extent_center_points(ps, 3, obb.axis, obb.To, obb.extent, &P);
  rss_from_projected(P, rss.axis, rss.To, rss.l, rss.r);
}

// recursiveRefitTree_bottomup without a previous frame (BVH_model-inl.h:961-1027 after
// beginReplaceModel dropped prev_vertices): leaves fit3, internal nodes as the update's
static void refit_node_replace(Mesh& m, int id) {
  Node& nd = m.nodes[id];
  if (nd.first_child < 0) {
    const Tri& t = m.tris[-(nd.first_child + 1)];
    V3 v[3] = {m.verts[t.v[0]], m.verts[t.v[1]], m.verts[t.v[2]]};
    fit3_obbrss(v, nd.obb, nd.rss);
    return;
  }
  refit_node_replace(m, nd.first_child);
  refit_node_replace(m, nd.first_child + 1);
  const Node& l = m.nodes[nd.first_child];
  const Node& r = m.nodes[nd.first_child + 1];
  Node& me = m.nodes[id];
  me.obb = obb_merge(l.obb, r.obb);
  me.rss = rss_merge(l.rss, r.rss);
}

void replace_refit_bottomup(Mesh& m, const std::vector<V3>& new_verts) {
  m.verts = new_verts;
  refit_node_replace(m, 0);
}

void update_refit_bottomup(Mesh& m, const std::vector<V3>& new_verts) {
  const std::vector<V3> prev = m.verts;
  m.verts = new_verts;
  refit_node(m, prev, 0);
}

}  // namespace oracle
