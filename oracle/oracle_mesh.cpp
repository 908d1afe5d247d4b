// FP64 CPU oracle for the BVHModel<OBBRSS> mesh path.  TEST INFRASTRUCTURE ONLY.
// Each function restates, operation by operation, the FCL 0.7.0 code it cites.
#include "oracle_mesh.h"

#include <algorithm>
#include <limits>
#include <list>
#include <utility>

namespace oracle {

// ===================================================================================
// BVH build
// ===================================================================================

// math/geometry-inl.h:1335-1421 (getCovariance, triangle branch, no second frame)
static void covariance(const Mesh& m, const unsigned* idx, int n, M3& M) {
  V3 S1 = mk(0, 0, 0);
  double S2[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
  for (int i = 0; i < n; ++i) {
    const Tri& t = m.tris[idx[i]];
    const V3& p1 = m.verts[t.v[0]];
    const V3& p2 = m.verts[t.v[1]];
    const V3& p3 = m.verts[t.v[2]];
    S1 = add(S1, add(add(p1, p2), p3));
    S2[0][0] += (p1[0] * p1[0] + p2[0] * p2[0] + p3[0] * p3[0]);
    S2[1][1] += (p1[1] * p1[1] + p2[1] * p2[1] + p3[1] * p3[1]);
    S2[2][2] += (p1[2] * p1[2] + p2[2] * p2[2] + p3[2] * p3[2]);
    S2[0][1] += (p1[0] * p1[1] + p2[0] * p2[1] + p3[0] * p3[1]);
    S2[0][2] += (p1[0] * p1[2] + p2[0] * p2[2] + p3[0] * p3[2]);
    S2[1][2] += (p1[1] * p1[2] + p2[1] * p2[2] + p3[1] * p3[2]);
  }
  const int n_points = 3 * n;
  M(0, 0) = S2[0][0] - S1[0] * S1[0] / n_points;
  M(1, 1) = S2[1][1] - S1[1] * S1[1] / n_points;
  M(2, 2) = S2[2][2] - S1[2] * S1[2] / n_points;
  M(0, 1) = S2[0][1] - S1[0] * S1[1] / n_points;
  M(1, 2) = S2[1][2] - S1[1] * S1[2] / n_points;
  M(0, 2) = S2[0][2] - S1[0] * S1[2] / n_points;
  M(1, 0) = M(0, 1);
  M(2, 0) = M(0, 2);
  M(2, 1) = M(1, 2);
}

// math/geometry-inl.h:477-558 (eigen_old: cyclic Jacobi); vout = v^T, i.e. column k
// of vout is row k of v.
void eigen_old(const M3& m, V3& dout, M3& vout) {
  M3 R = m;
  const int n = 3;
  int j, iq, ip, i;
  double tresh, theta, tau, t, sm, s, h, g, c;
  double b[3], z[3], d[3];
  double v[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
  for (ip = 0; ip < n; ++ip) {
    b[ip] = d[ip] = R(ip, ip);
    z[ip] = 0;
  }
  for (i = 0; i < 50; ++i) {
    sm = 0;
    for (ip = 0; ip < n; ++ip)
      for (iq = ip + 1; iq < n; ++iq) sm += std::abs(R(ip, iq));
    if (sm == 0.0) {
      for (int k = 0; k < 3; ++k) {
        vout(0, k) = v[k][0];
        vout(1, k) = v[k][1];
        vout(2, k) = v[k][2];
      }
      dout[0] = d[0];
      dout[1] = d[1];
      dout[2] = d[2];
      return;
    }
    if (i < 3)
      tresh = 0.2 * sm / (n * n);
    else
      tresh = 0.0;
    for (ip = 0; ip < n; ++ip) {
      for (iq = ip + 1; iq < n; ++iq) {
        g = 100.0 * std::abs(R(ip, iq));
        if (i > 3 && std::abs(d[ip]) + g == std::abs(d[ip]) && std::abs(d[iq]) + g == std::abs(d[iq]))
          R(ip, iq) = 0.0;
        else if (std::abs(R(ip, iq)) > tresh) {
          h = d[iq] - d[ip];
          if (std::abs(h) + g == std::abs(h))
            t = (R(ip, iq)) / h;
          else {
            theta = 0.5 * h / (R(ip, iq));
            t = 1.0 / (std::abs(theta) + std::sqrt(1.0 + theta * theta));
            if (theta < 0.0) t = -t;
          }
          c = 1.0 / std::sqrt(1 + t * t);
          s = t * c;
          tau = s / (1.0 + c);
          h = t * R(ip, iq);
          z[ip] -= h;
          z[iq] += h;
          d[ip] -= h;
          d[iq] += h;
          R(ip, iq) = 0.0;
          for (j = 0; j < ip; ++j) {
            g = R(j, ip); h = R(j, iq);
            R(j, ip) = g - s * (h + g * tau);
            R(j, iq) = h + s * (g - h * tau);
          }
          for (j = ip + 1; j < iq; ++j) {
            g = R(ip, j); h = R(j, iq);
            R(ip, j) = g - s * (h + g * tau);
            R(j, iq) = h + s * (g - h * tau);
          }
          for (j = iq + 1; j < n; ++j) {
            g = R(ip, j); h = R(iq, j);
            R(ip, j) = g - s * (h + g * tau);
            R(iq, j) = h + s * (g - h * tau);
          }
          for (j = 0; j < n; ++j) {
            g = v[j][ip]; h = v[j][iq];
            v[j][ip] = g - s * (h + g * tau);
            v[j][iq] = h + s * (g - h * tau);
          }
        }
      }
    }
    for (ip = 0; ip < n; ++ip) {
      b[ip] += z[ip];
      d[ip] = b[ip];
      z[ip] = 0.0;
    }
  }
  // The reference prints a warning and leaves the outputs untouched here.
}

// math/geometry-inl.h:563-598
void axis_from_eigen(const M3& eigenV, const V3& eigenS, M3& axis) {
  int mn, mid, mx;
  if (eigenS[0] > eigenS[1]) { mx = 0; mn = 1; }
  else { mn = 0; mx = 1; }
  if (eigenS[2] < eigenS[mn]) { mid = mn; mn = 2; }
  else if (eigenS[2] > eigenS[mx]) { mid = mx; mx = 2; }
  else { mid = 2; }
  setcol(axis, 0, row(eigenV, mx));
  setcol(axis, 1, row(eigenV, mid));
  setcol(axis, 2, cross(col(axis, 0), col(axis, 1)));
}

// math/geometry-inl.h (detail::getExtentAndCenter_mesh, no second frame)
static void extent_and_center(const Mesh& m, const unsigned* idx, int n, const M3& axis,
                              V3& center, V3& extent) {
  const double real_max = std::numeric_limits<double>::max();
  V3 mn = mk(real_max, real_max, real_max);
  V3 mx = mk(-real_max, -real_max, -real_max);
  for (int i = 0; i < n; ++i) {
    const Tri& t = m.tris[idx[i]];
    for (int j = 0; j < 3; ++j) {
      const V3& p = m.verts[t.v[j]];
      V3 proj = mk(dot(col(axis, 0), p), dot(col(axis, 1), p), dot(col(axis, 2), p));
      for (int k = 0; k < 3; ++k) {
        if (proj[k] > mx[k]) mx[k] = proj[k];
        if (proj[k] < mn[k]) mn[k] = proj[k];
      }
    }
  }
  V3 o = mk((mx[0] + mn[0]) / 2, (mx[1] + mn[1]) / 2, (mx[2] + mn[2]) / 2);
  center = mulv(axis, o);
  extent = mk((mx[0] - mn[0]) / 2, (mx[1] - mn[1]) / 2, (mx[2] - mn[2]) / 2);
}

// math/geometry-inl.h:709-990 (getRadiusAndOriginAndRectangleSize) over an already
// projected point list P (P[i] = (axis.col(k).dot(p))_k).
void rss_from_projected(const std::vector<V3>& P, const M3& axis, V3& origin, double l[2],
                               double& r) {
  const int size_P = (int)P.size();
  double minx, maxx, miny, maxy, minz, maxz;
  double cz, radsqr;
  minz = maxz = P[0][2];
  for (int i = 1; i < size_P; ++i) {
    double z_value = P[i][2];
    if (z_value < minz) minz = z_value;
    else if (z_value > maxz) maxz = z_value;
  }
  r = 0.5 * (maxz - minz);
  radsqr = r * r;
  cz = 0.5 * (maxz + minz);

  int minindex, maxindex;
  minindex = maxindex = 0;
  double mintmp, maxtmp;
  mintmp = maxtmp = P[0][0];
  for (int i = 1; i < size_P; ++i) {
    double x_value = P[i][0];
    if (x_value < mintmp) { minindex = i; mintmp = x_value; }
    else if (x_value > maxtmp) { maxindex = i; maxtmp = x_value; }
  }
  double x, dz;
  dz = P[minindex][2] - cz;
  minx = P[minindex][0] + std::sqrt(std::max<double>(radsqr - dz * dz, 0));
  dz = P[maxindex][2] - cz;
  maxx = P[maxindex][0] - std::sqrt(std::max<double>(radsqr - dz * dz, 0));
  for (int i = 0; i < size_P; ++i) {
    if (P[i][0] < minx) {
      dz = P[i][2] - cz;
      x = P[i][0] + std::sqrt(std::max<double>(radsqr - dz * dz, 0));
      if (x < minx) minx = x;
    }
  }
  for (int i = 0; i < size_P; ++i) {
    if (P[i][0] > maxx) {
      dz = P[i][2] - cz;
      x = P[i][0] - std::sqrt(std::max<double>(radsqr - dz * dz, 0));
      if (x > maxx) maxx = x;
    }
  }
  minindex = maxindex = 0;
  mintmp = maxtmp = P[0][1];
  for (int i = 1; i < size_P; ++i) {
    double y_value = P[i][1];
    if (y_value < mintmp) { minindex = i; mintmp = y_value; }
    else if (y_value > maxtmp) { maxindex = i; maxtmp = y_value; }
  }
  double y;
  dz = P[minindex][2] - cz;
  miny = P[minindex][1] + std::sqrt(std::max<double>(radsqr - dz * dz, 0));
  dz = P[maxindex][2] - cz;
  maxy = P[maxindex][1] - std::sqrt(std::max<double>(radsqr - dz * dz, 0));
  for (int i = 0; i < size_P; ++i) {
    if (P[i][1] < miny) {
      dz = P[i][2] - cz;
      y = P[i][1] + std::sqrt(std::max<double>(radsqr - dz * dz, 0));
      if (y < miny) miny = y;
    }
  }
  for (int i = 0; i < size_P; ++i) {
    if (P[i][1] > maxy) {
      dz = P[i][2] - cz;
      y = P[i][1] - std::sqrt(std::max<double>(radsqr - dz * dz, 0));
      if (y > maxy) maxy = y;
    }
  }
  double dx, dy, u, t;
  double a = std::sqrt(0.5);
  for (int i = 0; i < size_P; ++i) {
    if (P[i][0] > maxx) {
      if (P[i][1] > maxy) {
        dx = P[i][0] - maxx;
        dy = P[i][1] - maxy;
        u = dx * a + dy * a;
        t = (a * u - dx) * (a * u - dx) + (a * u - dy) * (a * u - dy) + (cz - P[i][2]) * (cz - P[i][2]);
        u = u - std::sqrt(std::max<double>(radsqr - t, 0));
        if (u > 0) { maxx += u * a; maxy += u * a; }
      } else if (P[i][1] < miny) {
        dx = P[i][0] - maxx;
        dy = P[i][1] - miny;
        u = dx * a - dy * a;
        t = (a * u - dx) * (a * u - dx) + (-a * u - dy) * (-a * u - dy) + (cz - P[i][2]) * (cz - P[i][2]);
        u = u - std::sqrt(std::max<double>(radsqr - t, 0));
        if (u > 0) { maxx += u * a; miny -= u * a; }
      }
    } else if (P[i][0] < minx) {
      if (P[i][1] > maxy) {
        dx = P[i][0] - minx;
        dy = P[i][1] - maxy;
        u = dy * a - dx * a;
        t = (-a * u - dx) * (-a * u - dx) + (a * u - dy) * (a * u - dy) + (cz - P[i][2]) * (cz - P[i][2]);
        u = u - std::sqrt(std::max<double>(radsqr - t, 0));
        if (u > 0) { minx -= u * a; maxy += u * a; }
      } else if (P[i][1] < miny) {
        dx = P[i][0] - minx;
        dy = P[i][1] - miny;
        u = -dx * a - dy * a;
        t = (-a * u - dx) * (-a * u - dx) + (-a * u - dy) * (-a * u - dy) + (cz - P[i][2]) * (cz - P[i][2]);
        u = u - std::sqrt(std::max<double>(radsqr - t, 0));
        if (u > 0) { minx -= u * a; miny -= u * a; }
      }
    }
  }
  // origin = axis.col(0)*minx + axis.col(1)*miny + axis.col(2)*cz
  V3 c0 = scale(col(axis, 0), minx), c1 = scale(col(axis, 1), miny), c2 = scale(col(axis, 2), cz);
  origin = add(add(c0, c1), c2);
  l[0] = maxx - minx;
  if (l[0] < 0) l[0] = 0;
  l[1] = maxy - miny;
  if (l[1] < 0) l[1] = 0;
}

static void rss_fit_mesh(const Mesh& m, const unsigned* idx, int n, const M3& axis, V3& origin,
                         double l[2], double& r) {
  std::vector<V3> P(3 * (size_t)n);
  int P_id = 0;
  for (int i = 0; i < n; ++i) {
    const Tri& t = m.tris[idx[i]];
    for (int j = 0; j < 3; ++j) {
      const V3& p = m.verts[t.v[j]];
      P[P_id] = mk(dot(col(axis, 0), p), dot(col(axis, 1), p), dot(col(axis, 2), p));
      P_id++;
    }
  }
  rss_from_projected(P, axis, origin, l, r);
}

// math/bv/utility-inl.h:208-230 (fit3 for RSS) -- used by the RSS known-answer test.
void rss_fit3(const V3 ps[3], RSS& bv) {
  const V3& p1 = ps[0];
  const V3& p2 = ps[1];
  const V3& p3 = ps[2];
  V3 e[3] = {sub(p1, p2), sub(p2, p3), sub(p3, p1)};
  double len[3] = {sqnorm(e[0]), sqnorm(e[1]), sqnorm(e[2])};
  int imax = 0;
  if (len[1] > len[0]) imax = 1;
  if (len[2] > len[imax]) imax = 2;
  V3 n = cross(e[0], e[1]);
  double nn = norm(n);
  setcol(bv.axis, 2, mk(n[0] / nn, n[1] / nn, n[2] / nn));
  double en = norm(e[imax]);
  setcol(bv.axis, 0, mk(e[imax][0] / en, e[imax][1] / en, e[imax][2] / en));
  setcol(bv.axis, 1, cross(col(bv.axis, 2), col(bv.axis, 0)));
  std::vector<V3> P(3);
  for (int i = 0; i < 3; ++i)
    P[i] = mk(dot(col(bv.axis, 0), ps[i]), dot(col(bv.axis, 1), ps[i]), dot(col(bv.axis, 2), ps[i]));
  rss_from_projected(P, bv.axis, bv.To, bv.l, bv.r);
}

// geometry/bvh/detail/BV_fitter-inl.h:448-478 (FitImpl<S, OBBRSS<S>>)
static void fit_obbrss(const Mesh& m, const unsigned* idx, int n, Node& node) {
  M3 M, E = ident();
  V3 s = mk(0, 0, 0);
  covariance(m, idx, n, M);
  eigen_old(M, s, E);
  axis_from_eigen(E, s, node.obb.axis);
  node.rss.axis = node.obb.axis;
  extent_and_center(m, idx, n, node.obb.axis, node.obb.To, node.obb.extent);
  rss_fit_mesh(m, idx, n, node.rss.axis, node.rss.To, node.rss.l, node.rss.r);
}

// geometry/bvh/BVH_model-inl.h:833-938 with the MEAN split rule
// (geometry/bvh/detail/BV_splitter-inl.h:422-436, 492-500, 540-546 and the
// triangle branch of computeSplitValue_mean).  The recursion is replaced by an
// explicit stack that visits nodes in the same order, so node ids are identical.
void build_bvh(Mesh& m) {
  const int nt = (int)m.tris.size();
  m.nodes.assign(2 * (size_t)nt - 1, Node());
  m.prim_idx.resize(2 * (size_t)nt - 1);
  for (int i = 0; i < nt; ++i) m.prim_idx[i] = (unsigned)i;
  int num_bvs = 1;
  struct Job { int bv_id, first, num; };
  std::vector<Job> stack;
  stack.push_back({0, 0, nt});
  while (!stack.empty()) {
    Job jb = stack.back();
    stack.pop_back();
    Node& node = m.nodes[jb.bv_id];
    unsigned* cur = m.prim_idx.data() + jb.first;
    fit_obbrss(m, cur, jb.num, node);
    // computeRule (mean): split_vector = obb.axis.col(0)
    V3 sv = col(node.obb.axis, 0);
    double c[3] = {0.0, 0.0, 0.0};
    for (int i = 0; i < jb.num; ++i) {
      const Tri& t = m.tris[cur[i]];
      const V3& p1 = m.verts[t.v[0]];
      const V3& p2 = m.verts[t.v[1]];
      const V3& p3 = m.verts[t.v[2]];
      c[0] += (p1[0] + p2[0] + p3[0]);
      c[1] += (p1[1] + p2[1] + p3[1]);
      c[2] += (p1[2] + p2[2] + p3[2]);
    }
    double split_value = (c[0] * sv[0] + c[1] * sv[1] + c[2] * sv[2]) / (3 * jb.num);
    node.first_primitive = jb.first;
    node.num_primitives = jb.num;
    if (jb.num == 1) {
      node.first_child = -((int)(*cur) + 1);
      continue;
    }
    node.first_child = num_bvs;
    num_bvs += 2;
    int c1 = 0;
    for (int i = 0; i < jb.num; ++i) {
      const Tri& t = m.tris[cur[i]];
      V3 p = add(add(m.verts[t.v[0]], m.verts[t.v[1]]), m.verts[t.v[2]]);
      p = mk(p[0] / 3.0, p[1] / 3.0, p[2] / 3.0);
      if (dot(sv, p) > split_value) {
        // right side
      } else {
        std::swap(cur[i], cur[c1]);
        c1++;
      }
    }
    if ((c1 == 0) || (c1 == jb.num)) c1 = jb.num / 2;
    const int left = node.first_child, right = node.first_child + 1;
    // recursion order: left subtree completely, then right subtree
    stack.push_back({right, jb.first + c1, jb.num - c1});
    stack.push_back({left, jb.first, c1});
  }
}

// ===================================================================================
// Bounding-volume tests
// ===================================================================================

// math/bv/OBB-inl.h:398-523
bool obb_disjoint(const M3& B, const V3& T, const V3& a, const V3& b) {
  double t, s;
  const double reps = 1e-6;
  M3 Bf;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) Bf(i, j) = std::abs(B(i, j)) + reps;

  t = ((T[0] < 0.0) ? -T[0] : T[0]);
  if (t > (a[0] + dot(row(Bf, 0), b))) return true;
  s = dot(col(B, 0), T);
  t = ((s < 0.0) ? -s : s);
  if (t > (b[0] + dot(col(Bf, 0), a))) return true;
  t = ((T[1] < 0.0) ? -T[1] : T[1]);
  if (t > (a[1] + dot(row(Bf, 1), b))) return true;
  t = ((T[2] < 0.0) ? -T[2] : T[2]);
  if (t > (a[2] + dot(row(Bf, 2), b))) return true;
  s = dot(col(B, 1), T);
  t = ((s < 0.0) ? -s : s);
  if (t > (b[1] + dot(col(Bf, 1), a))) return true;
  s = dot(col(B, 2), T);
  t = ((s < 0.0) ? -s : s);
  if (t > (b[2] + dot(col(Bf, 2), a))) return true;

  s = T[2] * B(1, 0) - T[1] * B(2, 0);
  t = ((s < 0.0) ? -s : s);
  if (t > (a[1] * Bf(2, 0) + a[2] * Bf(1, 0) + b[1] * Bf(0, 2) + b[2] * Bf(0, 1))) return true;
  s = T[2] * B(1, 1) - T[1] * B(2, 1);
  t = ((s < 0.0) ? -s : s);
  if (t > (a[1] * Bf(2, 1) + a[2] * Bf(1, 1) + b[0] * Bf(0, 2) + b[2] * Bf(0, 0))) return true;
  s = T[2] * B(1, 2) - T[1] * B(2, 2);
  t = ((s < 0.0) ? -s : s);
  if (t > (a[1] * Bf(2, 2) + a[2] * Bf(1, 2) + b[0] * Bf(0, 1) + b[1] * Bf(0, 0))) return true;
  s = T[0] * B(2, 0) - T[2] * B(0, 0);
  t = ((s < 0.0) ? -s : s);
  if (t > (a[0] * Bf(2, 0) + a[2] * Bf(0, 0) + b[1] * Bf(1, 2) + b[2] * Bf(1, 1))) return true;
  s = T[0] * B(2, 1) - T[2] * B(0, 1);
  t = ((s < 0.0) ? -s : s);
  if (t > (a[0] * Bf(2, 1) + a[2] * Bf(0, 1) + b[0] * Bf(1, 2) + b[2] * Bf(1, 0))) return true;
  s = T[0] * B(2, 2) - T[2] * B(0, 2);
  t = ((s < 0.0) ? -s : s);
  if (t > (a[0] * Bf(2, 2) + a[2] * Bf(0, 2) + b[0] * Bf(1, 1) + b[1] * Bf(1, 0))) return true;
  s = T[1] * B(0, 0) - T[0] * B(1, 0);
  t = ((s < 0.0) ? -s : s);
  if (t > (a[0] * Bf(1, 0) + a[1] * Bf(0, 0) + b[1] * Bf(2, 2) + b[2] * Bf(2, 1))) return true;
  s = T[1] * B(0, 1) - T[0] * B(1, 1);
  t = ((s < 0.0) ? -s : s);
  if (t > (a[0] * Bf(1, 1) + a[1] * Bf(0, 1) + b[0] * Bf(2, 2) + b[2] * Bf(2, 0))) return true;
  s = T[1] * B(0, 2) - T[0] * B(1, 2);
  t = ((s < 0.0) ? -s : s);
  if (t > (a[0] * Bf(1, 2) + a[1] * Bf(0, 2) + b[0] * Bf(2, 1) + b[1] * Bf(2, 0))) return true;
  return false;
}

// math/bv/OBB-inl.h:383-395
bool obb_overlap(const M3& R0, const V3& T0, const OBB& b1, const OBB& b2) {
  M3 R0b2 = mul(R0, b2.axis);
  M3 R = mulT(b1.axis, R0b2);
  V3 Ttemp = sub(add(mulv(R0, b2.To), T0), b1.To);
  V3 T = mulTv(b1.axis, Ttemp);
  return !obb_disjoint(R, T, b1.extent, b2.extent);
}

// math/bv/RSS-inl.h:450-455
static inline void clip_to_range(double& val, double a, double b) {
  if (val < a) val = a;
  else if (val > b) val = b;
}

// math/bv/RSS-inl.h:457-482
static void seg_coords(double& t, double& u, double a, double b, double A_dot_B, double A_dot_T,
                       double B_dot_T) {
  double denom = 1 - A_dot_B * A_dot_B;
  if (denom == 0)
    t = 0;
  else {
    t = (A_dot_T - B_dot_T * A_dot_B) / denom;
    clip_to_range(t, 0.0, a);
  }
  u = t * A_dot_B - B_dot_T;
  if (u < 0) {
    u = 0;
    t = A_dot_T;
    clip_to_range(t, 0.0, a);
  } else if (u > b) {
    u = b;
    t = u * A_dot_B + A_dot_T;
    clip_to_range(t, 0.0, a);
  }
}

// math/bv/RSS-inl.h:485-509
static bool in_voronoi(double a, double b, double Anorm_dot_B, double Anorm_dot_T, double A_dot_B,
                       double A_dot_T, double B_dot_T) {
  if (std::fabs(Anorm_dot_B) < 1e-7) return false;
  double t, u, v;
  u = -Anorm_dot_T / Anorm_dot_B;
  clip_to_range(u, 0.0, b);
  t = u * A_dot_B + A_dot_T;
  clip_to_range(t, 0.0, a);
  v = t * A_dot_B - B_dot_T;
  if (Anorm_dot_B > 0) {
    if (v > (u + 1e-7)) return true;
  } else {
    if (v < (u - 1e-7)) return true;
  }
  return false;
}

// math/bv/RSS-inl.h:512-1224 (rectDistance)
double rect_distance(const M3& Rab, const V3& Tab, const double a[2], const double b[2], V3* P,
                     V3* Q) {
  double A0_dot_B0 = Rab(0, 0), A0_dot_B1 = Rab(0, 1), A1_dot_B0 = Rab(1, 0), A1_dot_B1 = Rab(1, 1);
  double aA0_dot_B0 = a[0] * A0_dot_B0;
  double aA0_dot_B1 = a[0] * A0_dot_B1;
  double aA1_dot_B0 = a[1] * A1_dot_B0;
  double aA1_dot_B1 = a[1] * A1_dot_B1;
  double bA0_dot_B0 = b[0] * A0_dot_B0;
  double bA1_dot_B0 = b[0] * A1_dot_B0;
  double bA0_dot_B1 = b[1] * A0_dot_B1;
  double bA1_dot_B1 = b[1] * A1_dot_B1;
  V3 Tba = mulTv(Rab, Tab);
  V3 D;
  double t, u;

  auto finish = [&](double px, double py) -> double {
    if (P && Q) {
      *P = mk(px, py, 0);
      *Q = add(D, *P);
    }
    return norm(D);
  };

  double ALL_x, ALU_x, AUL_x, AUU_x, BLL_x, BLU_x, BUL_x, BUU_x;
  double LA1_lx, LA1_ux, UA1_lx, UA1_ux, LB1_lx, LB1_ux, UB1_lx, UB1_ux;
  ALL_x = -Tba[0];
  ALU_x = ALL_x + aA1_dot_B0;
  AUL_x = ALL_x + aA0_dot_B0;
  AUU_x = ALU_x + aA0_dot_B0;
  if (ALL_x < ALU_x) { LA1_lx = ALL_x; LA1_ux = ALU_x; UA1_lx = AUL_x; UA1_ux = AUU_x; }
  else { LA1_lx = ALU_x; LA1_ux = ALL_x; UA1_lx = AUU_x; UA1_ux = AUL_x; }
  BLL_x = Tab[0];
  BLU_x = BLL_x + bA0_dot_B1;
  BUL_x = BLL_x + bA0_dot_B0;
  BUU_x = BLU_x + bA0_dot_B0;
  if (BLL_x < BLU_x) { LB1_lx = BLL_x; LB1_ux = BLU_x; UB1_lx = BUL_x; UB1_ux = BUU_x; }
  else { LB1_lx = BLU_x; LB1_ux = BLL_x; UB1_lx = BUU_x; UB1_ux = BUL_x; }

  // UA1, UB1
  if ((UA1_ux > b[0]) && (UB1_ux > a[0])) {
    if (((UA1_lx > b[0]) || in_voronoi(b[1], a[1], A1_dot_B0, aA0_dot_B0 - b[0] - Tba[0], A1_dot_B1,
                                        aA0_dot_B1 - Tba[1], -Tab[1] - bA1_dot_B0)) &&
        ((UB1_lx > a[0]) || in_voronoi(a[1], b[1], A0_dot_B1, Tab[0] + bA0_dot_B0 - a[0], A1_dot_B1,
                                        Tab[1] + bA1_dot_B0, Tba[1] - aA0_dot_B1))) {
      seg_coords(t, u, a[1], b[1], A1_dot_B1, Tab[1] + bA1_dot_B0, Tba[1] - aA0_dot_B1);
      D[0] = Tab[0] + Rab(0, 0) * b[0] + Rab(0, 1) * u - a[0];
      D[1] = Tab[1] + Rab(1, 0) * b[0] + Rab(1, 1) * u - t;
      D[2] = Tab[2] + Rab(2, 0) * b[0] + Rab(2, 1) * u;
      return finish(a[0], t);
    }
  }
  // UA1, LB1
  if ((UA1_lx < 0) && (LB1_ux > a[0])) {
    if (((UA1_ux < 0) || in_voronoi(b[1], a[1], -A1_dot_B0, Tba[0] - aA0_dot_B0, A1_dot_B1,
                                     aA0_dot_B1 - Tba[1], -Tab[1])) &&
        ((LB1_lx > a[0]) || in_voronoi(a[1], b[1], A0_dot_B1, Tab[0] - a[0], A1_dot_B1, Tab[1],
                                        Tba[1] - aA0_dot_B1))) {
      seg_coords(t, u, a[1], b[1], A1_dot_B1, Tab[1], Tba[1] - aA0_dot_B1);
      D[0] = Tab[0] + Rab(0, 1) * u - a[0];
      D[1] = Tab[1] + Rab(1, 1) * u - t;
      D[2] = Tab[2] + Rab(2, 1) * u;
      return finish(a[0], t);
    }
  }
  // LA1, UB1
  if ((LA1_ux > b[0]) && (UB1_lx < 0)) {
    if (((LA1_lx > b[0]) || in_voronoi(b[1], a[1], A1_dot_B0, -Tba[0] - b[0], A1_dot_B1, -Tba[1],
                                        -Tab[1] - bA1_dot_B0)) &&
        ((UB1_ux < 0) || in_voronoi(a[1], b[1], -A0_dot_B1, -Tab[0] - bA0_dot_B0, A1_dot_B1,
                                     Tab[1] + bA1_dot_B0, Tba[1]))) {
      seg_coords(t, u, a[1], b[1], A1_dot_B1, Tab[1] + bA1_dot_B0, Tba[1]);
      D[0] = Tab[0] + Rab(0, 0) * b[0] + Rab(0, 1) * u;
      D[1] = Tab[1] + Rab(1, 0) * b[0] + Rab(1, 1) * u - t;
      D[2] = Tab[2] + Rab(2, 0) * b[0] + Rab(2, 1) * u;
      return finish(0, t);
    }
  }
  // LA1, LB1
  if ((LA1_lx < 0) && (LB1_lx < 0)) {
    if (((LA1_ux < 0) || in_voronoi(b[1], a[1], -A1_dot_B0, Tba[0], A1_dot_B1, -Tba[1], -Tab[1])) &&
        ((LB1_ux < 0) || in_voronoi(a[1], b[1], -A0_dot_B1, -Tab[0], A1_dot_B1, Tab[1], Tba[1]))) {
      seg_coords(t, u, a[1], b[1], A1_dot_B1, Tab[1], Tba[1]);
      D[0] = Tab[0] + Rab(0, 1) * u;
      D[1] = Tab[1] + Rab(1, 1) * u - t;
      D[2] = Tab[2] + Rab(2, 1) * u;
      return finish(0, t);
    }
  }

  double ALL_y, ALU_y, AUL_y, AUU_y;
  ALL_y = -Tba[1];
  ALU_y = ALL_y + aA1_dot_B1;
  AUL_y = ALL_y + aA0_dot_B1;
  AUU_y = ALU_y + aA0_dot_B1;
  double LA1_ly, LA1_uy, UA1_ly, UA1_uy, LB0_lx, LB0_ux, UB0_lx, UB0_ux;
  if (ALL_y < ALU_y) { LA1_ly = ALL_y; LA1_uy = ALU_y; UA1_ly = AUL_y; UA1_uy = AUU_y; }
  else { LA1_ly = ALU_y; LA1_uy = ALL_y; UA1_ly = AUU_y; UA1_uy = AUL_y; }
  if (BLL_x < BUL_x) { LB0_lx = BLL_x; LB0_ux = BUL_x; UB0_lx = BLU_x; UB0_ux = BUU_x; }
  else { LB0_lx = BUL_x; LB0_ux = BLL_x; UB0_lx = BUU_x; UB0_ux = BLU_x; }

  // UA1, UB0
  if ((UA1_uy > b[1]) && (UB0_ux > a[0])) {
    if (((UA1_ly > b[1]) || in_voronoi(b[0], a[1], A1_dot_B1, aA0_dot_B1 - Tba[1] - b[1], A1_dot_B0,
                                        aA0_dot_B0 - Tba[0], -Tab[1] - bA1_dot_B1)) &&
        ((UB0_lx > a[0]) || in_voronoi(a[1], b[0], A0_dot_B0, Tab[0] - a[0] + bA0_dot_B1, A1_dot_B0,
                                        Tab[1] + bA1_dot_B1, Tba[0] - aA0_dot_B0))) {
      seg_coords(t, u, a[1], b[0], A1_dot_B0, Tab[1] + bA1_dot_B1, Tba[0] - aA0_dot_B0);
      D[0] = Tab[0] + Rab(0, 1) * b[1] + Rab(0, 0) * u - a[0];
      D[1] = Tab[1] + Rab(1, 1) * b[1] + Rab(1, 0) * u - t;
      D[2] = Tab[2] + Rab(2, 1) * b[1] + Rab(2, 0) * u;
      return finish(a[0], t);
    }
  }
  // UA1, LB0
  if ((UA1_ly < 0) && (LB0_ux > a[0])) {
    if (((UA1_uy < 0) || in_voronoi(b[0], a[1], -A1_dot_B1, Tba[1] - aA0_dot_B1, A1_dot_B0,
                                     aA0_dot_B0 - Tba[0], -Tab[1])) &&
        ((LB0_lx > a[0]) || in_voronoi(a[1], b[0], A0_dot_B0, Tab[0] - a[0], A1_dot_B0, Tab[1],
                                        Tba[0] - aA0_dot_B0))) {
      seg_coords(t, u, a[1], b[0], A1_dot_B0, Tab[1], Tba[0] - aA0_dot_B0);
      D[0] = Tab[0] + Rab(0, 0) * u - a[0];
      D[1] = Tab[1] + Rab(1, 0) * u - t;
      D[2] = Tab[2] + Rab(2, 0) * u;
      return finish(a[0], t);
    }
  }
  // LA1, UB0
  if ((LA1_uy > b[1]) && (UB0_lx < 0)) {
    if (((LA1_ly > b[1]) || in_voronoi(b[0], a[1], A1_dot_B1, -Tba[1] - b[1], A1_dot_B0, -Tba[0],
                                        -Tab[1] - bA1_dot_B1)) &&
        ((UB0_ux < 0) || in_voronoi(a[1], b[0], -A0_dot_B0, -Tab[0] - bA0_dot_B1, A1_dot_B0,
                                     Tab[1] + bA1_dot_B1, Tba[0]))) {
      seg_coords(t, u, a[1], b[0], A1_dot_B0, Tab[1] + bA1_dot_B1, Tba[0]);
      D[0] = Tab[0] + Rab(0, 1) * b[1] + Rab(0, 0) * u;
      D[1] = Tab[1] + Rab(1, 1) * b[1] + Rab(1, 0) * u - t;
      D[2] = Tab[2] + Rab(2, 1) * b[1] + Rab(2, 0) * u;
      return finish(0, t);
    }
  }
  // LA1, LB0
  if ((LA1_ly < 0) && (LB0_lx < 0)) {
    if (((LA1_uy < 0) || in_voronoi(b[0], a[1], -A1_dot_B1, Tba[1], A1_dot_B0, -Tba[0], -Tab[1])) &&
        ((LB0_ux < 0) || in_voronoi(a[1], b[0], -A0_dot_B0, -Tab[0], A1_dot_B0, Tab[1], Tba[0]))) {
      seg_coords(t, u, a[1], b[0], A1_dot_B0, Tab[1], Tba[0]);
      D[0] = Tab[0] + Rab(0, 0) * u;
      D[1] = Tab[1] + Rab(1, 0) * u - t;
      D[2] = Tab[2] + Rab(2, 0) * u;
      return finish(0, t);
    }
  }

  double BLL_y, BLU_y, BUL_y, BUU_y;
  BLL_y = Tab[1];
  BLU_y = BLL_y + bA1_dot_B1;
  BUL_y = BLL_y + bA1_dot_B0;
  BUU_y = BLU_y + bA1_dot_B0;
  double LA0_lx, LA0_ux, UA0_lx, UA0_ux, LB1_ly, LB1_uy, UB1_ly, UB1_uy;
  if (ALL_x < AUL_x) { LA0_lx = ALL_x; LA0_ux = AUL_x; UA0_lx = ALU_x; UA0_ux = AUU_x; }
  else { LA0_lx = AUL_x; LA0_ux = ALL_x; UA0_lx = AUU_x; UA0_ux = ALU_x; }
  if (BLL_y < BLU_y) { LB1_ly = BLL_y; LB1_uy = BLU_y; UB1_ly = BUL_y; UB1_uy = BUU_y; }
  else { LB1_ly = BLU_y; LB1_uy = BLL_y; UB1_ly = BUU_y; UB1_uy = BUL_y; }

  // UA0, UB1
  if ((UA0_ux > b[0]) && (UB1_uy > a[1])) {
    if (((UA0_lx > b[0]) || in_voronoi(b[1], a[0], A0_dot_B0, aA1_dot_B0 - Tba[0] - b[0], A0_dot_B1,
                                        aA1_dot_B1 - Tba[1], -Tab[0] - bA0_dot_B0)) &&
        ((UB1_ly > a[1]) || in_voronoi(a[0], b[1], A1_dot_B1, Tab[1] - a[1] + bA1_dot_B0, A0_dot_B1,
                                        Tab[0] + bA0_dot_B0, Tba[1] - aA1_dot_B1))) {
      seg_coords(t, u, a[0], b[1], A0_dot_B1, Tab[0] + bA0_dot_B0, Tba[1] - aA1_dot_B1);
      D[0] = Tab[0] + Rab(0, 0) * b[0] + Rab(0, 1) * u - t;
      D[1] = Tab[1] + Rab(1, 0) * b[0] + Rab(1, 1) * u - a[1];
      D[2] = Tab[2] + Rab(2, 0) * b[0] + Rab(2, 1) * u;
      return finish(t, a[1]);
    }
  }
  // UA0, LB1
  if ((UA0_lx < 0) && (LB1_uy > a[1])) {
    if (((UA0_ux < 0) || in_voronoi(b[1], a[0], -A0_dot_B0, Tba[0] - aA1_dot_B0, A0_dot_B1,
                                     aA1_dot_B1 - Tba[1], -Tab[0])) &&
        ((LB1_ly > a[1]) || in_voronoi(a[0], b[1], A1_dot_B1, Tab[1] - a[1], A0_dot_B1, Tab[0],
                                        Tba[1] - aA1_dot_B1))) {
      seg_coords(t, u, a[0], b[1], A0_dot_B1, Tab[0], Tba[1] - aA1_dot_B1);
      D[0] = Tab[0] + Rab(0, 1) * u - t;
      D[1] = Tab[1] + Rab(1, 1) * u - a[1];
      D[2] = Tab[2] + Rab(2, 1) * u;
      return finish(t, a[1]);
    }
  }
  // LA0, UB1
  if ((LA0_ux > b[0]) && (UB1_ly < 0)) {
    if (((LA0_lx > b[0]) || in_voronoi(b[1], a[0], A0_dot_B0, -b[0] - Tba[0], A0_dot_B1, -Tba[1],
                                        -bA0_dot_B0 - Tab[0])) &&
        ((UB1_uy < 0) || in_voronoi(a[0], b[1], -A1_dot_B1, -Tab[1] - bA1_dot_B0, A0_dot_B1,
                                     Tab[0] + bA0_dot_B0, Tba[1]))) {
      seg_coords(t, u, a[0], b[1], A0_dot_B1, Tab[0] + bA0_dot_B0, Tba[1]);
      D[0] = Tab[0] + Rab(0, 0) * b[0] + Rab(0, 1) * u - t;
      D[1] = Tab[1] + Rab(1, 0) * b[0] + Rab(1, 1) * u;
      D[2] = Tab[2] + Rab(2, 0) * b[0] + Rab(2, 1) * u;
      return finish(t, 0);
    }
  }
  // LA0, LB1
  if ((LA0_lx < 0) && (LB1_ly < 0)) {
    if (((LA0_ux < 0) || in_voronoi(b[1], a[0], -A0_dot_B0, Tba[0], A0_dot_B1, -Tba[1], -Tab[0])) &&
        ((LB1_uy < 0) || in_voronoi(a[0], b[1], -A1_dot_B1, -Tab[1], A0_dot_B1, Tab[0], Tba[1]))) {
      seg_coords(t, u, a[0], b[1], A0_dot_B1, Tab[0], Tba[1]);
      D[0] = Tab[0] + Rab(0, 1) * u - t;
      D[1] = Tab[1] + Rab(1, 1) * u;
      D[2] = Tab[2] + Rab(2, 1) * u;
      return finish(t, 0);
    }
  }

  double LA0_ly, LA0_uy, UA0_ly, UA0_uy, LB0_ly, LB0_uy, UB0_ly, UB0_uy;
  if (ALL_y < AUL_y) { LA0_ly = ALL_y; LA0_uy = AUL_y; UA0_ly = ALU_y; UA0_uy = AUU_y; }
  else { LA0_ly = AUL_y; LA0_uy = ALL_y; UA0_ly = AUU_y; UA0_uy = ALU_y; }
  if (BLL_y < BUL_y) { LB0_ly = BLL_y; LB0_uy = BUL_y; UB0_ly = BLU_y; UB0_uy = BUU_y; }
  else { LB0_ly = BUL_y; LB0_uy = BLL_y; UB0_ly = BUU_y; UB0_uy = BLU_y; }

  // UA0, UB0
  if ((UA0_uy > b[1]) && (UB0_uy > a[1])) {
    if (((UA0_ly > b[1]) || in_voronoi(b[0], a[0], A0_dot_B1, aA1_dot_B1 - Tba[1] - b[1], A0_dot_B0,
                                        aA1_dot_B0 - Tba[0], -Tab[0] - bA0_dot_B1)) &&
        ((UB0_ly > a[1]) || in_voronoi(a[0], b[0], A1_dot_B0, Tab[1] - a[1] + bA1_dot_B1, A0_dot_B0,
                                        Tab[0] + bA0_dot_B1, Tba[0] - aA1_dot_B0))) {
      seg_coords(t, u, a[0], b[0], A0_dot_B0, Tab[0] + bA0_dot_B1, Tba[0] - aA1_dot_B0);
      D[0] = Tab[0] + Rab(0, 1) * b[1] + Rab(0, 0) * u - t;
      D[1] = Tab[1] + Rab(1, 1) * b[1] + Rab(1, 0) * u - a[1];
      D[2] = Tab[2] + Rab(2, 1) * b[1] + Rab(2, 0) * u;
      return finish(t, a[1]);
    }
  }
  // UA0, LB0
  if ((UA0_ly < 0) && (LB0_uy > a[1])) {
    if (((UA0_uy < 0) || in_voronoi(b[0], a[0], -A0_dot_B1, Tba[1] - aA1_dot_B1, A0_dot_B0,
                                     aA1_dot_B0 - Tba[0], -Tab[0])) &&
        ((LB0_ly > a[1]) || in_voronoi(a[0], b[0], A1_dot_B0, Tab[1] - a[1], A0_dot_B0, Tab[0],
                                        Tba[0] - aA1_dot_B0))) {
      seg_coords(t, u, a[0], b[0], A0_dot_B0, Tab[0], Tba[0] - aA1_dot_B0);
      D[0] = Tab[0] + Rab(0, 0) * u - t;
      D[1] = Tab[1] + Rab(1, 0) * u - a[1];
      D[2] = Tab[2] + Rab(2, 0) * u;
      return finish(t, a[1]);
    }
  }
  // LA0, UB0
  if ((LA0_uy > b[1]) && (UB0_ly < 0)) {
    if (((LA0_ly > b[1]) || in_voronoi(b[0], a[0], A0_dot_B1, -Tba[1] - b[1], A0_dot_B0, -Tba[0],
                                        -Tab[0] - bA0_dot_B1)) &&
        ((UB0_uy < 0) || in_voronoi(a[0], b[0], -A1_dot_B0, -Tab[1] - bA1_dot_B1, A0_dot_B0,
                                     Tab[0] + bA0_dot_B1, Tba[0]))) {
      seg_coords(t, u, a[0], b[0], A0_dot_B0, Tab[0] + bA0_dot_B1, Tba[0]);
      D[0] = Tab[0] + Rab(0, 1) * b[1] + Rab(0, 0) * u - t;
      D[1] = Tab[1] + Rab(1, 1) * b[1] + Rab(1, 0) * u;
      D[2] = Tab[2] + Rab(2, 1) * b[1] + Rab(2, 0) * u;
      return finish(t, 0);
    }
  }
  // LA0, LB0
  if ((LA0_ly < 0) && (LB0_ly < 0)) {
    if (((LA0_uy < 0) || in_voronoi(b[0], a[0], -A0_dot_B1, Tba[1], A0_dot_B0, -Tba[0], -Tab[0])) &&
        ((LB0_uy < 0) || in_voronoi(a[0], b[0], -A1_dot_B0, -Tab[1], A0_dot_B0, Tab[0], Tba[0]))) {
      seg_coords(t, u, a[0], b[0], A0_dot_B0, Tab[0], Tba[0]);
      D[0] = Tab[0] + Rab(0, 0) * u - t;
      D[1] = Tab[1] + Rab(1, 0) * u;
      D[2] = Tab[2] + Rab(2, 0) * u;
      return finish(t, 0);
    }
  }

  // no edges passed, take max separation along face normals
  double sep1, sep2;
  if (Tab[2] > 0.0) {
    sep1 = Tab[2];
    if (Rab(2, 0) < 0.0) sep1 += b[0] * Rab(2, 0);
    if (Rab(2, 1) < 0.0) sep1 += b[1] * Rab(2, 1);
  } else {
    sep1 = -Tab[2];
    if (Rab(2, 0) > 0.0) sep1 -= b[0] * Rab(2, 0);
    if (Rab(2, 1) > 0.0) sep1 -= b[1] * Rab(2, 1);
  }
  if (Tba[2] < 0) {
    sep2 = -Tba[2];
    if (Rab(0, 2) < 0.0) sep2 += a[0] * Rab(0, 2);
    if (Rab(1, 2) < 0.0) sep2 += a[1] * Rab(1, 2);
  } else {
    sep2 = Tba[2];
    if (Rab(0, 2) > 0.0) sep2 -= a[0] * Rab(0, 2);
    if (Rab(1, 2) > 0.0) sep2 -= a[1] * Rab(1, 2);
  }
  if (sep1 >= sep2 && sep1 >= 0) {
    if (Tab[2] > 0)
      D = mk(0, 0, sep1);
    else
      D = mk(0, 0, -sep1);
    if (P && Q) {
      *Q = D;
      *P = mk(0, 0, 0);
    }
  }
  if (sep2 >= sep1 && sep2 >= 0) {
    V3 Q_ = mk(Tab[0], Tab[1], Tab[2]);
    V3 P_;
    if (Tba[2] < 0) {
      P_[0] = Rab(0, 2) * sep2 + Tab[0];
      P_[1] = Rab(1, 2) * sep2 + Tab[1];
      P_[2] = Rab(2, 2) * sep2 + Tab[2];
    } else {
      P_[0] = -Rab(0, 2) * sep2 + Tab[0];
      P_[1] = -Rab(1, 2) * sep2 + Tab[1];
      P_[2] = -Rab(2, 2) * sep2 + Tab[2];
    }
    D = sub(Q_, P_);
    if (P && Q) {
      *P = P_;
      *Q = Q_;
    }
  }
  double sep = (sep1 > sep2 ? sep1 : sep2);
  return (sep > 0 ? sep : 0);
}

// math/bv/RSS-inl.h:1956-1974
double rss_distance(const M3& R0, const V3& T0, const RSS& b1, const RSS& b2, V3* P, V3* Q) {
  M3 R0b2 = mul(R0, b2.axis);
  M3 R = mulT(b1.axis, R0b2);
  V3 Ttemp = sub(add(mulv(R0, b2.To), T0), b1.To);
  V3 T = mulTv(b1.axis, Ttemp);
  double dist = rect_distance(R, T, b1.l, b2.l, P, Q);
  dist -= (b1.r + b2.r);
  return (dist < 0.0) ? 0.0 : dist;
}

// math/bv/RSS-inl.h:432-446 (RSS::distance member)
double rss_member_distance(const RSS& a, const RSS& b) {
  V3 t = sub(b.To, a.To);
  V3 T = mk(dot(col(a.axis, 0), t), dot(col(a.axis, 1), t), dot(col(a.axis, 2), t));
  M3 R = mulT(a.axis, b.axis);
  double dist = rect_distance(R, T, a.l, b.l, nullptr, nullptr);
  dist -= (a.r + b.r);
  return (dist < 0.0) ? 0.0 : dist;
}

// ===================================================================================
// Leaf tests
// ===================================================================================

// narrowphase/detail/traversal/collision/intersect-inl.h:1085-1106
static inline int project6(const V3& ax, const V3& p1, const V3& p2, const V3& p3, const V3& q1,
                           const V3& q2, const V3& q3) {
  double P1 = dot(ax, p1), P2 = dot(ax, p2), P3 = dot(ax, p3);
  double Q1 = dot(ax, q1), Q2 = dot(ax, q2), Q3 = dot(ax, q3);
  double mn1 = std::min(P1, std::min(P2, P3));
  double mx2 = std::max(Q1, std::max(Q2, Q3));
  if (mn1 > mx2) return 0;
  double mx1 = std::max(P1, std::max(P2, P3));
  double mn2 = std::min(Q1, std::min(Q2, Q3));
  if (mn2 > mx1) return 0;
  return 1;
}

// intersect-inl.h:597-617 then 727-798 (no contact information)
bool tri_intersect(const V3& P1, const V3& P2, const V3& P3, const V3& Q1, const V3& Q2,
                   const V3& Q3, const M3& R, const V3& T) {
  V3 Q1_ = add(mulv(R, Q1), T);
  V3 Q2_ = add(mulv(R, Q2), T);
  V3 Q3_ = add(mulv(R, Q3), T);
  V3 p1 = sub(P1, P1), p2 = sub(P2, P1), p3 = sub(P3, P1);
  V3 q1 = sub(Q1_, P1), q2 = sub(Q2_, P1), q3 = sub(Q3_, P1);
  V3 e1 = sub(p2, p1), e2 = sub(p3, p2);
  V3 n1 = cross(e1, e2);
  if (!project6(n1, p1, p2, p3, q1, q2, q3)) return false;
  V3 f1 = sub(q2, q1), f2 = sub(q3, q2);
  V3 m1 = cross(f1, f2);
  if (!project6(m1, p1, p2, p3, q1, q2, q3)) return false;
  V3 ef11 = cross(e1, f1);
  if (!project6(ef11, p1, p2, p3, q1, q2, q3)) return false;
  V3 ef12 = cross(e1, f2);
  if (!project6(ef12, p1, p2, p3, q1, q2, q3)) return false;
  V3 f3 = sub(q1, q3);
  V3 ef13 = cross(e1, f3);
  if (!project6(ef13, p1, p2, p3, q1, q2, q3)) return false;
  V3 ef21 = cross(e2, f1);
  if (!project6(ef21, p1, p2, p3, q1, q2, q3)) return false;
  V3 ef22 = cross(e2, f2);
  if (!project6(ef22, p1, p2, p3, q1, q2, q3)) return false;
  V3 ef23 = cross(e2, f3);
  if (!project6(ef23, p1, p2, p3, q1, q2, q3)) return false;
  V3 e3 = sub(p1, p3);
  V3 ef31 = cross(e3, f1);
  if (!project6(ef31, p1, p2, p3, q1, q2, q3)) return false;
  V3 ef32 = cross(e3, f2);
  if (!project6(ef32, p1, p2, p3, q1, q2, q3)) return false;
  V3 ef33 = cross(e3, f3);
  if (!project6(ef33, p1, p2, p3, q1, q2, q3)) return false;
  V3 g1 = cross(e1, n1);
  if (!project6(g1, p1, p2, p3, q1, q2, q3)) return false;
  V3 g2 = cross(e2, n1);
  if (!project6(g2, p1, p2, p3, q1, q2, q3)) return false;
  V3 g3 = cross(e3, n1);
  if (!project6(g3, p1, p2, p3, q1, q2, q3)) return false;
  V3 h1 = cross(f1, m1);
  if (!project6(h1, p1, p2, p3, q1, q2, q3)) return false;
  V3 h2 = cross(f2, m1);
  if (!project6(h2, p1, p2, p3, q1, q2, q3)) return false;
  V3 h3 = cross(f3, m1);
  if (!project6(h3, p1, p2, p3, q1, q2, q3)) return false;
  return true;
}

// intersect-inl.h:1040-1053 (buildTrianglePlane).  FCL leaves the plane unset for a
// triangle without a normal; this restatement gives it the zero plane.
static void build_triangle_plane(const V3& a, const V3& b, const V3& c, V3& n, double& t) {
  V3 m = cross(sub(b, a), sub(c, a));
  double sq = sqnorm(m);
  if (sq > 0) {
    double l = std::sqrt(sq);
    n = mk(m[0] / l, m[1] / l, m[2] / l);
    t = dot(n, a);
  } else {
    n = mk(0, 0, 0);
    t = 0;
  }
}

// intersect-inl.h:848-886 (computeDeepestPoints), getEpsilon() = 1e-5 (:1117-1120)
static void compute_deepest_points(const V3* pts, int np, const V3& n, double t, double& depth, V3* out,
                                   int& nout) {
  const double eps = 1e-5;
  double max_depth = -std::numeric_limits<double>::max();
  int k = 0, num_neg = 0, num_pos = 0, num_zero = 0;
  for (int i = 0; i < np; ++i) {
    double dist = -(dot(n, pts[i]) - t);  // -distanceToPlane (:1033-1037)
    if (dist > eps)
      num_pos++;
    else if (dist < -eps)
      num_neg++;
    else
      num_zero++;
    if (dist > max_depth) {
      max_depth = dist;
      k = 1;
      out[k - 1] = pts[i];
    } else if (dist + 1e-6 >= max_depth) {
      k++;
      out[k - 1] = pts[i];
    }
  }
  if (max_depth < -eps) k = 0;
  if (num_zero == 0 && ((num_neg == 0) || (num_pos == 0))) k = 0;
  depth = max_depth;
  nout = k;
}

// intersect-inl.h:800-844: the contact part of intersect_Triangle, on P and on Q
// already moved into P's frame (R Q + T)
int tri_contact_info(const V3 P[3], const V3 Qm[3], V3 cp[2], V3& normal, double& depth) {
  V3 n1, n2;
  double t1, t2;
  build_triangle_plane(P[0], P[1], P[2], n1, t1);
  build_triangle_plane(Qm[0], Qm[1], Qm[2], n2, t2);
  V3 deep1[3], deep2[3];
  int nd1 = 0, nd2 = 0;
  double pd1, pd2;
  compute_deepest_points(Qm, 3, n1, t1, pd2, deep2, nd2);
  compute_deepest_points(P, 3, n2, t2, pd1, deep1, nd1);
  int k;
  if (pd1 > pd2) {
    k = std::min(nd2, 2);
    for (int i = 0; i < k; ++i) cp[i] = deep2[i];
    normal = n1;
    depth = pd2;
  } else {
    k = std::min(nd1, 2);
    for (int i = 0; i < k; ++i) cp[i] = deep1[i];
    normal = neg(n2);
    depth = pd1;
  }
  return k;
}

// narrowphase/detail/primitive_shape_algorithm/triangle_distance-inl.h:54-167
static void seg_points(const V3& P, const V3& A, const V3& Q, const V3& B, V3& VEC, V3& X, V3& Y) {
  V3 T, TMP;
  double A_dot_A, B_dot_B, A_dot_B, A_dot_T, B_dot_T;
  T = sub(Q, P);
  A_dot_A = dot(A, A);
  B_dot_B = dot(B, B);
  A_dot_B = dot(A, B);
  A_dot_T = dot(A, T);
  B_dot_T = dot(B, T);
  double t, u;
  double denom = A_dot_A * B_dot_B - A_dot_B * A_dot_B;
  t = (A_dot_T * B_dot_B - B_dot_T * A_dot_B) / denom;
  if ((t < 0) || std::isnan(t)) t = 0;
  else if (t > 1) t = 1;
  u = (t * A_dot_B - B_dot_T) / B_dot_B;
  if ((u <= 0) || std::isnan(u)) {
    Y = Q;
    t = A_dot_T / A_dot_A;
    if ((t <= 0) || std::isnan(t)) {
      X = P;
      VEC = sub(Q, P);
    } else if (t >= 1) {
      X = add(P, A);
      VEC = sub(Q, X);
    } else {
      X = add(P, scale(A, t));
      TMP = cross(T, A);
      VEC = cross(A, TMP);
    }
  } else if (u >= 1) {
    Y = add(Q, B);
    t = (A_dot_B + A_dot_T) / A_dot_A;
    if ((t <= 0) || std::isnan(t)) {
      X = P;
      VEC = sub(Y, P);
    } else if (t >= 1) {
      X = add(P, A);
      VEC = sub(Y, X);
    } else {
      X = add(P, scale(A, t));
      T = sub(Y, P);
      TMP = cross(T, A);
      VEC = cross(A, TMP);
    }
  } else {
    Y = add(Q, scale(B, u));
    if ((t <= 0) || std::isnan(t)) {
      X = P;
      TMP = cross(T, B);
      VEC = cross(B, TMP);
    } else if (t >= 1) {
      X = add(P, A);
      T = sub(Q, X);
      TMP = cross(T, B);
      VEC = cross(B, TMP);
    } else {
      X = add(P, scale(A, t));
      VEC = cross(A, B);
      if (dot(VEC, T) < 0) VEC = scale(VEC, -1);
    }
  }
}

// triangle_distance-inl.h:170-394
double tri_distance(const V3 T1[3], const V3 T2[3], V3& P, V3& Q) {
  V3 Sv[3], Tv[3], VEC;
  Sv[0] = sub(T1[1], T1[0]);
  Sv[1] = sub(T1[2], T1[1]);
  Sv[2] = sub(T1[0], T1[2]);
  Tv[0] = sub(T2[1], T2[0]);
  Tv[1] = sub(T2[2], T2[1]);
  Tv[2] = sub(T2[0], T2[2]);
  V3 V, Z;
  V3 minP = mk(0, 0, 0), minQ = mk(0, 0, 0);
  double mindd;
  int shown_disjoint = 0;
  mindd = sqnorm(sub(T1[0], T2[0])) + 1;
  for (int i = 0; i < 3; ++i) {
    for (int j = 0; j < 3; ++j) {
      seg_points(T1[i], Sv[i], T2[j], Tv[j], VEC, P, Q);
      V = sub(Q, P);
      double dd = dot(V, V);
      if (dd <= mindd) {
        minP = P;
        minQ = Q;
        mindd = dd;
        Z = sub(T1[(i + 2) % 3], P);
        double a = dot(Z, VEC);
        Z = sub(T2[(j + 2) % 3], Q);
        double b = dot(Z, VEC);
        if ((a <= 0) && (b >= 0)) return std::sqrt(dd);
        double p = dot(V, VEC);
        if (a < 0) a = 0;
        if (b > 0) b = 0;
        if ((p - a + b) > 0) shown_disjoint = 1;
      }
    }
  }
  V3 Sn;
  double Snl;
  Sn = cross(Sv[0], Sv[1]);
  Snl = dot(Sn, Sn);
  if (Snl > 1e-15) {
    V3 Tp;
    V = sub(T1[0], T2[0]);
    Tp[0] = dot(V, Sn);
    V = sub(T1[0], T2[1]);
    Tp[1] = dot(V, Sn);
    V = sub(T1[0], T2[2]);
    Tp[2] = dot(V, Sn);
    int point = -1;
    if ((Tp[0] > 0) && (Tp[1] > 0) && (Tp[2] > 0)) {
      if (Tp[0] < Tp[1]) point = 0; else point = 1;
      if (Tp[2] < Tp[point]) point = 2;
    } else if ((Tp[0] < 0) && (Tp[1] < 0) && (Tp[2] < 0)) {
      if (Tp[0] > Tp[1]) point = 0; else point = 1;
      if (Tp[2] > Tp[point]) point = 2;
    }
    if (point >= 0) {
      shown_disjoint = 1;
      V = sub(T2[point], T1[0]);
      Z = cross(Sn, Sv[0]);
      if (dot(V, Z) > 0) {
        V = sub(T2[point], T1[1]);
        Z = cross(Sn, Sv[1]);
        if (dot(V, Z) > 0) {
          V = sub(T2[point], T1[2]);
          Z = cross(Sn, Sv[2]);
          if (dot(V, Z) > 0) {
            P = add(T2[point], scale(Sn, Tp[point] / Snl));
            Q = T2[point];
            return norm(sub(P, Q));
          }
        }
      }
    }
  }
  V3 Tn;
  double Tnl;
  Tn = cross(Tv[0], Tv[1]);
  Tnl = dot(Tn, Tn);
  if (Tnl > 1e-15) {
    V3 Sp;
    V = sub(T2[0], T1[0]);
    Sp[0] = dot(V, Tn);
    V = sub(T2[0], T1[1]);
    Sp[1] = dot(V, Tn);
    V = sub(T2[0], T1[2]);
    Sp[2] = dot(V, Tn);
    int point = -1;
    if ((Sp[0] > 0) && (Sp[1] > 0) && (Sp[2] > 0)) {
      if (Sp[0] < Sp[1]) point = 0; else point = 1;
      if (Sp[2] < Sp[point]) point = 2;
    } else if ((Sp[0] < 0) && (Sp[1] < 0) && (Sp[2] < 0)) {
      if (Sp[0] > Sp[1]) point = 0; else point = 1;
      if (Sp[2] > Sp[point]) point = 2;
    }
    if (point >= 0) {
      shown_disjoint = 1;
      V = sub(T1[point], T2[0]);
      Z = cross(Tn, Tv[0]);
      if (dot(V, Z) > 0) {
        V = sub(T1[point], T2[1]);
        Z = cross(Tn, Tv[1]);
        if (dot(V, Z) > 0) {
          V = sub(T1[point], T2[2]);
          Z = cross(Tn, Tv[2]);
          if (dot(V, Z) > 0) {
            P = T1[point];
            Q = add(T1[point], scale(Tn, Sp[point] / Tnl));
            return norm(sub(P, Q));
          }
        }
      }
    }
  }
  if (shown_disjoint) {
    P = minP;
    Q = minQ;
    return std::sqrt(mindd);
  } else
    return 0;
}

// ===================================================================================
// Queries
// ===================================================================================

namespace {

struct CollideCtx {
  const Mesh* m1;
  const Mesh* m2;
  M3 R;
  V3 T;
  size_t num_max_contacts;
  std::vector<int>* contacts;  // pairs (b1,b2)
  size_t n_contacts;
  std::vector<ContactOut>* full;  // enable_contact: contacts with their geometry
  Tf tf1;
  CollideStats st;
  bool can_stop() const { return n_contacts > 0 && num_max_contacts <= n_contacts; }
};

// mesh_collision_traversal_node-inl.h:494-500
inline bool bv_testing(CollideCtx& c, int b1, int b2) {
  c.st.num_bv_tests++;
  return !obb_overlap(c.R, c.T, c.m1->nodes[b1].obb, c.m2->nodes[b2].obb);
}

// mesh_collision_traversal_node-inl.h:526-620 (enable_contact = false branch)
inline void leaf_testing(CollideCtx& c, int b1, int b2) {
  c.st.num_leaf_tests++;
  const int p1 = -(c.m1->nodes[b1].first_child + 1);
  const int p2 = -(c.m2->nodes[b2].first_child + 1);
  const Tri& t1 = c.m1->tris[p1];
  const Tri& t2 = c.m2->tris[p2];
  const auto& v1 = c.m1->verts;
  const auto& v2 = c.m2->verts;
  if (tri_intersect(v1[t1.v[0]], v1[t1.v[1]], v1[t1.v[2]], v2[t2.v[0]], v2[t2.v[1]], v2[t2.v[2]],
                    c.R, c.T)) {
    if (c.full) {
      // enable_contact branch (mesh_collision_traversal_node-inl.h:579-600)
      V3 P[3] = {v1[t1.v[0]], v1[t1.v[1]], v1[t1.v[2]]};
      V3 Qm[3];
      for (int k = 0; k < 3; ++k) Qm[k] = add(mulv(c.R, v2[t2.v[k]]), c.T);
      V3 cp[2], nrm;
      double depth;
      size_t k = (size_t)tri_contact_info(P, Qm, cp, nrm, depth);
      if (c.num_max_contacts < c.n_contacts + k)
        k = (c.num_max_contacts > c.n_contacts) ? (c.num_max_contacts - c.n_contacts) : 0;
      for (size_t i = 0; i < k; ++i) {
        ContactOut o;
        o.b1 = p1;
        o.b2 = p2;
        o.pos = apply(c.tf1, cp[i]);
        o.normal = mulv(c.tf1.R, nrm);
        o.depth = depth;
        c.full->push_back(o);
        c.n_contacts++;
      }
      return;
    }
    if (c.n_contacts < c.num_max_contacts) {
      c.contacts->push_back(p1);
      c.contacts->push_back(p2);
      c.n_contacts++;
    }
  }
}

// bvh_collision_traversal_node-inl.h:77-89
inline bool first_over_second(const Mesh& m1, const Mesh& m2, int b1, int b2) {
  double sz1 = obb_size(m1.nodes[b1].obb);
  double sz2 = obb_size(m2.nodes[b2].obb);
  bool l1 = m1.nodes[b1].first_child < 0;
  bool l2 = m2.nodes[b2].first_child < 0;
  return l2 || (!l1 && (sz1 > sz2));
}

// traversal_recurse-inl.h:82-129 (collisionRecurse without front list)
void collision_recurse(CollideCtx& c, int b1, int b2) {
  bool l1 = c.m1->nodes[b1].first_child < 0;
  bool l2 = c.m2->nodes[b2].first_child < 0;
  if (l1 && l2) {
    if (bv_testing(c, b1, b2)) return;
    leaf_testing(c, b1, b2);
    return;
  }
  if (bv_testing(c, b1, b2)) return;
  if (first_over_second(*c.m1, *c.m2, b1, b2)) {
    int c1 = c.m1->nodes[b1].first_child, c2 = c1 + 1;
    collision_recurse(c, c1, b2);
    if (c.can_stop()) return;
    collision_recurse(c, c2, b2);
  } else {
    int c1 = c.m2->nodes[b2].first_child, c2 = c1 + 1;
    collision_recurse(c, b1, c1);
    if (c.can_stop()) return;
    collision_recurse(c, b1, c2);
  }
}

// BVHFrontList (geometry/bvh/detail/BVH_front.h): a std::list of (left, right, valid)
struct FrontNode {
  int left, right;
  bool valid;
};
using FrontList = std::list<FrontNode>;

// traversal_recurse-inl.h:82-129 (collisionRecurse with a front list): leaf pairs join the
// list before their BV test, disjoint pairs after it; no early stop while a list is given
void collision_recurse_front(CollideCtx& c, int b1, int b2, FrontList* fl) {
  bool l1 = c.m1->nodes[b1].first_child < 0;
  bool l2 = c.m2->nodes[b2].first_child < 0;
  if (l1 && l2) {
    if (fl) fl->push_back({b1, b2, true});
    if (bv_testing(c, b1, b2)) return;
    leaf_testing(c, b1, b2);
    return;
  }
  if (bv_testing(c, b1, b2)) {
    if (fl) fl->push_back({b1, b2, true});
    return;
  }
  if (first_over_second(*c.m1, *c.m2, b1, b2)) {
    int c1 = c.m1->nodes[b1].first_child, c2 = c1 + 1;
    collision_recurse_front(c, c1, b2, fl);
    if (c.can_stop() && !fl) return;
    collision_recurse_front(c, c2, b2, fl);
  } else {
    int c1 = c.m2->nodes[b2].first_child, c2 = c1 + 1;
    collision_recurse_front(c, b1, c1, fl);
    if (c.can_stop() && !fl) return;
    collision_recurse_front(c, b1, c2, fl);
  }
}

// traversal_recurse-inl.h:463-521 (propagateBVHFrontListCollisionRecurse): the loop walks
// the std::list while the recursions append to it, so appended entries are visited too
void propagate_front(CollideCtx& c, FrontList& fl) {
  FrontList append;
  for (auto it = fl.begin(); it != fl.end(); ++it) {
    const int b1 = it->left, b2 = it->right;
    const bool l1 = c.m1->nodes[b1].first_child < 0;
    const bool l2 = c.m2->nodes[b2].first_child < 0;
    if (l1 & l2) {
      it->valid = false;
      collision_recurse_front(c, b1, b2, &append);
    } else if (!bv_testing(c, b1, b2)) {
      it->valid = false;
      if (first_over_second(*c.m1, *c.m2, b1, b2)) {
        int c1 = c.m1->nodes[b1].first_child, c2 = c1 + 1;
        collision_recurse_front(c, c1, b2, &fl);
        collision_recurse_front(c, c2, b2, &fl);
      } else {
        int c1 = c.m2->nodes[b2].first_child, c2 = c1 + 1;
        collision_recurse_front(c, b1, c1, &fl);
        collision_recurse_front(c, b1, c2, &fl);
      }
    }
  }
  for (auto it = fl.begin(); it != fl.end();) {
    if (!it->valid)
      it = fl.erase(it);
    else
      ++it;
  }
  for (const auto& e : append) fl.push_back(e);
}

struct DistCtx {
  const Mesh* m1;
  const Mesh* m2;
  M3 R;
  V3 T;
  bool nearest;
  double min_distance;
  int b1, b2;
  V3 p1, p2;
  CollideStats st;
  // distance_result-inl.h:84-105 (strict "min_distance > distance")
  void update(double d, int i1, int i2, const V3& P, const V3& Q) {
    if (min_distance > d) {
      min_distance = d;
      b1 = i1;
      b2 = i2;
      if (nearest) {
        p1 = P;
        p2 = Q;
      }
    }
  }
  // mesh_distance_traversal_node-inl.h:147-153 with rel_err = abs_err = 0
  bool can_stop(double c) const { return (c >= min_distance - 0.0) && (c * (1 + 0.0) >= min_distance); }
};

// mesh_distance_traversal_node-inl.h:452-499 (leaf with a rigid transform)
void dist_leaf(DistCtx& c, int b1, int b2) {
  c.st.num_leaf_tests++;
  const int p1 = -(c.m1->nodes[b1].first_child + 1);
  const int p2 = -(c.m2->nodes[b2].first_child + 1);
  const Tri& t1 = c.m1->tris[p1];
  const Tri& t2 = c.m2->tris[p2];
  V3 A[3] = {c.m1->verts[t1.v[0]], c.m1->verts[t1.v[1]], c.m1->verts[t1.v[2]]};
  V3 B[3];
  for (int k = 0; k < 3; ++k) B[k] = add(mulv(c.R, c.m2->verts[t2.v[k]]), c.T);
  V3 P, Q;
  double d = tri_distance(A, B, P, Q);
  c.update(d, p1, p2, P, Q);
}

// traversal_recurse-inl.h:257-316 (distanceRecurse without front list)
void distance_recurse(DistCtx& c, int b1, int b2) {
  bool l1 = c.m1->nodes[b1].first_child < 0;
  bool l2 = c.m2->nodes[b2].first_child < 0;
  if (l1 && l2) {
    dist_leaf(c, b1, b2);
    return;
  }
  int a1, a2, c1, c2;
  if (first_over_second(*c.m1, *c.m2, b1, b2)) {
    a1 = c.m1->nodes[b1].first_child;
    a2 = b2;
    c1 = a1 + 1;
    c2 = b2;
  } else {
    a1 = b1;
    a2 = c.m2->nodes[b2].first_child;
    c1 = b1;
    c2 = a2 + 1;
  }
  c.st.num_bv_tests++;
  double d1 = rss_distance(c.R, c.T, c.m1->nodes[a1].rss, c.m2->nodes[a2].rss, nullptr, nullptr);
  c.st.num_bv_tests++;
  double d2 = rss_distance(c.R, c.T, c.m1->nodes[c1].rss, c.m2->nodes[c2].rss, nullptr, nullptr);
  if (d2 < d1) {
    if (!c.can_stop(d2)) distance_recurse(c, c1, c2);
    if (!c.can_stop(d1)) distance_recurse(c, a1, a2);
  } else {
    if (!c.can_stop(d1)) distance_recurse(c, a1, a2);
    if (!c.can_stop(d2)) distance_recurse(c, c1, c2);
  }
}

}  // namespace

// narrowphase/collision-inl.h:93-149 -> collision_func_matrix-inl.h:571-626 ->
// mesh_collision_traversal_node-inl.h:715-745 (relativeTransform, math/geometry-inl.h:655-682)
size_t collide_mesh(const Mesh& m1, const Tf& tf1, const Mesh& m2, const Tf& tf2,
                    size_t num_max_contacts, std::vector<int>& contacts, CollideStats* st) {
  if (num_max_contacts == 0) return 0;
  CollideCtx c;
  c.m1 = &m1;
  c.m2 = &m2;
  c.R = mulT(tf1.R, tf2.R);
  c.T = mulTv(tf1.R, sub(tf2.t, tf1.t));
  c.num_max_contacts = num_max_contacts;
  c.contacts = &contacts;
  c.n_contacts = 0;
  c.full = nullptr;
  c.tf1 = tf1;
  collision_recurse(c, 0, 0);
  if (st) *st = c.st;
  return c.n_contacts;
}

// collide(node, front_list) (collision_node-inl.h:72-82) on the oriented OBBRSS node
// initialised as collide_mesh does; front is the list in and out as (b1, b2) pairs
size_t collide_mesh_front(const Mesh& m1, const Tf& tf1, const Mesh& m2, const Tf& tf2, size_t num_max_contacts,
                          std::vector<int>& front, std::vector<int>& contacts, CollideStats* st) {
  CollideCtx c;
  c.m1 = &m1;
  c.m2 = &m2;
  c.R = mulT(tf1.R, tf2.R);
  c.T = mulTv(tf1.R, sub(tf2.t, tf1.t));
  c.num_max_contacts = num_max_contacts;
  c.contacts = &contacts;
  c.n_contacts = 0;
  c.full = nullptr;
  c.tf1 = tf1;
  FrontList fl;
  for (size_t k = 0; k + 1 < front.size(); k += 2) fl.push_back({front[k], front[k + 1], true});
  if (!fl.empty())
    propagate_front(c, fl);
  else
    collision_recurse_front(c, 0, 0, &fl);
  front.clear();
  for (const auto& e : fl) {
    front.push_back(e.left);
    front.push_back(e.right);
  }
  if (st) *st = c.st;
  return c.n_contacts;
}

size_t collide_mesh_contacts(const Mesh& m1, const Tf& tf1, const Mesh& m2, const Tf& tf2,
                             size_t num_max_contacts, std::vector<ContactOut>& out, CollideStats* st) {
  if (num_max_contacts == 0) return 0;
  CollideCtx c;
  c.m1 = &m1;
  c.m2 = &m2;
  c.R = mulT(tf1.R, tf2.R);
  c.T = mulTv(tf1.R, sub(tf2.t, tf1.t));
  c.num_max_contacts = num_max_contacts;
  c.contacts = nullptr;
  c.n_contacts = 0;
  c.full = &out;
  c.tf1 = tf1;
  collision_recurse(c, 0, 0);
  if (st) *st = c.st;
  return c.n_contacts;
}

// narrowphase/distance-inl.h:91-193 -> distance_func_matrix-inl.h:385-404 ->
// mesh_distance_traversal_node-inl.h:545-633 and collision_node-inl.h:136-147
double distance_mesh(const Mesh& m1, const Tf& tf1, const Mesh& m2, const Tf& tf2,
                     bool nearest_points, DistanceOut& out, CollideStats* st) {
  DistCtx c;
  c.m1 = &m1;
  c.m2 = &m2;
  // tf = tf1.inverse(Isometry) * tf2
  M3 Rinv = transpose(tf1.R);
  V3 tinv = neg(mulv(Rinv, tf1.t));
  c.R = mul(Rinv, tf2.R);
  c.T = add(mulv(Rinv, tf2.t), tinv);
  c.nearest = nearest_points;
  c.min_distance = std::numeric_limits<double>::max();
  c.b1 = c.b2 = -1;
  c.p1 = c.p2 = mk(0, 0, 0);
  // preprocess: triangle 0 against triangle 0
  {
    const Tri& t1 = m1.tris[0];
    const Tri& t2 = m2.tris[0];
    V3 A[3] = {m1.verts[t1.v[0]], m1.verts[t1.v[1]], m1.verts[t1.v[2]]};
    V3 B[3];
    for (int k = 0; k < 3; ++k) B[k] = add(mulv(c.R, m2.verts[t2.v[k]]), c.T);
    V3 P, Q;
    double d = tri_distance(A, B, P, Q);
    c.update(d, 0, 0, P, Q);
  }
  distance_recurse(c, 0, 0);
  out.min_distance = c.min_distance;
  out.b1 = c.b1;
  out.b2 = c.b2;
  if (nearest_points) {
    out.p1 = apply(tf1, c.p1);
    out.p2 = apply(tf1, c.p2);
  } else {
    out.p1 = out.p2 = mk(0, 0, 0);
  }
  if (st) *st = c.st;
  return c.min_distance;
}

}  // namespace oracle
