// BVHModel<OBBRSS> x convex shape, FP64 on the device: the shape's OBBRSS fitted to its
// bound vertices, the shape-triangle leaves of GJKSolver_indep and both traversals.
//
// Reference (FCL 0.7.0, paths relative to the FCL repository):
//   computeBV<OBBRSS>(shape, tf)    geometry/shape/utility-inl.h:123-133 (generic: fit the
//                                   bound vertices), math/bv/utility-inl.h:133-145, 247-260,
//                                   516-520; getBoundVertices in geometry/shape/*-inl.h
//   shapeTriangleIntersect          narrowphase/detail/gjk_solver_indep-inl.h:449-548
//   shapeTriangleDistance           narrowphase/detail/gjk_solver_indep-inl.h:946-1040
//   sphere-triangle                 narrowphase/detail/primitive_shape_algorithm/sphere_triangle-inl.h
//   Project::projectTriangle(p)     math/detail/project-inl.h:54-136
//   collide traversal               mesh_shape_collision_traversal_node-inl.h:191-265, 351-375;
//                                   traversal_recurse-inl.h:82-129
//   distance traversal              mesh_shape_distance_traversal_node-inl.h:164-226, 345-455;
//                                   traversal_recurse-inl.h:257-316
// Every operation follows the oracle restatement's order (no FMA), so results are
// bit-identical to it.
#pragma once
#include <cfloat>

#include "filter32.cuh"
#include "geom.cuh"
#include "shape_pair.cuh"

namespace fclgpu {

// ----------------------------------------------------------- shape bounding volume ----

FCLG_HD int bound_vertex_count(const DevShape& s) {
  switch (s.type) {
    case SHAPE_BOX: return 8;
    case SHAPE_SPHERE: return 12;
    case SHAPE_CAPSULE: return 36;
    case SHAPE_CYLINDER: return 12;
    case SHAPE_CONE: return 7;
    default: return s.vcnt;
  }
}

// local bound vertex i (getBoundVertices before the transform)
FCLG_HD D3v bound_vertex_local(const DevShape& s, const double* pool, int i) {
  switch (s.type) {
    case SHAPE_BOX: {
      const double a = s.p[0] / 2, b = s.p[1] / 2, c = s.p[2] / 2;
      return v3((i & 4) ? -a : a, (i & 2) ? -b : b, (i & 1) ? -c : c);
    }
    case SHAPE_SPHERE:
    case SHAPE_CAPSULE: {
      const double m = (1 + sqrt(5.0)) / 2.0;
      const double edge = s.p[0] * 6 / (sqrt(27.0) + sqrt(15.0));
      const double a = edge, b = m * edge;
      const double hl = s.type == SHAPE_CAPSULE ? s.p[1] * 0.5 : 0.0;
      if (i < 24) {
        const int k = i % 12;
        // icosahedron vertices; the capsule shifts the first 12 by +hl and the next 12 by -hl
        double x, y, z;
        switch (k) {
          case 0: x = 0; y = a; z = b; break;
          case 1: x = 0; y = -a; z = b; break;
          case 2: x = 0; y = a; z = -b; break;
          case 3: x = 0; y = -a; z = -b; break;
          case 4: x = a; y = b; z = 0; break;
          case 5: x = -a; y = b; z = 0; break;
          case 6: x = a; y = -b; z = 0; break;
          case 7: x = -a; y = -b; z = 0; break;
          case 8: x = b; y = 0; z = a; break;
          case 9: x = b; y = 0; z = -a; break;
          case 10: x = -b; y = 0; z = a; break;
          default: x = -b; y = 0; z = -a; break;
        }
        if (s.type == SHAPE_SPHERE) return v3(x, y, z);
        return v3(x, y, (i < 12) ? z + hl : z - hl);
      }
      // capsule rims
      const double r2 = s.p[0] * 2 / sqrt(3.0);
      const double c = 0.5 * r2, d = s.p[0];
      const int k = (i - 24) % 6;
      const double zz = (i < 30) ? hl : -hl;
      switch (k) {
        case 0: return v3(r2, 0.0, zz);
        case 1: return v3(c, d, zz);
        case 2: return v3(-c, d, zz);
        case 3: return v3(-r2, 0.0, zz);
        case 4: return v3(-c, -d, zz);
        default: return v3(c, -d, zz);
      }
    }
    case SHAPE_CYLINDER:
    case SHAPE_CONE: {
      const double hl = s.p[1] * 0.5;
      const double r2 = s.p[0] * 2 / sqrt(3.0);
      const double a = 0.5 * r2, b = s.p[0];
      if (s.type == SHAPE_CONE && i == 6) return v3(0.0, 0.0, hl);
      const double zz = (i < 6) ? -hl : hl;
      switch (i % 6) {
        case 0: return v3(r2, 0.0, zz);
        case 1: return v3(a, b, zz);
        case 2: return v3(-a, b, zz);
        case 3: return v3(-r2, 0.0, zz);
        case 4: return v3(-a, -b, zz);
        default: return v3(a, -b, zz);
      }
    }
    default: {
      const double* V = pool + 3 * (long long)(s.voff + i);
      return v3(V[0], V[1], V[2]);
    }
  }
}

struct ShapeBV {
  NodeD obb;  // axis, To, ext (child unused)
  double rTo[3], rl[2], rr;
};

// cyclic Jacobi (math/geometry-inl.h:477-558); evecs[k] = k-th eigenvector
FCLG_HD void jacobi3(const double C[3][3], double evals[3], double evecs[3][3]) {
  double R[3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) R[i][j] = C[i][j];
  double v[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
  double b[3], d[3], z[3];
  for (int p = 0; p < 3; ++p) {
    b[p] = d[p] = R[p][p];
    z[p] = 0;
  }
  auto rot = [](double& x, double& y, double s, double tau) {
    const double g = x, h = y;
    x = g - s * (h + g * tau);
    y = h + s * (g - h * tau);
  };
  for (int sweep = 0; sweep < 50; ++sweep) {
    double sm = 0;
    for (int p = 0; p < 3; ++p)
      for (int q = p + 1; q < 3; ++q) sm += fabs(R[p][q]);
    if (sm == 0.0) {
      for (int k = 0; k < 3; ++k) {
        evals[k] = d[k];
        for (int j = 0; j < 3; ++j) evecs[k][j] = v[j][k];
      }
      return;
    }
    const double tresh = (sweep < 3) ? 0.2 * sm / (3 * 3) : 0.0;
    for (int p = 0; p < 3; ++p) {
      for (int q = p + 1; q < 3; ++q) {
        const double g = 100.0 * fabs(R[p][q]);
        if (sweep > 3 && fabs(d[p]) + g == fabs(d[p]) && fabs(d[q]) + g == fabs(d[q])) {
          R[p][q] = 0.0;
        } else if (fabs(R[p][q]) > tresh) {
          double h = d[q] - d[p];
          double t;
          if (fabs(h) + g == fabs(h)) {
            t = (R[p][q]) / h;
          } else {
            const double theta = 0.5 * h / (R[p][q]);
            t = 1.0 / (fabs(theta) + sqrt(1.0 + theta * theta));
            if (theta < 0.0) t = -t;
          }
          const double c = 1.0 / sqrt(1 + t * t);
          const double s = t * c;
          const double tau = s / (1.0 + c);
          h = t * R[p][q];
          z[p] -= h;
          z[q] += h;
          d[p] -= h;
          d[q] += h;
          R[p][q] = 0.0;
          for (int j = 0; j < p; ++j) rot(R[j][p], R[j][q], s, tau);
          for (int j = p + 1; j < q; ++j) rot(R[p][j], R[j][q], s, tau);
          for (int j = q + 1; j < 3; ++j) rot(R[p][j], R[q][j], s, tau);
          for (int j = 0; j < 3; ++j) rot(v[j][p], v[j][q], s, tau);
        }
      }
    }
    for (int p = 0; p < 3; ++p) {
      b[p] += z[p];
      d[p] = b[p];
      z[p] = 0.0;
    }
  }
  // no convergence in 50 sweeps: FCL leaves its outputs unchanged (identity, zeros)
  for (int k = 0; k < 3; ++k) {
    evals[k] = 0.0;
    for (int j = 0; j < 3; ++j) evecs[k][j] = (k == j) ? 1.0 : 0.0;
  }
}

// ---- point-set fits (math/geometry-inl.h, math/bv/utility-inl.h) ----------------------
// pts(i) returns point i (FP64); every function reads the points in index order.

// getCovariance, point branch (math/geometry-inl.h:1383-1421)
template <class Pts>
FCLG_HD void covariance_of(Pts pts, int n, double C[3][3]) {
  double s1x = 0, s1y = 0, s1z = 0, sxx = 0, syy = 0, szz = 0, sxy = 0, sxz = 0, syz = 0;
  for (int i = 0; i < n; ++i) {
    const D3v p = pts(i);
    s1x += p.x;
    s1y += p.y;
    s1z += p.z;
    sxx += (p.x * p.x);
    syy += (p.y * p.y);
    szz += (p.z * p.z);
    sxy += (p.x * p.y);
    sxz += (p.x * p.z);
    syz += (p.y * p.z);
  }
  C[0][0] = sxx - s1x * s1x / n;
  C[1][1] = syy - s1y * s1y / n;
  C[2][2] = szz - s1z * s1z / n;
  C[0][1] = sxy - s1x * s1y / n;
  C[1][2] = syz - s1y * s1z / n;
  C[0][2] = sxz - s1x * s1z / n;
  C[1][0] = C[0][1];
  C[2][0] = C[0][2];
  C[2][1] = C[1][2];
}

// the (min, mid, max) order of three eigenvalues used by axisFromEigen and the merges
FCLG_HD void order3(const double e[3], int& lo, int& mid, int& hi) {
  if (e[0] > e[1]) {
    hi = 0;
    lo = 1;
  } else {
    lo = 0;
    hi = 1;
  }
  if (e[2] < e[lo]) {
    mid = lo;
    lo = 2;
  } else if (e[2] > e[hi]) {
    mid = hi;
    hi = 2;
  } else {
    mid = 2;
  }
}

FCLG_HD void set_axis9(double a9[9], const D3v ax[3]) {
  a9[0] = ax[0].x; a9[1] = ax[1].x; a9[2] = ax[2].x;
  a9[3] = ax[0].y; a9[4] = ax[1].y; a9[5] = ax[2].y;
  a9[6] = ax[0].z; a9[7] = ax[1].z; a9[8] = ax[2].z;
}

// getExtentAndCenter_pointcloud (math/geometry-inl.h:229-287)
template <class Pts>
FCLG_HD void extent_center_of(Pts pts, int n, const D3v ax[3], double To[3], double ext[3]) {
  double mn[3] = {DBL_MAX, DBL_MAX, DBL_MAX}, mx[3] = {-DBL_MAX, -DBL_MAX, -DBL_MAX};
  for (int i = 0; i < n; ++i) {
    const D3v p = pts(i);
    const double c3[3] = {dot(ax[0], p), dot(ax[1], p), dot(ax[2], p)};
    for (int j = 0; j < 3; ++j) {
      if (c3[j] > mx[j]) mx[j] = c3[j];
      if (c3[j] < mn[j]) mn[j] = c3[j];
    }
  }
  const double o0 = (mx[0] + mn[0]) / 2, o1 = (mx[1] + mn[1]) / 2, o2 = (mx[2] + mn[2]) / 2;
  const double a9[9] = {ax[0].x, ax[1].x, ax[2].x, ax[0].y, ax[1].y, ax[2].y, ax[0].z, ax[1].z, ax[2].z};
  for (int r = 0; r < 3; ++r) To[r] = (a9[3 * r] * o0 + a9[3 * r + 1] * o1) + a9[3 * r + 2] * o2;
  for (int k = 0; k < 3; ++k) ext[k] = (mx[k] - mn[k]) * 0.5;
}

// getRadiusAndOriginAndRectangleSize over the points projected onto ax
// (math/geometry-inl.h:709-990, point branch)
template <class Pts>
FCLG_HD void rss_fit_of(Pts pts, int n, const D3v ax[3], double rTo[3], double rl[2], double& rr) {
  auto proj = [&](int i) {
    const D3v p = pts(i);
    return v3(dot(ax[0], p), dot(ax[1], p), dot(ax[2], p));
  };
  const D3v p0 = proj(0);
  double minz = p0.z, maxz = p0.z;
  for (int i = 1; i < n; ++i) {
    const double zv = proj(i).z;
    if (zv < minz) minz = zv;
    else if (zv > maxz) maxz = zv;
  }
  const double r = 0.5 * (maxz - minz);
  const double radsqr = r * r;
  const double cz = 0.5 * (maxz + minz);
  auto cap = [&](const D3v& q) {
    const double dz = q.z - cz;
    return sqrt(fmax(radsqr - dz * dz, 0.0));
  };
  int imin = 0, imax = 0;
  double vmin = p0.x, vmax = p0.x;
  for (int i = 1; i < n; ++i) {
    const double xv = proj(i).x;
    if (xv < vmin) {
      imin = i;
      vmin = xv;
    } else if (xv > vmax) {
      imax = i;
      vmax = xv;
    }
  }
  D3v qa = proj(imin), qb = proj(imax);
  double minx = qa.x + cap(qa);
  double maxx = qb.x - cap(qb);
  for (int i = 0; i < n; ++i) {
    const D3v q = proj(i);
    if (q.x < minx) {
      const double x = q.x + cap(q);
      if (x < minx) minx = x;
    }
  }
  for (int i = 0; i < n; ++i) {
    const D3v q = proj(i);
    if (q.x > maxx) {
      const double x = q.x - cap(q);
      if (x > maxx) maxx = x;
    }
  }
  imin = imax = 0;
  vmin = vmax = p0.y;
  for (int i = 1; i < n; ++i) {
    const double yv = proj(i).y;
    if (yv < vmin) {
      imin = i;
      vmin = yv;
    } else if (yv > vmax) {
      imax = i;
      vmax = yv;
    }
  }
  qa = proj(imin);
  qb = proj(imax);
  double miny = qa.y + cap(qa);
  double maxy = qb.y - cap(qb);
  for (int i = 0; i < n; ++i) {
    const D3v q = proj(i);
    if (q.y < miny) {
      const double y = q.y + cap(q);
      if (y < miny) miny = y;
    }
  }
  for (int i = 0; i < n; ++i) {
    const D3v q = proj(i);
    if (q.y > maxy) {
      const double y = q.y - cap(q);
      if (y > maxy) maxy = y;
    }
  }
  const double a = sqrt(0.5);
  for (int i = 0; i < n; ++i) {
    const D3v q = proj(i);
    const double X = q.x, Y = q.y, Z = q.z;
    if (X > maxx) {
      if (Y > maxy) {
        const double dx = X - maxx, dy = Y - maxy;
        double u = dx * a + dy * a;
        const double tt = (a * u - dx) * (a * u - dx) + (a * u - dy) * (a * u - dy) + (cz - Z) * (cz - Z);
        u = u - sqrt(fmax(radsqr - tt, 0.0));
        if (u > 0) {
          maxx += u * a;
          maxy += u * a;
        }
      } else if (Y < miny) {
        const double dx = X - maxx, dy = Y - miny;
        double u = dx * a - dy * a;
        const double tt = (a * u - dx) * (a * u - dx) + (-a * u - dy) * (-a * u - dy) + (cz - Z) * (cz - Z);
        u = u - sqrt(fmax(radsqr - tt, 0.0));
        if (u > 0) {
          maxx += u * a;
          miny -= u * a;
        }
      }
    } else if (X < minx) {
      if (Y > maxy) {
        const double dx = X - minx, dy = Y - maxy;
        double u = dy * a - dx * a;
        const double tt = (-a * u - dx) * (-a * u - dx) + (a * u - dy) * (a * u - dy) + (cz - Z) * (cz - Z);
        u = u - sqrt(fmax(radsqr - tt, 0.0));
        if (u > 0) {
          minx -= u * a;
          maxy += u * a;
        }
      } else if (Y < miny) {
        const double dx = X - minx, dy = Y - miny;
        double u = -dx * a - dy * a;
        const double tt = (-a * u - dx) * (-a * u - dx) + (-a * u - dy) * (-a * u - dy) + (cz - Z) * (cz - Z);
        u = u - sqrt(fmax(radsqr - tt, 0.0));
        if (u > 0) {
          minx -= u * a;
          miny -= u * a;
        }
      }
    }
  }
  const double ox[3] = {ax[0].x * minx, ax[0].y * minx, ax[0].z * minx};
  const double oy[3] = {ax[1].x * miny, ax[1].y * miny, ax[1].z * miny};
  const double oz[3] = {ax[2].x * cz, ax[2].y * cz, ax[2].z * cz};
  for (int k = 0; k < 3; ++k) rTo[k] = (ox[k] + oy[k]) + oz[k];
  rl[0] = maxx - minx;
  if (rl[0] < 0) rl[0] = 0;
  rl[1] = maxy - miny;
  if (rl[1] < 0) rl[1] = 0;
  rr = r;
}


// fit<OBBRSS> of n >= 4 points: OBB fitn and RSS fitn share the covariance, the eigen
// decomposition and the axes (math/bv/utility-inl.h:133-145, 247-259)
template <class Pts>
FCLG_HD void fit_points_bv(Pts pts, int n, NodeD& obb, double rTo[3], double rl[2], double& rr) {
  double C[3][3];
  covariance_of(pts, n, C);
  double evals[3], evecs[3][3];
  jacobi3(C, evals, evecs);
  // axisFromEigen (math/geometry-inl.h:294-318)
  int lo, mid, hi;
  order3(evals, lo, mid, hi);
  const D3v a0 = v3(evecs[hi][0], evecs[hi][1], evecs[hi][2]);
  const D3v a1 = v3(evecs[mid][0], evecs[mid][1], evecs[mid][2]);
  const D3v ax[3] = {a0, a1, cross(a0, a1)};
  set_axis9(obb.axis, ax);
  extent_center_of(pts, n, ax, obb.To, obb.ext);
  obb.child = 0;
  obb.pad = 0;
  rss_fit_of(pts, n, ax, rTo, rl, rr);
}

// computeBV<OBBRSS>(shape, tf): OBB and RSS fitted to the world bound vertices
FCLG_HD void shape_obbrss(const DevShape& s, const double* pool, const M3<double>& R, const D3v& t, ShapeBV& bv) {
  const int n = bound_vertex_count(s);
  auto world = [&](int i) { return mulv(R, bound_vertex_local(s, pool, i)) + t; };
  fit_points_bv(world, n, bv.obb, bv.rTo, bv.rl, bv.rr);
}

// ------------------------------------------------------------- sphere-triangle ----

FCLG_HD D3v normalized3(const D3v& v) {
  const double z = sqnorm(v);
  if (z > 0) {
    const double n = sqrt(z);
    return v3(v.x / n, v.y / n, v.z / n);
  }
  return v;
}

FCLG_HD double segment_sqr_distance(const D3v& from, const D3v& to, const D3v& p, D3v& nearest) {
  D3v diff = p - from;
  const D3v v = to - from;
  double t = dot(v, diff);
  if (t > 0) {
    const double dotVV = dot(v, v);
    if (t < dotVV) {
      t /= dotVV;
      diff = diff - d3scale(v, t);
    } else {
      t = 1;
      diff = diff - v;
    }
  } else {
    t = 0;
  }
  nearest = from + d3scale(v, t);
  return dot(diff, diff);
}

FCLG_HD bool project_in_triangle(const D3v& p1, const D3v& p2, const D3v& p3, const D3v& normal, const D3v& p) {
  const D3v e1 = p2 - p1, e2 = p3 - p2, e3 = p1 - p3;
  const double r1 = dot(cross(e1, normal), p - p1);
  const double r2 = dot(cross(e2, normal), p - p2);
  const double r3 = dot(cross(e3, normal), p - p3);
  return (r1 > 0 && r2 > 0 && r3 > 0) || (r1 <= 0 && r2 <= 0 && r3 <= 0);
}

// sphereTriangleIntersect (sphere_triangle-inl.h:139-220); with the optional outputs the
// contact point, normal_ and penetration_depth it reports
FCLG_HD bool sphere_triangle_intersect(double radius, const D3v& center, const D3v& P1, const D3v& P2,
                                       const D3v& P3, D3v* contact_point = nullptr, D3v* normal_out = nullptr,
                                       double* depth = nullptr) {
  D3v normal = normalized3(cross(P2 - P1, P3 - P1));
  const double rwt = radius + DBL_EPSILON;
  double dfp = dot(center - P1, normal);
  if (dfp < 0) {
    dfp *= -1;
    normal = d3scale(normal, -1.0);
  }
  bool has_contact = false;
  D3v contact = v3(0.0, 0.0, 0.0);
  if (dfp < rwt) {
    if (project_in_triangle(P1, P2, P3, normal, center)) {
      has_contact = true;
      contact = center - d3scale(normal, dfp);
    } else {
      const double cap2 = rwt * rwt;
      D3v nearest;
      if (segment_sqr_distance(P1, P2, center, nearest) < cap2) {
        has_contact = true;
        contact = nearest;
      }
      if (segment_sqr_distance(P2, P3, center, nearest) < cap2) {
        has_contact = true;
        contact = nearest;
      }
      if (segment_sqr_distance(P3, P1, center, nearest) < cap2) {
        has_contact = true;
        contact = nearest;
      }
    }
  }
  if (!has_contact) return false;
  const D3v c2c = contact - center;
  const double dsq = sqnorm(c2c);
  if (!(dsq < rwt * rwt)) return false;
  if (contact_point) *contact_point = contact;
  if (dsq > 0) {
    if (normal_out) *normal_out = normalized3(c2c);
    if (depth) *depth = -(radius - sqrt(dsq));
  } else {
    if (normal_out) *normal_out = d3scale(normal, -1.0);
    if (depth) *depth = -radius;
  }
  return true;
}

struct ProjResult {
  double param[3];
  double sqr_distance;
  unsigned encode;
};

FCLG_HD ProjResult project_line_p(const D3v& a, const D3v& b, const D3v& p) {
  ProjResult res;
  res.param[0] = res.param[1] = res.param[2] = 0;
  res.sqr_distance = -1;
  res.encode = 0;
  const D3v d = b - a;
  const double l = sqnorm(d);
  if (l > 0) {
    const double t = dot(p - a, d);
    res.param[1] = (t >= l) ? 1 : ((t <= 0) ? 0 : (t / l));
    res.param[0] = 1 - res.param[1];
    if (t >= l) {
      res.sqr_distance = sqnorm(p - b);
      res.encode = 2;
    } else if (t <= 0) {
      res.sqr_distance = sqnorm(p - a);
      res.encode = 1;
    } else {
      res.sqr_distance = sqnorm((a + d3scale(d, res.param[1])) - p);
      res.encode = 3;
    }
  }
  return res;
}

FCLG_HD ProjResult project_triangle_p(const D3v& a, const D3v& b, const D3v& c, const D3v& p) {
  ProjResult res;
  res.param[0] = res.param[1] = res.param[2] = 0;
  res.sqr_distance = -1;
  res.encode = 0;
  const D3v vt[3] = {a, b, c};
  const D3v dl[3] = {a - b, b - c, c - a};
  const D3v n = cross(dl[0], dl[1]);
  const double l = sqnorm(n);
  if (l > 0) {
    double mindist = -1;
    for (int i = 0; i < 3; ++i) {
      if (dot(vt[i] - p, cross(dl[i], n)) > 0) {
        const int j = (i + 1) % 3;
        const ProjResult rl = project_line_p(vt[i], vt[j], p);
        if (mindist < 0 || rl.sqr_distance < mindist) {
          mindist = rl.sqr_distance;
          res.encode = ((rl.encode & 1) ? 1u << i : 0u) + ((rl.encode & 2) ? 1u << j : 0u);
          res.param[i] = rl.param[0];
          res.param[j] = rl.param[1];
          res.param[(j + 1) % 3] = 0;
        }
      }
    }
    if (mindist < 0) {
      const double dd = dot(a - p, n);
      const double s = sqrt(l);
      const D3v p_to_project = d3scale(n, dd / l);
      mindist = sqnorm(p_to_project);
      res.encode = 7;
      res.param[0] = d3norm(cross(dl[1], (b - p) - p_to_project)) / s;
      res.param[1] = d3norm(cross(dl[2], (c - p) - p_to_project)) / s;
      res.param[2] = 1 - res.param[0] - res.param[1];
    }
    res.sqr_distance = mindist;
  }
  return res;
}

// ------------------------------------------------------------- shape-triangle ----

FCLG_HD D3v iso_inv_apply(const M3<double>& R, const D3v& t, const D3v& p) {
  // Transform3::inverse(Isometry) * p = R^T p + (-(R^T t))
  const D3v rt = mulTv(R, t);
  return mulTv(R, p) + v3(-rt.x, -rt.y, -rt.z);
}

// shapeTriangleIntersect: triangle P (3 points, 9 doubles) in the mesh frame (Rm, tm)
FCLG_HD bool shape_triangle_intersect(const ShapeRef& A, const M3<double>& Rs, const D3v& ts, const double* P,
                                      const M3<double>& Rm, const D3v& tm, SimplexVert* V, EpaState* epa) {
  const D3v P1 = v3(P[0], P[1], P[2]), P2 = v3(P[3], P[4], P[5]), P3 = v3(P[6], P[7], P[8]);
  if (A.s.type == SHAPE_SPHERE)
    return sphere_triangle_intersect(A.s.p[0], ts, mulv(Rm, P1) + tm, mulv(Rm, P2) + tm, mulv(Rm, P3) + tm);
  ShapeRef B;
  B.s.type = SHAPE_TRIANGLE;
  B.s.voff = 0;
  B.s.vcnt = 3;
  B.s.pad = 0;
  B.s.p[0] = B.s.p[1] = B.s.p[2] = 0;
  B.verts = P;
  PairOut o;
  gjk_intersect(A, Rs, ts, B, Rm, tm, V, epa, o);
  return o.hit != 0;
}

// shapeTriangleIntersect without contact information (gjk_solver_indep-inl.h:
// shapeTriangleIntersect): the sphere closed form, else GJK on the shape and TriangleP;
// GJK Inside is an intersection, because the EPA that follows only fills the contact:
// EPA::evaluate never returns Failed (epa-inl.h sets Failed only in initialize, :118,
// and evaluate ends Valid/.../FallBack).  In two stages: stage 1 settles the sphere
// closed form (0 / 2) and the pairs the FP32 GJK certifies disjoint (0); the rest (1)
// need stage 2, the FP64 GJK.
FCLG_HD ShapeRef triangle_ref(const double* P) {
  ShapeRef B;
  B.s.type = SHAPE_TRIANGLE;
  B.s.voff = 0;
  B.s.vcnt = 3;
  B.s.pad = 0;
  B.s.p[0] = B.s.p[1] = B.s.p[2] = 0;
  B.verts = P;
  return B;
}
FCLG_HD int shape_triangle_stage1(const ShapeRef& A, const M3<double>& Rs, const D3v& ts, const double* P,
                                  const M3<double>& Rm, const D3v& tm) {
  if (A.s.type == SHAPE_SPHERE) {
    const D3v P1 = v3(P[0], P[1], P[2]), P2 = v3(P[3], P[4], P[5]), P3 = v3(P[6], P[7], P[8]);
    return sphere_triangle_intersect(A.s.p[0], ts, mulv(Rm, P1) + tm, mulv(Rm, P2) + tm, mulv(Rm, P3) + tm) ? 2
                                                                                                          : 0;
  }
  LeafCert32 c;
  leaf_cert_init(A, Rs, ts, Rm, tm, c);
  return leaf_cert_disjoint(c, P) ? 0 : 1;
}
// the same with the pair's certificate data prepared once (leaf_cert_init(A, Rs, ts, Rm, tm))
FCLG_HD int shape_triangle_stage1(LeafCert32& c, const ShapeRef& A, const D3v& ts, const double* P,
                                  const M3<double>& Rm, const D3v& tm) {
  if (A.s.type == SHAPE_SPHERE) {
    const D3v P1 = v3(P[0], P[1], P[2]), P2 = v3(P[3], P[4], P[5]), P3 = v3(P[6], P[7], P[8]);
    return sphere_triangle_intersect(A.s.p[0], ts, mulv(Rm, P1) + tm, mulv(Rm, P2) + tm, mulv(Rm, P3) + tm) ? 2
                                                                                                          : 0;
  }
  return leaf_cert_disjoint(c, P) ? 0 : 1;
}
// The contact MeshShapeCollisionTraversalNodeOBBRSS::leafTesting records with
// enable_contact (mesh_shape_collision_traversal_node-inl.h:233-244): shapeTriangleIntersect
// with its outputs, stored as Contact(..., contactp, -normal, penetration).  Sphere: the
// closed form's point and depth, its normal negated; the other shapes: the shape-pair
// EPA contact (ShapeTransformedTriangleIntersectIndepImpl, gjk_solver_indep-inl.h:449-505,
// reports -epa.normal, so the recorded normal is epa.normal).  pos/normal in the world frame.
FCLG_HD bool shape_triangle_contact(const ShapeRef& A, const M3<double>& Rs, const D3v& ts, const double* P,
                                    const M3<double>& Rm, const D3v& tm, SimplexVert* V, EpaState* epa, D3v& pos,
                                    D3v& normal, double& depth) {
  if (A.s.type == SHAPE_SPHERE) {
    const D3v P1 = v3(P[0], P[1], P[2]), P2 = v3(P[3], P[4], P[5]), P3 = v3(P[6], P[7], P[8]);
    D3v n;
    if (!sphere_triangle_intersect(A.s.p[0], ts, mulv(Rm, P1) + tm, mulv(Rm, P2) + tm, mulv(Rm, P3) + tm, &pos, &n,
                                   &depth))
      return false;
    normal = d3scale(n, -1.0);
    return true;
  }
  PairOut o;
  gjk_intersect(A, Rs, ts, triangle_ref(P), Rm, tm, V, epa, o);
  pos = o.point;
  normal = o.normal;
  depth = o.depth;
  return o.hit != 0;
}

FCLG_HD bool shape_triangle_gjk64(const ShapeRef& A, const M3<double>& Rs, const D3v& ts, const double* P,
                                  const M3<double>& Rm, const D3v& tm, SimplexVert* V) {
  GjkState g;
  make_minkowski(A, Rs, ts, triangle_ref(P), Rm, tm, g.shape);
  const SolverParams sp = solver_params();
  g.V = V;
  g.tolerance = sp.gjk_tolerance;
  return g.evaluate(d3neg(v3(1.0, 0.0, 0.0)), sp.gjk_max_iterations) == GJK_INSIDE;
}

// shape_triangle_gjk64 that gives up (false) once stop() reports that the answer is no
// longer needed (asked every 8 GJK iterations); otherwise the same result
template <class Stop>
FCLG_HD bool shape_triangle_gjk64_until(const ShapeRef& A, const M3<double>& Rs, const D3v& ts, const double* P,
                                        const M3<double>& Rm, const D3v& tm, SimplexVert* V, Stop stop) {
  GjkState g;
  make_minkowski(A, Rs, ts, triangle_ref(P), Rm, tm, g.shape);
  const SolverParams sp = solver_params();
  g.V = V;
  g.tolerance = sp.gjk_tolerance;
  g.begin(d3neg(v3(1.0, 0.0, 0.0)), sp.gjk_max_iterations);
  for (int it = 1; !g.step(); ++it)
    if ((it & 7) == 0 && stop()) return false;
  return g.finish() == GJK_INSIDE;
}

// shapeTriangleDistance; ps on the shape, pt on the triangle, in FCL's frames
FCLG_HD bool shape_triangle_distance(const ShapeRef& A, const M3<double>& Rs, const D3v& ts, const double* P,
                                     const M3<double>& Rm, const D3v& tm, SimplexVert* V, double& d, D3v& ps,
                                     D3v& pt) {
  const D3v P1 = v3(P[0], P[1], P[2]), P2 = v3(P[3], P[4], P[5]), P3 = v3(P[6], P[7], P[8]);
  if (A.s.type == SHAPE_SPHERE) {
    const D3v W1 = mulv(Rm, P1) + tm, W2 = mulv(Rm, P2) + tm, W3 = mulv(Rm, P3) + tm;
    const ProjResult r = project_triangle_p(W1, W2, W3, ts);
    const double rad = A.s.p[0];
    if (r.sqr_distance > rad * rad) {
      d = sqrt(r.sqr_distance) - rad;
      const D3v project_p = (d3scale(W1, r.param[0]) + d3scale(W2, r.param[1])) + d3scale(W3, r.param[2]);
      const D3v dir = normalized3(ts - project_p);
      ps = iso_inv_apply(Rs, ts, ts - d3scale(dir, rad));
      pt = iso_inv_apply(Rm, tm, project_p);
      return true;
    }
    d = -1;
    ps = pt = v3(0.0, 0.0, 0.0);
    return false;
  }
  ShapeRef B;
  B.s.type = SHAPE_TRIANGLE;
  B.s.voff = 0;
  B.s.vcnt = 3;
  B.s.pad = 0;
  B.s.p[0] = B.s.p[1] = B.s.p[2] = 0;
  B.verts = P;
  PairOut o;
  o.p1 = o.p2 = v3(0.0, 0.0, 0.0);
  gjk_distance(A, Rs, ts, B, Rm, tm, V, o);
  d = o.dist;
  ps = o.p1;
  pt = o.p2;
  return o.gstat == GJK_VALID;
}

// ------------------------------------------------------------------ traversals ----

struct MeshShapeOut {
  int32_t count;   // collide: contacts added (<= max_contacts)
  int32_t tri;     // distance: triangle of the minimum
  double dist;
  D3v pmesh, pshape;
  int64_t nbv, nleaf;
  int status;      // 1 = stack overflow
};

FCLG_HD void load_tri_local(const DevMesh& m, int prim, double* P) {
  const int32_t* t = m.tris + 3 * (long long)prim;
  for (int k = 0; k < 3; ++k) {
    const double* v = m.verts64 + 3 * (long long)t[k];
    P[3 * k] = v[0];
    P[3 * k + 1] = v[1];
    P[3 * k + 2] = v[2];
  }
}

// ------------------------------------------------- leaf collection (split form) ----
// The split form runs the BVH part of a pair on one thread and hands the leaf tests
// (GJK/EPA in FP64, the expensive part) to one thread each.  The set of leaves it
// collects makes the result equal to the serial traversal's:
//  * collide: every leaf whose OBB overlaps the shape's; the contact count is
//    min(max_contacts, intersecting leaves), which is what the serial DFS returns
//    whether or not it stops early;
//  * distance: the first triangle (FCL's preprocess seed), then every leaf whose RSS
//    lower bound does not exceed an upper bound of the pair's distance (the distance
//    from each visited triangle's centroid to the shape's support point toward it);
//    the minimiser is always among them.

// a point of the shape's surface toward world point c (support along the unit
// direction from the shape's origin), and its distance to c
FCLG_HD double shape_point_ub(const ShapeRef& A, const M3<double>& Rs, const D3v& ts, const D3v& c) {
  const D3v d = c - ts;
  const double len = d3norm(d);
  if (!(len > 0)) return 0.0;
  const D3v ld = mulTv(Rs, d3scale(d, 1.0 / len));
  const D3v p = mulv(Rs, shape_support(A, ld)) + ts;
  return d3norm(p - c);
}

FCLG_HD int float_bits(float x) {
#if defined(__CUDA_ARCH__)
  return __float_as_int(x);
#else
  int i;
  memcpy(&i, &x, 4);
  return i;
#endif
}

// The shape's BV as an FP32 node (axis column k with To[k], then the extents) for the
// filtered OBB test of filter32.cuh, with its per-pair error-bound state.
struct ShapeBV32 {
  QueryF32 q;
  float4 a0, a1, a2, ea;
};
FCLG_HD void make_shape_bv32(const M3<double>& Rm, const D3v& tm, const ShapeBV& bv, const DevMesh& m,
                             ShapeBV32& o) {
  const double* ax = bv.obb.axis;
  const double* to = bv.obb.To;
  make_query_f32(Rm, tm, sqrt((to[0] * to[0] + to[1] * to[1]) + to[2] * to[2]), m.cmax, 0.0, 0.0, o.q);
  o.a0 = make_float4((float)ax[0], (float)ax[3], (float)ax[6], (float)to[0]);
  o.a1 = make_float4((float)ax[1], (float)ax[4], (float)ax[7], (float)to[1]);
  o.a2 = make_float4((float)ax[2], (float)ax[5], (float)ax[8], (float)to[2]);
  o.ea = make_float4((float)bv.obb.ext[0], (float)bv.obb.ext[1], (float)bv.obb.ext[2], 0.f);
}

// BV test of MeshShapeCollisionTraversalNodeOBBRSS (mesh_shape_collision_traversal_node-inl.h):
// overlap(tf_mesh, shape BV, node) -- FP32 with a rigorous error bound, the FP64 test
// (same decision as FCL's) only where the bound cannot settle it.  Returns the node's
// first_child in *child when it overlaps.
FCLG_HD bool shape_node_overlap(const DevMesh& m, const M3<double>& Rm, const D3v& tm, const ShapeBV& bv,
                                const ShapeBV32& b32, int b, int* child) {
  const float4* pn = reinterpret_cast<const float4*>(m.nodes32) + 4 * (long long)b;
  const float4 x0 = FCLG_LDG(pn), x1 = FCLG_LDG(pn + 1), x2 = FCLG_LDG(pn + 2), eb = FCLG_LDG(pn + 3);
  int r = obb_overlap_f32(b32.q, b32.a0, b32.a1, b32.a2, b32.ea, x0, x1, x2, eb);
  if (r == F_UNSURE) r = obb_overlap64(Rm, tm, bv.obb, m.nodes64[b]) ? F_TRUE : F_FALSE;
  *child = float_bits(eb.w);
  return r == F_TRUE;
}

// Certified FP32 lower bound of the distance between a posed shape and a mesh node's
// RSS (the node bound of the warp mesh-shape distance).  Along a direction n (mesh
// frame; any n != 0 gives a valid bound):
//   dist(shape, RSS) >= (min_shape n.x - max_RSS n.y) / |n|,
//   max_RSS n.y = n.To + l0 max(0, n.a0) + l1 max(0, n.a1) + r|n|,
//   min_shape n.x = n.t - h_A(-Rrel^T n)   (h_A the shape's support function),
// with (Rrel, t) the shape's pose in the mesh frame and the RSS data FCL's FP64 values
// rounded to FP32.  Forward error (u = 2^-24, no fused multiply-adds): 3-term dot
// products of rounded inputs err by 4.1u ||n||_1 times the input's magnitude (|To| <=
// rmax, |t_i| <= T, unit axes); the clamped axis terms by 6.2u ||n||_1 l; r|n| by 4.1u
// ||n||_1 r; the rotated direction by 4.1u ||n||_1 per component, moving the support
// value by at most sqrt(3) that times the shape's radius rho, and the support value
// itself by under 10u ||n||_1 rho; the six final additions by 6u ||n||_1 times the sum
// of the magnitudes.  Together under 24u ||n||_1 (rmax + T + rho + l0 + l1 + r); the
// bound subtracts 32u ||n||_1 (...) (times 1.01 for its own rounding) and scales the
// quotient by 1 - 8u (the division and |n|).
struct MdPair {
  float Rr[9];  // the shape's rotation in the mesh frame (row-major)
  G3f tr;       // the shape's origin in the mesh frame
  float rho;    // the shape's radius bound
  float base;   // rmax + T + rho of the node error bound
};
FCLG_HD void md_pair(const DevMesh& m, const ShapeRef& A, const M3<double>& Rm, const D3v& tm, const M3<double>& Rs,
                     const D3v& ts, MdPair& q) {
  const M3<double> Rrel = mulT(Rm, Rs);
  const D3v trel = mulTv(Rm, ts - tm);
  for (int k = 0; k < 9; ++k) q.Rr[k] = (float)Rrel.m[k];
  q.tr = g3f((float)trel.x, (float)trel.y, (float)trel.z);
  q.rho = shape_radius32(A);
  const float T = fmaxf(fabsf(q.tr.x), fmaxf(fabsf(q.tr.y), fabsf(q.tr.z)));
  q.base = ((float)m.rmax * 1.0001f + T * 1.0001f) + q.rho;
}
FCLG_HD float md_node_lb(const ShapeRef& A, const MdPair& q, G3f n, float l0, float l1, float r, G3f To, G3f a0,
                         G3f a1) {
  const float nn = sqrtf(gdot(n, n));
  if (!(nn > 0.f)) return -INFINITY;
  const float n1 = (fabsf(n.x) + fabsf(n.y)) + fabsf(n.z);
  const float hR = ((gdot(n, To) + l0 * fmaxf(0.f, gdot(n, a0))) + l1 * fmaxf(0.f, gdot(n, a1))) + r * nn;
  const G3f uA = rot32T(q.Rr, n);
  const G3f mu = g3f(-uA.x, -uA.y, -uA.z);
  const float hA = gdot(mu, support32(A, mu));
  const float gap = (gdot(n, q.tr) - hA) - hR;
  const float E = 1.90734863e-06f * n1 * ((q.base + l0) + (l1 + r)) * 1.01f;  // 32u
  const float g = gap - E;
  if (!(g > 0.f)) return -INFINITY;
  return g * (1.f - 4.76837158e-07f) / nn;  // 1 - 8u
}
// The larger of the bounds along two directions: from the RSS rectangle's point nearest
// to the shape's origin to that origin, and dir when have_dir.
FCLG_HD float md_node_bound(const float4* rss32, int b, const ShapeRef& A, const MdPair& q, bool have_dir, G3f dir) {
  const float4 c0 = FCLG_LDG(rss32 + 5 * (long long)b), c1 = FCLG_LDG(rss32 + 5 * (long long)b + 1);
  const float4 x0 = FCLG_LDG(rss32 + 5 * (long long)b + 2), x1 = FCLG_LDG(rss32 + 5 * (long long)b + 3);
  const float4 x2 = FCLG_LDG(rss32 + 5 * (long long)b + 4);
  const G3f To = g3f(c0.x, c0.y, c0.z), a0 = g3f(x0.x, x0.y, x0.z), a1 = g3f(x1.x, x1.y, x1.z);
  const float r = c0.w, l0 = c1.x, l1 = c1.y;
  const G3f d = q.tr - To;
  const float s = fminf(fmaxf(gdot(d, a0), 0.f), l0), t = fminf(fmaxf(gdot(d, a1), 0.f), l1);
  G3f n = d - a0 * s - a1 * t;
  if (!(gdot(n, n) > 1e-12f * (gdot(d, d) + 1e-30f))) {
    const G3f a2 = g3f(x2.x, x2.y, x2.z);
    n = gdot(d, a2) >= 0.f ? a2 : g3f(-a2.x, -a2.y, -a2.z);
  }
  float lb = md_node_lb(A, q, n, l0, l1, r, To, a0, a1);
  if (have_dir) lb = fmaxf(lb, md_node_lb(A, q, dir, l0, l1, r, To, a0, a1));
  return lb;
}

// Resumable collide DFS of one pair over an explicit stack (stack[0..sp), capacity cap):
// visits nodes in FCL's order and emits overlapping leaves until max_emit leaves have
// been emitted, max_visits nodes have been tested or the stack is empty.  Returns the
// number emitted, or -1 when the stack would overflow.
template <class Emit>
FCLG_HD int mesh_shape_dfs_resume(const DevMesh& m, const M3<double>& Rm, const D3v& tm, const ShapeBV& bv,
                                  const ShapeBV32& b32, int* stack, int& sp, int cap, int max_emit, int max_visits,
                                  Emit emit) {
  int ne = 0;
  for (int visits = 0; sp > 0 && ne < max_emit && visits < max_visits; ++visits) {
    const int b = stack[--sp];
    int child;
    if (!shape_node_overlap(m, Rm, tm, bv, b32, b, &child)) continue;
    if (child < 0) {
      emit(ne++, -(child + 1));
      continue;
    }
    if (sp + 2 > cap) return -1;
    stack[sp++] = child + 1;
    stack[sp++] = child;
  }
  return ne;
}

template <int STACK, class Emit>
FCLG_HD int mesh_shape_collect_distance(const DevMesh& m, const M3<double>& Rm, const D3v& tm, const ShapeRef& A,
                                        const M3<double>& Rs, const D3v& ts, const ShapeBV& bv, double* ub_out,
                                        Emit emit) {
  M3<double> Ab;
  for (int i = 0; i < 9; ++i) Ab.m[i] = bv.obb.axis[i];
  const D3v Tob = v3(bv.rTo[0], bv.rTo[1], bv.rTo[2]);
  auto tri_ub = [&](int prim) {
    double P[9];
    load_tri_local(m, prim, P);
    const D3v c = mulv(Rm, v3((P[0] + P[3] + P[6]) / 3.0, (P[1] + P[4] + P[7]) / 3.0, (P[2] + P[5] + P[8]) / 3.0)) + tm;
    return shape_point_ub(A, Rs, ts, c);
  };
  auto bvd = [&](int b) {
    const RssD& rs = m.rss64[b];
    M3<double> A2;
    for (int i = 0; i < 9; ++i) A2.m[i] = rs.axis[i];
    return rss_distance<double>(Rm, tm, Ab, Tob, bv.rl, bv.rr, A2, v3(rs.To[0], rs.To[1], rs.To[2]), rs.l, rs.r);
  };
  double ub = tri_ub(0);
  emit(0, -1.0);  // the seed triangle is always evaluated
  int stack[STACK];
  double sd[STACK];
  int sp = 0;
  stack[sp] = 0;
  sd[sp] = -1.0;
  ++sp;
  while (sp > 0) {
    --sp;
    const int b = stack[sp];
    const double lb = sd[sp];
    if (lb > ub) continue;
    const int child = m.nodes64[b].child;
    if (child < 0) {
      const int prim = -(child + 1);
      if (prim != 0) {
        emit(prim, lb);
        ub = fmin(ub, tri_ub(prim));
      }
      continue;
    }
    const double d1 = bvd(child), d2 = bvd(child + 1);
    if (sp + 2 > STACK) return 1;
    if (d2 < d1) {
      stack[sp] = child;
      sd[sp] = d1;
      ++sp;
      stack[sp] = child + 1;
      sd[sp] = d2;
      ++sp;
    } else {
      stack[sp] = child + 1;
      sd[sp] = d2;
      ++sp;
      stack[sp] = child;
      sd[sp] = d1;
      ++sp;
    }
  }
  *ub_out = ub;
  return 0;
}

template <int STACK>
FCLG_HD void mesh_shape_collide(const DevMesh& m, const M3<double>& Rm, const D3v& tm, const ShapeRef& A,
                                const M3<double>& Rs, const D3v& ts, int max_contacts, MeshShapeOut& o) {
  ShapeBV bv;
  shape_obbrss(A.s, A.verts, Rs, ts, bv);
  SimplexVert V[kSimplexSlots];
  EpaState epa;
  int stack[STACK];
  int sp = 0;
  stack[sp++] = 0;
  o.count = 0;
  while (sp > 0) {
    if (o.count > 0 && max_contacts <= o.count) break;  // canStop
    const int b = stack[--sp];
    const NodeD nd = m.nodes64[b];
    ++o.nbv;
    if (!obb_overlap64(Rm, tm, bv.obb, nd)) continue;  // model2_bv first, mesh node second
    if (nd.child < 0) {
      ++o.nleaf;
      const int prim = -(nd.child + 1);
      double P[9];
      load_tri_local(m, prim, P);
      if (shape_triangle_intersect(A, Rs, ts, P, Rm, tm, V, &epa) && max_contacts > o.count) ++o.count;
      continue;
    }
    if (sp + 2 > STACK) {
      o.status = 1;
      break;
    }
    stack[sp++] = nd.child + 1;
    stack[sp++] = nd.child;
  }
}

template <int STACK>
FCLG_HD void mesh_shape_distance(const DevMesh& m, const M3<double>& Rm, const D3v& tm, const ShapeRef& A,
                                 const M3<double>& Rs, const D3v& ts, MeshShapeOut& o) {
  ShapeBV bv;
  shape_obbrss(A.s, A.verts, Rs, ts, bv);
  M3<double> Ab;
  for (int i = 0; i < 9; ++i) Ab.m[i] = bv.obb.axis[i];
  const D3v Tob = v3(bv.rTo[0], bv.rTo[1], bv.rTo[2]);
  SimplexVert V[kSimplexSlots];
  o.dist = DBL_MAX;
  o.tri = -1;
  auto leaf = [&](int prim) {
    double P[9];
    load_tri_local(m, prim, P);
    double d;
    D3v ps, pt;
    shape_triangle_distance(A, Rs, ts, P, Rm, tm, V, d, ps, pt);
    if (o.dist > d) {
      o.dist = d;
      o.tri = prim;
      o.pmesh = pt;
      o.pshape = ps;
    }
  };
  auto bvd = [&](int b) {
    ++o.nbv;
    const RssD& rs = m.rss64[b];
    M3<double> A2;
    for (int i = 0; i < 9; ++i) A2.m[i] = rs.axis[i];
    return rss_distance<double>(Rm, tm, Ab, Tob, bv.rl, bv.rr, A2, v3(rs.To[0], rs.To[1], rs.To[2]), rs.l, rs.r);
  };
  leaf(0);  // preprocess seeds with the first triangle
  int stack[STACK];
  double sd[STACK];
  int sp = 0;
  stack[sp] = 0;
  sd[sp] = -1.0;  // the root is entered unconditionally
  ++sp;
  while (sp > 0) {
    --sp;
    const int b = stack[sp];
    if (!(sd[sp] < 0.0) && sd[sp] >= o.dist) continue;  // canStop(d): d >= min_distance
    const int child = m.nodes64[b].child;
    if (child < 0) {
      ++o.nleaf;
      leaf(-(child + 1));
      continue;
    }
    const double d1 = bvd(child), d2 = bvd(child + 1);
    if (sp + 2 > STACK) {
      o.status = 1;
      break;
    }
    // visit the nearer child first: push it last
    if (d2 < d1) {
      stack[sp] = child;
      sd[sp] = d1;
      ++sp;
      stack[sp] = child + 1;
      sd[sp] = d2;
      ++sp;
    } else {
      stack[sp] = child + 1;
      sd[sp] = d2;
      ++sp;
      stack[sp] = child;
      sd[sp] = d1;
      ++sp;
    }
  }
}

}  // namespace fclgpu
