// FP64 mesh-shape oracle (see oracle_meshshape.h).  TEST INFRASTRUCTURE ONLY.
#include "oracle_meshshape.h"

#include <cmath>
#include <limits>

namespace oracle {

namespace {

// Transform3::inverse(Eigen::Isometry): (R^T, -(R^T t))
Tf isometry_inverse(const Tf& f) {
  Tf r;
  r.R = transpose(f.R);
  r.t = neg(mulv(r.R, f.t));
  return r;
}

// Eigen normalize(): divide by the norm when the squared norm is positive
V3 normalized(const V3& v) {
  const double z = sqnorm(v);
  if (z > 0) {
    const double n = std::sqrt(z);
    return mk(v[0] / n, v[1] / n, v[2] / n);
  }
  return v;
}

// sphere_triangle-inl.h: segmentSqrDistance
double segment_sqr_distance(const V3& from, const V3& to, const V3& p, V3& nearest) {
  V3 diff = sub(p, from);
  const V3 v = sub(to, from);
  double t = dot(v, diff);
  if (t > 0) {
    const double dotVV = dot(v, v);
    if (t < dotVV) {
      t /= dotVV;
      diff = sub(diff, scale(v, t));
    } else {
      t = 1;
      diff = sub(diff, v);
    }
  } else {
    t = 0;
  }
  nearest = add(from, scale(v, t));
  return dot(diff, diff);
}

// sphere_triangle-inl.h: projectInTriangle
bool project_in_triangle(const V3& p1, const V3& p2, const V3& p3, const V3& normal, const V3& p) {
  const V3 e1 = sub(p2, p1), e2 = sub(p3, p2), e3 = sub(p1, p3);
  const V3 p1p = sub(p, p1), p2p = sub(p, p2), p3p = sub(p, p3);
  const double r1 = dot(cross(e1, normal), p1p);
  const double r2 = dot(cross(e2, normal), p2p);
  const double r3 = dot(cross(e3, normal), p3p);
  return (r1 > 0 && r2 > 0 && r3 > 0) || (r1 <= 0 && r2 <= 0 && r3 <= 0);
}

// geometry/shape/sphere-inl.h:95-120 and capsule-inl.h:107-160 share the icosahedron
// of edge 6 r / (sqrt(27) + sqrt(15)); m = golden ratio
void icosa_params(double radius, double& a, double& b) {
  const double m = (1 + std::sqrt(5.0)) / 2.0;
  const double edge = radius * 6 / (std::sqrt(27.0) + std::sqrt(15.0));
  a = edge;
  b = m * edge;
}

}  // namespace

std::vector<V3> bound_vertices(const Shape& s, const Tf& tf) {
  std::vector<V3> r;
  auto put = [&](double x, double y, double z) { r.push_back(apply(tf, mk(x, y, z))); };
  switch (s.type) {
    case SH_BOX: {
      const double a = s.p[0] / 2, b = s.p[1] / 2, c = s.p[2] / 2;
      put(a, b, c); put(a, b, -c); put(a, -b, c); put(a, -b, -c);
      put(-a, b, c); put(-a, b, -c); put(-a, -b, c); put(-a, -b, -c);
      break;
    }
    case SH_SPHERE: {
      double a, b;
      icosa_params(s.p[0], a, b);
      put(0, a, b); put(0, -a, b); put(0, a, -b); put(0, -a, -b);
      put(a, b, 0); put(-a, b, 0); put(a, -b, 0); put(-a, -b, 0);
      put(b, 0, a); put(b, 0, -a); put(-b, 0, a); put(-b, 0, -a);
      break;
    }
    case SH_CAPSULE: {
      const double hl = s.p[1] * 0.5;
      double a, b;
      icosa_params(s.p[0], a, b);
      const double r2 = s.p[0] * 2 / std::sqrt(3.0);
      put(0, a, b + hl); put(0, -a, b + hl); put(0, a, -b + hl); put(0, -a, -b + hl);
      put(a, b, hl); put(-a, b, hl); put(a, -b, hl); put(-a, -b, hl);
      put(b, 0, a + hl); put(b, 0, -a + hl); put(-b, 0, a + hl); put(-b, 0, -a + hl);
      put(0, a, b - hl); put(0, -a, b - hl); put(0, a, -b - hl); put(0, -a, -b - hl);
      put(a, b, -hl); put(-a, b, -hl); put(a, -b, -hl); put(-a, -b, -hl);
      put(b, 0, a - hl); put(b, 0, -a - hl); put(-b, 0, a - hl); put(-b, 0, -a - hl);
      const double c = 0.5 * r2, d = s.p[0];
      put(r2, 0, hl); put(c, d, hl); put(-c, d, hl); put(-r2, 0, hl); put(-c, -d, hl); put(c, -d, hl);
      put(r2, 0, -hl); put(c, d, -hl); put(-c, d, -hl); put(-r2, 0, -hl); put(-c, -d, -hl); put(c, -d, -hl);
      break;
    }
    case SH_CYLINDER: {
      const double hl = s.p[1] * 0.5;
      const double r2 = s.p[0] * 2 / std::sqrt(3.0);
      const double a = 0.5 * r2, b = s.p[0];
      put(r2, 0, -hl); put(a, b, -hl); put(-a, b, -hl); put(-r2, 0, -hl); put(-a, -b, -hl); put(a, -b, -hl);
      put(r2, 0, hl); put(a, b, hl); put(-a, b, hl); put(-r2, 0, hl); put(-a, -b, hl); put(a, -b, hl);
      break;
    }
    case SH_CONE: {
      const double hl = s.p[1] * 0.5;
      const double r2 = s.p[0] * 2 / std::sqrt(3.0);
      const double a = 0.5 * r2, b = s.p[0];
      put(r2, 0, -hl); put(a, b, -hl); put(-a, b, -hl); put(-r2, 0, -hl); put(-a, -b, -hl); put(a, -b, -hl);
      put(0, 0, hl);
      break;
    }
    default:  // SH_CONVEX
      for (int i = 0; i < s.nverts; ++i) r.push_back(apply(tf, s.verts[i]));
      break;
  }
  return r;
}

void shape_obbrss(const Shape& s, const Tf& tf, OBB& obb, RSS& rss) {
  const std::vector<V3> ps = bound_vertices(s, tf);
  fit_points_obbrss(ps.data(), (int)ps.size(), obb, rss);
}

bool sphere_triangle_intersect(double radius, const V3& center, const V3& P1, const V3& P2, const V3& P3,
                               V3* contact_point, V3* normal_out, double* depth) {
  V3 normal = normalized(cross(sub(P2, P1), sub(P3, P1)));
  const double rwt = radius + std::numeric_limits<double>::epsilon();
  const V3 p1_to_center = sub(center, P1);
  double dfp = dot(p1_to_center, normal);
  if (dfp < 0) {
    dfp *= -1;
    normal = scale(normal, -1);
  }
  const bool inside_plane = dfp < rwt;
  bool has_contact = false;
  const double qnan = std::numeric_limits<double>::quiet_NaN();
  V3 contact = mk(qnan, qnan, qnan);
  if (inside_plane) {
    if (project_in_triangle(P1, P2, P3, normal, center)) {
      has_contact = true;
      contact = sub(center, scale(normal, dfp));
    } else {
      const double cap2 = rwt * rwt;
      V3 nearest;
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
  if (has_contact) {
    const V3 c2c = sub(contact, center);
    const double dsq = sqnorm(c2c);
    if (dsq < rwt * rwt) {
      if (dsq > 0) {
        const double d = std::sqrt(dsq);
        if (normal_out) *normal_out = normalized(c2c);
        if (contact_point) *contact_point = contact;
        if (depth) *depth = -(radius - d);
      } else {
        if (normal_out) *normal_out = scale(normal, -1);
        if (contact_point) *contact_point = contact;
        if (depth) *depth = -radius;
      }
      return true;
    }
  }
  return false;
}

bool shape_triangle_contact(const Shape& s, const Tf& tfs, const V3& P1, const V3& P2, const V3& P3, const Tf& tfm,
                            V3& pos, V3& normal, double& depth) {
  if (s.type == SH_SPHERE) {
    V3 n;
    if (!sphere_triangle_intersect(s.p[0], tfs.t, apply(tfm, P1), apply(tfm, P2), apply(tfm, P3), &pos, &n, &depth))
      return false;
    normal = scale(n, -1);  // the leaf records -normal (mesh_shape_collision_traversal_node-inl.h:97-102)
    return true;
  }
  const V3 tv[3] = {P1, P2, P3};
  Shape tri;
  tri.type = SH_TRIANGLE;
  tri.verts = tv;
  tri.nverts = 3;
  int gs, es;
  // EPA's contact: normal epa.normal (the leaf's -(-epa.normal)), point
  // tf1 (w0 - epa.normal epa.depth / 2), depth -epa.depth (gjk_solver_indep-inl.h:488-497)
  return gjk_intersect(s, tfs, tri, tfm, &normal, &pos, &depth, &gs, &es);
}

ProjectResult project_line_p(const V3& a, const V3& b, const V3& p) {
  ProjectResult res;
  const V3 d = sub(b, a);
  const double l = sqnorm(d);
  if (l > 0) {
    const double t = dot(sub(p, a), d);
    res.parameterization[1] = (t >= l) ? 1 : ((t <= 0) ? 0 : (t / l));
    res.parameterization[0] = 1 - res.parameterization[1];
    if (t >= l) {
      res.sqr_distance = sqnorm(sub(p, b));
      res.encode = 2;
    } else if (t <= 0) {
      res.sqr_distance = sqnorm(sub(p, a));
      res.encode = 1;
    } else {
      res.sqr_distance = sqnorm(sub(add(a, scale(d, res.parameterization[1])), p));
      res.encode = 3;
    }
  }
  return res;
}

ProjectResult project_triangle_p(const V3& a, const V3& b, const V3& c, const V3& p) {
  ProjectResult res;
  static const int nexti[3] = {1, 2, 0};
  const V3* vt[3] = {&a, &b, &c};
  const V3 dl[3] = {sub(a, b), sub(b, c), sub(c, a)};
  const V3 n = cross(dl[0], dl[1]);
  const double l = sqnorm(n);
  if (l > 0) {
    double mindist = -1;
    for (int i = 0; i < 3; ++i) {
      if (dot(sub(*vt[i], p), cross(dl[i], n)) > 0) {
        const int j = nexti[i];
        const ProjectResult rl = project_line_p(*vt[i], *vt[j], p);
        if (mindist < 0 || rl.sqr_distance < mindist) {
          mindist = rl.sqr_distance;
          res.encode = (unsigned)(((rl.encode & 1) ? 1 << i : 0) + ((rl.encode & 2) ? 1 << j : 0));
          res.parameterization[i] = rl.parameterization[0];
          res.parameterization[j] = rl.parameterization[1];
          res.parameterization[nexti[j]] = 0;
        }
      }
    }
    if (mindist < 0) {
      const double d = dot(sub(a, p), n);
      const double s = std::sqrt(l);
      const V3 p_to_project = scale(n, d / l);
      mindist = sqnorm(p_to_project);
      res.encode = 7;
      res.parameterization[0] = norm(cross(dl[1], sub(sub(b, p), p_to_project))) / s;
      res.parameterization[1] = norm(cross(dl[2], sub(sub(c, p), p_to_project))) / s;
      res.parameterization[2] = 1 - res.parameterization[0] - res.parameterization[1];
    }
    res.sqr_distance = mindist;
  }
  return res;
}

bool shape_triangle_intersect(const Shape& s, const Tf& tfs, const V3& P1, const V3& P2, const V3& P3,
                              const Tf& tfm) {
  if (s.type == SH_SPHERE)  // ShapeTransformedTriangleIntersectIndepImpl<Sphere> (:527-547)
    return sphere_triangle_intersect(s.p[0], tfs.t, apply(tfm, P1), apply(tfm, P2), apply(tfm, P3), nullptr, nullptr,
                                     nullptr);
  const V3 tv[3] = {P1, P2, P3};
  Shape tri;
  tri.type = SH_TRIANGLE;
  tri.verts = tv;
  tri.nverts = 3;
  V3 nrm, pt;
  double depth;
  int gs, es;
  return gjk_intersect(s, tfs, tri, tfm, &nrm, &pt, &depth, &gs, &es);
}

bool shape_triangle_distance(const Shape& s, const Tf& tfs, const V3& P1, const V3& P2, const V3& P3,
                             const Tf& tfm, double& d, V3& ps, V3& pt) {
  if (s.type == SH_SPHERE) {
    // sphereTriangleDistance with witnesses (sphere_triangle-inl.h, three-transform form)
    const V3 W1 = apply(tfm, P1), W2 = apply(tfm, P2), W3 = apply(tfm, P3);
    const V3 o = tfs.t;
    const ProjectResult r = project_triangle_p(W1, W2, W3, o);
    const double rad = s.p[0];
    if (r.sqr_distance > rad * rad) {
      d = std::sqrt(r.sqr_distance) - rad;
      const V3 project_p =
          add(add(scale(W1, r.parameterization[0]), scale(W2, r.parameterization[1])), scale(W3, r.parameterization[2]));
      const V3 dir = normalized(sub(o, project_p));
      ps = apply(isometry_inverse(tfs), sub(o, scale(dir, rad)));
      pt = apply(isometry_inverse(tfm), project_p);
      return true;
    }
    // FCL leaves the distance and the witnesses unset here; the oracle reports -1 (the
    // value of the witness-free branch) and zero witnesses
    d = -1;
    ps = pt = mk(0, 0, 0);
    return false;
  }
  const V3 tv[3] = {P1, P2, P3};
  Shape tri;
  tri.type = SH_TRIANGLE;
  tri.verts = tv;
  tri.nverts = 3;
  int gs;
  d = -1;
  ps = pt = mk(0, 0, 0);
  gjk_distance(s, tfs, tri, tfm, &d, &ps, &pt, &gs);
  return gs == 0;  // GJK Valid
}

namespace {

struct MsCollide {
  const Mesh& m;
  const Tf& tfm;
  const Shape& s;
  const Tf& tfs;
  OBB sbv;
  size_t max_contacts;
  size_t count = 0;
  std::vector<int>* tris;
  CollideStats* st;
  // MeshShapeCollisionTraversalNodeOBBRSS::BVTesting: true = disjoint
  bool bv_testing(int b) {
    if (st) ++st->num_bv_tests;
    return !obb_overlap(tfm.R, tfm.t, sbv, m.nodes[b].obb);
  }
  void leaf_testing(int b) {
    if (st) ++st->num_leaf_tests;
    const int prim = -(m.nodes[b].first_child + 1);
    const Tri& t = m.tris[prim];
    if (shape_triangle_intersect(s, tfs, m.verts[t.v[0]], m.verts[t.v[1]], m.verts[t.v[2]], tfm)) {
      if (max_contacts > count) {
        ++count;
        if (tris) tris->push_back(prim);
      }
    }
  }
  bool can_stop() const { return count > 0 && max_contacts <= count; }
  void recurse(int b) {
    const bool leaf = m.nodes[b].first_child < 0;
    if (leaf) {
      if (bv_testing(b)) return;
      leaf_testing(b);
      return;
    }
    if (bv_testing(b)) return;
    const int c1 = m.nodes[b].first_child, c2 = c1 + 1;
    recurse(c1);
    if (can_stop()) return;
    recurse(c2);
  }
};

struct MsDistance {
  const Mesh& m;
  const Tf& tfm;
  const Shape& s;
  const Tf& tfs;
  RSS sbv;
  DistanceOut& out;
  CollideStats* st;
  double bv_testing(int b) {
    if (st) ++st->num_bv_tests;
    return rss_distance(tfm.R, tfm.t, sbv, m.nodes[b].rss, nullptr, nullptr);
  }
  // meshShapeDistanceOrientedNodeLeafTesting / distancePreprocessOrientedNode
  void leaf(int prim) {
    const Tri& t = m.tris[prim];
    double d;
    V3 ps, pt;
    shape_triangle_distance(s, tfs, m.verts[t.v[0]], m.verts[t.v[1]], m.verts[t.v[2]], tfm, d, ps, pt);
    if (out.min_distance > d) {  // DistanceResult::update
      out.min_distance = d;
      out.b1 = prim;
      out.b2 = -1;
      out.p1 = pt;
      out.p2 = ps;
    }
  }
  bool can_stop(double c) const { return c >= out.min_distance; }
  void recurse(int b) {
    if (m.nodes[b].first_child < 0) {
      if (st) ++st->num_leaf_tests;
      leaf(-(m.nodes[b].first_child + 1));
      return;
    }
    const int a1 = m.nodes[b].first_child, c1 = a1 + 1;
    const double d1 = bv_testing(a1);
    const double d2 = bv_testing(c1);
    if (d2 < d1) {
      if (!can_stop(d2)) recurse(c1);
      if (!can_stop(d1)) recurse(a1);
    } else {
      if (!can_stop(d1)) recurse(a1);
      if (!can_stop(d2)) recurse(c1);
    }
  }
};

}  // namespace

size_t collide_mesh_shape(const Mesh& m, const Tf& tfm, const Shape& s, const Tf& tfs, size_t max_contacts,
                          std::vector<int>* tris, CollideStats* st) {
  MsCollide c{m, tfm, s, tfs, OBB(), max_contacts, 0, tris, st};
  RSS unused;
  shape_obbrss(s, tfs, c.sbv, unused);
  c.recurse(0);
  return c.count;
}

double distance_mesh_shape(const Mesh& m, const Tf& tfm, const Shape& s, const Tf& tfs, DistanceOut& out,
                           CollideStats* st) {
  out.min_distance = std::numeric_limits<double>::max();
  out.b1 = out.b2 = -1;
  out.p1 = out.p2 = mk(0, 0, 0);
  MsDistance c{m, tfm, s, tfs, RSS(), out, st};
  OBB unused;
  shape_obbrss(s, tfs, unused, c.sbv);
  c.leaf(0);  // preprocess: the first triangle seeds the result
  c.recurse(0);
  return out.min_distance;
}

}  // namespace oracle
