// FP64 broadphase oracle (see oracle_broadphase.h).  TEST INFRASTRUCTURE ONLY.
#include "oracle_broadphase.h"

#include <algorithm>
#include <cmath>
#include <limits>

namespace oracle {

namespace {

const double kDmax = std::numeric_limits<double>::max();

AABB empty_box() {
  AABB b;
  b.mn = mk(kDmax, kDmax, kDmax);
  b.mx = mk(-kDmax, -kDmax, -kDmax);
  return b;
}

// AABB::operator+=(Vector3) and operator+=(AABB) (AABB-inl.h:162-176): cwiseMin/Max
void grow(AABB& b, const V3& p) {
  for (int k = 0; k < 3; ++k) {
    b.mn[k] = std::min(b.mn[k], p[k]);
    b.mx[k] = std::max(b.mx[k], p[k]);
  }
}
AABB merged(const AABB& a, const AABB& b) {
  AABB r = a;
  for (int k = 0; k < 3; ++k) {
    r.mn[k] = std::min(r.mn[k], b.mn[k]);
    r.mx[k] = std::max(r.mx[k], b.mx[k]);
  }
  return r;
}
// AABB::center (AABB-inl.h:230-233)
V3 center_of(const AABB& b) { return scale(add(b.mn, b.mx), 0.5); }
// AABB::size (AABB-inl.h:216-219): squared norm of the diagonal
double size_of(const AABB& b) { return sqnorm(sub(b.mx, b.mn)); }

// Eigen's MatrixBase::isIdentity with NumTraits<double>::dummy_precision() = 1e-12:
// diagonal entries isApprox(1) (|a - 1| <= 1e-12 * min(|a|, 1)), the others
// isMuchSmallerThan(1) (|a| <= 1e-12).
bool is_identity(const M3& R) {
  const double prec = 1e-12;
  for (int j = 0; j < 3; ++j)
    for (int i = 0; i < 3; ++i) {
      const double a = R(i, j);
      if (i == j) {
        if (!(std::fabs(a - 1.0) <= std::min(std::fabs(a), 1.0) * prec)) return false;
      } else {
        if (!(std::fabs(a) <= prec)) return false;
      }
    }
  return true;
}

}  // namespace

void compute_local_aabb(BpGeom& g) {
  if (g.kind == 1) {
    // BVH_model-inl.h:1080-1100
    AABB b = empty_box();
    for (const V3& v : g.mesh->verts) grow(b, v);
    g.center = center_of(b);
    double r = 0;
    for (const V3& v : g.mesh->verts) {
      const double s = sqnorm(sub(g.center, v));
      if (s > r) r = s;
    }
    g.radius = std::sqrt(r);
    g.local = b;
    return;
  }
  const Shape& s = g.shape;
  V3 d;
  switch (s.type) {
    case SH_BOX:  // box-inl.h:80-88
      d = scale(mk(s.p[0], s.p[1], s.p[2]), 0.5);
      break;
    case SH_SPHERE:  // sphere-inl.h:62-69 (aabb_radius = radius, set below)
      d = mk(s.p[0], s.p[0], s.p[0]);
      break;
    case SH_CAPSULE:  // capsule-inl.h:64-72
      d = mk(s.p[0], s.p[0], 0.5 * s.p[1] + s.p[0]);
      break;
    case SH_CYLINDER:  // cylinder-inl.h:64-72
    case SH_CONE:      // cone-inl.h:64-72
      d = mk(s.p[0], s.p[0], 0.5 * s.p[1]);
      break;
    default: {  // SH_CONVEX, convex-inl.h:86-96
      AABB b = empty_box();
      for (int i = 0; i < s.nverts; ++i) grow(b, s.verts[i]);
      g.local = b;
      g.center = center_of(b);
      g.radius = norm(sub(b.mn, g.center));
      return;
    }
  }
  g.local.mx = d;
  g.local.mn = neg(d);
  g.center = center_of(g.local);
  g.radius = s.type == SH_SPHERE ? s.p[0] : norm(sub(g.local.mn, g.center));
}

AABB compute_aabb(const BpGeom& g, const Tf& tf) {
  AABB b;
  if (is_identity(tf.R)) {
    // translate(aabb_local, t) (AABB-inl.h:345-352)
    b.mn = add(g.local.mn, tf.t);
    b.mx = add(g.local.mx, tf.t);
  } else {
    const V3 c = apply(tf, g.center);
    const V3 d = mk(g.radius, g.radius, g.radius);
    b.mn = sub(c, d);
    b.mx = add(c, d);
  }
  return b;
}

bool aabb_overlap(const AABB& a, const AABB& b) {
  for (int k = 0; k < 3; ++k)
    if (a.mn[k] > b.mx[k]) return false;
  for (int k = 0; k < 3; ++k)
    if (a.mx[k] < b.mn[k]) return false;
  return true;
}

double aabb_distance(const AABB& a, const AABB& b) {
  double result = 0;
  for (int k = 0; k < 3; ++k) {
    if (a.mn[k] > b.mx[k]) {
      const double delta = b.mx[k] - a.mn[k];
      result += delta * delta;
    } else if (b.mn[k] > a.mx[k]) {
      const double delta = a.mx[k] - b.mn[k];
      result += delta * delta;
    }
  }
  return std::sqrt(result);
}

// ---------------------------------------------------------------- tree build ----

namespace {

struct Builder {
  std::vector<DynTree::Node>& nodes;
  int make(const AABB& bv, int c0, int c1, int obj) {
    nodes.push_back(DynTree::Node{bv, {c0, c1}, obj});
    return (int)nodes.size() - 1;
  }
  // hierarchy_tree-inl.h:344-377: merge the pair whose union is smallest until one
  // node remains at *lbeg
  void bottomup(int* lbeg, int* lend) {
    int* lcur_end = lend;
    while (lbeg < lcur_end - 1) {
      int *min1 = nullptr, *min2 = nullptr;
      double min_size = kDmax;
      for (int* it1 = lbeg; it1 < lcur_end; ++it1)
        for (int* it2 = it1 + 1; it2 < lcur_end; ++it2) {
          const double cur = size_of(merged(nodes[*it1].bv, nodes[*it2].bv));
          if (cur < min_size) {
            min_size = cur;
            min1 = it1;
            min2 = it2;
          }
        }
      const int n0 = *min1, n1 = *min2;
      const int p = make(merged(nodes[n0].bv, nodes[n1].bv), n0, n1, -1);
      *min1 = p;
      const int tmp = *min2;
      --lcur_end;
      *min2 = *lcur_end;
      *lcur_end = tmp;
    }
  }
  // hierarchy_tree-inl.h:424-459
  int topdown0(int* lbeg, int* lend) {
    const int num = (int)(lend - lbeg);
    if (num > 1) {
      if (num > 2) {  // bu_threshold
        AABB vol = nodes[*lbeg].bv;
        for (int* it = lbeg + 1; it < lend; ++it) vol = merged(vol, nodes[*it].bv);
        int best = 0;
        const double ext[3] = {vol.mx[0] - vol.mn[0], vol.mx[1] - vol.mn[1], vol.mx[2] - vol.mn[2]};
        if (ext[1] > ext[0]) best = 1;
        if (ext[2] > ext[best]) best = 2;
        int* lcenter = lbeg + num / 2;
        // nodeBaseLess (hierarchy_tree-inl.h:1050-1054) on the AABB centers
        std::nth_element(lbeg, lcenter, lend, [&](int a, int b) {
          return center_of(nodes[a].bv)[best] < center_of(nodes[b].bv)[best];
        });
        const int node = make(vol, -1, -1, -1);
        const int c0 = topdown0(lbeg, lcenter);
        const int c1 = topdown0(lcenter, lend);
        nodes[node].child[0] = c0;
        nodes[node].child[1] = c1;
        return node;
      }
      bottomup(lbeg, lend);
      return *lbeg;
    }
    return *lbeg;
  }
};

// SelectImpl<S, AABB<S>>::run(query, node1, node2) (hierarchy_tree-inl.h:1117-1131)
int select_child(const AABB& q, const AABB& b1, const AABB& b2) {
  const V3 v = add(q.mn, q.mx);
  const V3 v1 = sub(v, add(b1.mn, b1.mx));
  const V3 v2 = sub(v, add(b2.mn, b2.mx));
  const double d1 = std::fabs(v1[0]) + std::fabs(v1[1]) + std::fabs(v1[2]);
  const double d2 = std::fabs(v2[0]) + std::fabs(v2[1]) + std::fabs(v2[2]);
  return (d1 < d2) ? 0 : 1;
}

// ------------------------------------------------------------- narrowphase ----

// fcl::collide(o1, o2, request, result) accumulating into one CollisionResult
// (collision-inl.h:79-149): ShapeShapeCollide (collision_func_matrix-inl.h:278-311)
// or orientedMeshCollide (:571-626).  Returns the contacts it added.
// With ids, each added contact's (b1, b2) is appended: NONE (-1) for shapes, the mesh
// triangle as b1 for a mesh-shape pair (FCL records the mesh first whichever argument
// order it got, collision-inl.h:124-131).
int64_t narrow_collide(const BpObject& o1, const BpObject& o2, int64_t max_contacts, int64_t cur,
                       std::vector<int>* ids = nullptr) {
  if (cur > 0 && max_contacts <= cur) return 0;  // CollisionRequest::isSatisfied
  const BpGeom& g1 = *o1.geom;
  const BpGeom& g2 = *o2.geom;
  if (g1.kind == 0 && g2.kind == 0) {
    // ShapeCollisionTraversalNode::leafTesting (shape_collision_traversal_node-inl.h:70-136)
    ShapeResult r;
    const bool hit = shape_intersect(g1.shape, o1.tf, g2.shape, o2.tf, r, false);
    const int64_t added = (hit && max_contacts > cur) ? 1 : 0;
    if (ids && added) {
      ids->push_back(-1);
      ids->push_back(-1);
    }
    return added;
  }
  if (g1.kind == 1 && g2.kind == 1) {
    std::vector<int> contacts;
    const size_t k =
        collide_mesh(*g1.mesh, o1.tf, *g2.mesh, o2.tf, (size_t)(max_contacts - cur), contacts, nullptr);
    if (ids) ids->insert(ids->end(), contacts.begin(), contacts.begin() + 2 * k);
    return (int64_t)k;
  }
  // BVHShapeCollider; a shape first is swapped to mesh first (collision-inl.h:100-111)
  const BpObject& om = g1.kind == 1 ? o1 : o2;
  const BpObject& os = g1.kind == 1 ? o2 : o1;
  std::vector<int> tris;
  const size_t k = collide_mesh_shape(*om.geom->mesh, om.tf, os.geom->shape, os.tf, (size_t)(max_contacts - cur),
                                      ids ? &tris : nullptr, nullptr);
  if (ids)
    for (size_t i = 0; i < k; ++i) {
      ids->push_back(tris[i]);
      ids->push_back(-1);
    }
  return (int64_t)k;
}

// fcl::distance(o1, o2, request, result) accumulating into one DistanceResult:
// ShapeShapeDistance (distance_func_matrix-inl.h:207-226) or orientedMeshDistance
// (:385-404); DistanceResult::update keeps a strictly smaller distance
// (distance_result-inl.h:84-105).
void narrow_distance(const BpObject& o1, int obj_index, const BpObject& o2, BpDistanceOut& out) {
  if (out.min_distance <= 0) return;  // DistanceRequest::isSatisfied
  const BpGeom& g1 = *o1.geom;
  const BpGeom& g2 = *o2.geom;
  ++out.narrow_calls;
  if (g1.kind == 0 && g2.kind == 0) {
    ShapeResult r;
    r.distance = -1;
    r.p1 = r.p2 = mk(0, 0, 0);
    shape_distance(g1.shape, o1.tf, g2.shape, o2.tf, r);
    if (out.min_distance > r.distance) {
      out.min_distance = r.distance;
      out.object = obj_index;
      out.b1 = out.b2 = -1;
      out.p1 = r.p1;
      out.p2 = r.p2;
    }
    return;
  }
  {
    DistanceOut d;
    if (g1.kind == 1 && g2.kind == 1) {
      distance_mesh(*g1.mesh, o1.tf, *g2.mesh, o2.tf, true, d, nullptr);
    } else {
      // BVHShapeDistancer; a shape first is swapped to mesh first (distance-inl.h:117-126)
      const BpObject& om = g1.kind == 1 ? o1 : o2;
      const BpObject& os = g1.kind == 1 ? o2 : o1;
      distance_mesh_shape(*om.geom->mesh, om.tf, os.geom->shape, os.tf, d, nullptr);
    }
    if (out.min_distance > d.min_distance) {
      out.min_distance = d.min_distance;
      out.object = obj_index;
      out.b1 = d.b1;
      out.b2 = d.b2;
      out.p1 = d.p1;
      out.p2 = d.p2;
    }
  }
}

struct CollideCtx {
  const std::vector<BpObject>& scene;
  const BpObject& query;
  int64_t max_contacts;
  BpCollideOut& out;
  bool done = false;
  // DefaultCollisionFunction (default_broadphase_callbacks.h:88-106)
  bool callback(int obj) {
    if (done) return true;
    ++out.narrow_calls;
    const int64_t added = narrow_collide(scene[obj], query, max_contacts, out.num_contacts);
    if (added > 0) out.hit_objects.push_back(obj);
    out.num_contacts += added;
    if (out.num_contacts > 0 && out.num_contacts >= max_contacts) done = true;
    return done;
  }
};

// collisionRecurse(root, query, ...) (broadphase_dynamic_AABB_tree-inl.h:526-547)
bool collide_recurse(const DynTree& t, int node, CollideCtx& c) {
  const DynTree::Node& n = t.nodes[node];
  if (n.obj >= 0) {
    if (!aabb_overlap(n.bv, c.query.aabb)) return false;
    return c.callback(n.obj);
  }
  if (!aabb_overlap(n.bv, c.query.aabb)) return false;
  const int sel = select_child(c.query.aabb, t.nodes[n.child[0]].bv, t.nodes[n.child[1]].bv);
  if (collide_recurse(t, n.child[sel], c)) return true;
  if (collide_recurse(t, n.child[1 - sel], c)) return true;
  return false;
}

struct DistanceCtx {
  const std::vector<BpObject>& scene;
  const BpObject& query;
  BpDistanceOut& out;
  // DefaultDistanceFunction (default_broadphase_callbacks.h:195-215); `done` never
  // becomes true there, the stop comes from dist <= 0
  bool callback(int obj, double& dist) {
    narrow_distance(scene[obj], obj, query, out);
    dist = out.min_distance;
    return dist <= 0;
  }
};

// distanceRecurse(root, query, ..., min_dist) (broadphase_dynamic_AABB_tree-inl.h:658-701)
bool distance_recurse(const DynTree& t, int node, DistanceCtx& c, double& min_dist) {
  const DynTree::Node& n = t.nodes[node];
  if (n.obj >= 0) return c.callback(n.obj, min_dist);
  const int a = n.child[0], b = n.child[1];
  const double d1 = aabb_distance(c.query.aabb, t.nodes[a].bv);
  const double d2 = aabb_distance(c.query.aabb, t.nodes[b].bv);
  if (d2 < d1) {
    if (d2 < min_dist && distance_recurse(t, b, c, min_dist)) return true;
    if (d1 < min_dist && distance_recurse(t, a, c, min_dist)) return true;
  } else {
    if (d1 < min_dist && distance_recurse(t, a, c, min_dist)) return true;
    if (d2 < min_dist && distance_recurse(t, b, c, min_dist)) return true;
  }
  return false;
}

}  // namespace

void bp_collide_lists(const std::vector<BpObject>& scene, const BpObject& query, int64_t max_per_pair,
                      std::vector<int>& out) {
  for (int i = 0; i < (int)scene.size(); ++i) {
    if (!aabb_overlap(scene[i].aabb, query.aabb)) continue;
    std::vector<int> ids;
    const int64_t k = narrow_collide(scene[i], query, max_per_pair, 0, &ids);
    for (int64_t t = 0; t < k; ++t) {
      out.push_back(i);
      out.push_back(ids[2 * t]);
      out.push_back(ids[2 * t + 1]);
    }
  }
}

int64_t bp_self_collide_naive(const std::vector<BpObject>& scene, int64_t max_contacts) {
  int64_t num = 0;
  for (int i = 0; i < (int)scene.size(); ++i)
    for (int j = i + 1; j < (int)scene.size(); ++j) {
      if (!aabb_overlap(scene[i].aabb, scene[j].aabb)) continue;
      num += narrow_collide(scene[i], scene[j], max_contacts, num);
      if (num > 0 && num >= max_contacts) return num;  // DefaultCollisionFunction's done
    }
  return num;
}

void bp_self_collide_lists(const std::vector<BpObject>& scene, int64_t max_per_pair, std::vector<int64_t>& counts,
                           std::vector<int>& out) {
  counts.assign(scene.size(), 0);
  for (int j = 0; j < (int)scene.size(); ++j)
    for (int i = 0; i < j; ++i) {
      if (!aabb_overlap(scene[i].aabb, scene[j].aabb)) continue;
      std::vector<int> ids;
      const int64_t k = narrow_collide(scene[i], scene[j], max_per_pair, 0, &ids);
      counts[j] += k;
      for (int64_t t = 0; t < k; ++t) {
        out.push_back(i);
        out.push_back(ids[2 * t]);
        out.push_back(ids[2 * t + 1]);
      }
    }
}

void bp_self_distance_naive(const std::vector<BpObject>& scene, BpSelfDistanceOut& out) {
  BpDistanceOut d;
  d.min_distance = std::numeric_limits<double>::max();
  out = BpSelfDistanceOut();
  double min_dist = std::numeric_limits<double>::max();
  for (int i = 0; i < (int)scene.size(); ++i)
    for (int j = i + 1; j < (int)scene.size(); ++j) {
      if (!(aabb_distance(scene[i].aabb, scene[j].aabb) < min_dist)) continue;
      const double before = d.min_distance;
      narrow_distance(scene[i], i, scene[j], d);
      if (d.min_distance < before) out.o2 = j;
      min_dist = d.min_distance;
      if (min_dist <= 0) break;
    }
  out.min_distance = d.min_distance;
  out.o1 = d.object;
  out.b1 = d.b1;
  out.b2 = d.b2;
  out.p1 = d.p1;
  out.p2 = d.p2;
}

void DynTree::build(const std::vector<AABB>& leaf_bv) {
  nodes.clear();
  root = -1;
  if (leaf_bv.empty()) return;
  nodes.reserve(2 * leaf_bv.size());
  std::vector<int> leaves(leaf_bv.size());
  for (size_t i = 0; i < leaf_bv.size(); ++i) {
    nodes.push_back(Node{leaf_bv[i], {-1, -1}, (int)i});
    leaves[i] = (int)i;
  }
  Builder b{nodes};
  root = b.topdown0(leaves.data(), leaves.data() + leaves.size());
}

void bp_collide(const std::vector<BpObject>& scene, const DynTree* tree, const BpObject& query,
                int64_t max_contacts, BpCollideOut& out) {
  out = BpCollideOut();
  if (scene.empty()) return;
  CollideCtx c{scene, query, max_contacts, out};
  if (tree) {
    collide_recurse(*tree, tree->root, c);
  } else {
    for (int i = 0; i < (int)scene.size(); ++i)
      if (c.callback(i)) return;
  }
}

void bp_distance(const std::vector<BpObject>& scene, const DynTree* tree, const BpObject& query,
                 BpDistanceOut& out) {
  out = BpDistanceOut();
  out.min_distance = kDmax;  // DistanceResult() (distance_result-inl.h:52-62)
  out.p1 = out.p2 = mk(0, 0, 0);
  if (scene.empty()) return;
  DistanceCtx c{scene, query, out};
  double min_dist = kDmax;
  if (tree) {
    distance_recurse(*tree, tree->root, c, min_dist);
  } else {
    for (int i = 0; i < (int)scene.size(); ++i)
      if (aabb_distance(query.aabb, scene[i].aabb) < min_dist)
        if (c.callback(i, min_dist)) return;
  }
}

}  // namespace oracle
