// C entry points of the FP64 CPU oracle, loaded by tests/ and by bench.py's CPU
// baseline through ctypes.  TEST INFRASTRUCTURE ONLY: the shipped library never
// links or calls this file.
//
// Transforms are 3x4 row-major doubles [R | t] (12 per pose).
#include <atomic>
#include <cstring>
#include <limits>
#include <thread>
#include <vector>

#include "oracle_broadphase.h"
#include "oracle_meshshape.h"
#include "oracle_mesh.h"

using namespace oracle;

namespace {

Tf load_tf(const double* p) {
  Tf f;
  for (int r = 0; r < 3; ++r) {
    for (int c = 0; c < 3; ++c) f.R(r, c) = p[4 * r + c];
    f.t[r] = p[4 * r + 3];
  }
  return f;
}
Tf identity_tf() {
  Tf f;
  f.R = ident();
  f.t = mk(0, 0, 0);
  return f;
}

template <class F>
void parallel_for(int64_t n, int nthreads, F fn) {
  if (nthreads <= 1 || n < 2) {
    for (int64_t i = 0; i < n; ++i) fn(i, 0);
    return;
  }
  std::atomic<int64_t> next(0);
  std::vector<std::thread> th;
  for (int t = 0; t < nthreads; ++t)
    th.emplace_back([&, t]() {
      for (;;) {
        int64_t i = next.fetch_add(1);
        if (i >= n) break;
        fn(i, t);
      }
    });
  for (auto& x : th) x.join();
}

}  // namespace

extern "C" {

void* orc_mesh_create(const double* verts, int nv, const int* tris, int nt) {
  Mesh* m = new Mesh();
  m->verts.resize(nv);
  for (int i = 0; i < nv; ++i) m->verts[i] = mk(verts[3 * i], verts[3 * i + 1], verts[3 * i + 2]);
  m->tris.resize(nt);
  for (int i = 0; i < nt; ++i)
    for (int k = 0; k < 3; ++k) m->tris[i].v[k] = tris[3 * i + k];
  build_bvh(*m);
  return m;
}

void orc_mesh_free(void* h) { delete static_cast<Mesh*>(h); }

// BVHModel update with the default bottom-up refit: new vertex positions (3 per vertex)
void orc_mesh_update(void* h, const double* verts) {
  Mesh* m = static_cast<Mesh*>(h);
  std::vector<V3> nv(m->verts.size());
  for (size_t i = 0; i < nv.size(); ++i) nv[i] = mk(verts[3 * i], verts[3 * i + 1], verts[3 * i + 2]);
  update_refit_bottomup(*m, nv);
}

void orc_mesh_replace(void* h, const double* verts) {
  Mesh* m = static_cast<Mesh*>(h);
  std::vector<V3> nv(m->verts.size());
  for (size_t i = 0; i < nv.size(); ++i) nv[i] = mk(verts[3 * i], verts[3 * i + 1], verts[3 * i + 2]);
  replace_refit_bottomup(*m, nv);
}

// endUpdateModel(refit = false) / endReplaceModel(refit = false) (BVH_model-inl.h:594-620,
// 703-734): buildTree on the new vertices; an update then refits bottom-up over both frames.
void orc_mesh_rebuild(void* h, const double* verts, int update) {
  Mesh* m = static_cast<Mesh*>(h);
  std::vector<V3> nv(m->verts.size());
  for (size_t i = 0; i < nv.size(); ++i) nv[i] = mk(verts[3 * i], verts[3 * i + 1], verts[3 * i + 2]);
  Mesh built = *m;
  built.verts = nv;
  build_bvh(built);
  m->nodes = built.nodes;
  m->prim_idx = built.prim_idx;
  if (update)
    update_refit_bottomup(*m, nv);  // previous frame: the vertices before the call
  else
    m->verts = nv;
}

int orc_mesh_num_nodes(void* h) { return (int)static_cast<Mesh*>(h)->nodes.size(); }

// Per node: obb.axis (9, row-major), obb.To (3), obb.extent (3), rss.axis (9),
// rss.To (3), rss.l (2), rss.r (1) = 30 doubles; first_child in a separate array.
void orc_mesh_get_nodes(void* h, double* out, int* first_child) {
  const Mesh* m = static_cast<Mesh*>(h);
  for (size_t i = 0; i < m->nodes.size(); ++i) {
    const Node& n = m->nodes[i];
    double* o = out + 30 * i;
    for (int r = 0; r < 3; ++r)
      for (int c = 0; c < 3; ++c) o[3 * r + c] = n.obb.axis(r, c);
    for (int k = 0; k < 3; ++k) o[9 + k] = n.obb.To[k];
    for (int k = 0; k < 3; ++k) o[12 + k] = n.obb.extent[k];
    for (int r = 0; r < 3; ++r)
      for (int c = 0; c < 3; ++c) o[15 + 3 * r + c] = n.rss.axis(r, c);
    for (int k = 0; k < 3; ++k) o[24 + k] = n.rss.To[k];
    o[27] = n.rss.l[0];
    o[28] = n.rss.l[1];
    o[29] = n.rss.r;
    first_child[i] = n.first_child;
  }
}

// Batched fcl::collide over n poses of one mesh pair.  tf1 may be NULL (identity).
// counts[i] = number of contacts of pose i; contacts (b1,b2) are written pose after
// pose in the reference's DFS order into out (capacity cap pairs).  Returns the total
// number of contact pairs (even if it exceeds cap; then out holds only a prefix).
int64_t orc_collide_batch(void* h1, void* h2, int64_t n, const double* tf1, const double* tf2,
                          int64_t num_max_contacts, int nthreads, int64_t* counts, int64_t* nbv,
                          int64_t* nleaf, int* out, int64_t cap) {
  const Mesh* m1 = static_cast<Mesh*>(h1);
  const Mesh* m2 = static_cast<Mesh*>(h2);
  std::vector<std::vector<int>> per(n);
  parallel_for(n, nthreads, [&](int64_t i, int) {
    Tf a = tf1 ? load_tf(tf1 + 12 * i) : identity_tf();
    Tf b = load_tf(tf2 + 12 * i);
    CollideStats st;
    size_t k = collide_mesh(*m1, a, *m2, b, (size_t)num_max_contacts, per[i], &st);
    counts[i] = (int64_t)k;
    if (nbv) nbv[i] = st.num_bv_tests;
    if (nleaf) nleaf[i] = st.num_leaf_tests;
  });
  int64_t total = 0;
  for (int64_t i = 0; i < n; ++i) {
    const int64_t k = counts[i];
    if (out && total + k <= cap) std::memcpy(out + 2 * total, per[i].data(), sizeof(int) * 2 * k);
    total += k;
  }
  return total;
}

// collide(node, front_list) for one pose of a mesh pair: the front (b1, b2 pairs) in and
// out.  Returns the number of contacts; *nfront_out and the contacts / front written up
// to their capacities (pairs).
int64_t orc_collide_front(void* h1, void* h2, const double* tf1, const double* tf2, int64_t num_max_contacts,
                          const int* front_in, int64_t nfront_in, int* front_out, int64_t front_cap,
                          int64_t* nfront_out, int* contacts, int64_t cont_cap, int64_t* nbv, int64_t* nleaf) {
  const Mesh* m1 = static_cast<Mesh*>(h1);
  const Mesh* m2 = static_cast<Mesh*>(h2);
  std::vector<int> front(front_in, front_in + 2 * nfront_in), cont;
  CollideStats st;
  const size_t k = collide_mesh_front(*m1, tf1 ? load_tf(tf1) : identity_tf(), *m2, load_tf(tf2),
                                      (size_t)num_max_contacts, front, cont, &st);
  *nfront_out = (int64_t)front.size() / 2;
  for (int64_t j = 0; j < std::min<int64_t>(*nfront_out, front_cap); ++j) {
    front_out[2 * j] = front[2 * j];
    front_out[2 * j + 1] = front[2 * j + 1];
  }
  for (int64_t j = 0; j < std::min<int64_t>((int64_t)k, cont_cap); ++j) {
    contacts[2 * j] = cont[2 * j];
    contacts[2 * j + 1] = cont[2 * j + 1];
  }
  if (nbv) *nbv = st.num_bv_tests;
  if (nleaf) *nleaf = st.num_leaf_tests;
  return (int64_t)k;
}

// Batched fcl::collide with enable_contact = true over n poses of one mesh pair.
// counts[i] = contacts of pose i; per contact (pose after pose, DFS order): ids (b1,b2),
// pos (3), normal (3), depth (1), up to cap contacts.  Returns the total.
int64_t orc_collide_contacts_batch(void* h1, void* h2, int64_t n, const double* tf1, const double* tf2,
                                   int64_t num_max_contacts, int nthreads, int64_t* counts, int* ids,
                                   double* pos, double* normal, double* depth, int64_t cap) {
  const Mesh* m1 = static_cast<Mesh*>(h1);
  const Mesh* m2 = static_cast<Mesh*>(h2);
  std::vector<std::vector<ContactOut>> per(n);
  parallel_for(n, nthreads, [&](int64_t i, int) {
    Tf a = tf1 ? load_tf(tf1 + 12 * i) : identity_tf();
    Tf b = load_tf(tf2 + 12 * i);
    counts[i] = (int64_t)collide_mesh_contacts(*m1, a, *m2, b, (size_t)num_max_contacts, per[i], nullptr);
  });
  int64_t total = 0;
  for (int64_t i = 0; i < n; ++i) {
    for (const ContactOut& c : per[i]) {
      if (total < cap) {
        ids[2 * total] = c.b1;
        ids[2 * total + 1] = c.b2;
        for (int k = 0; k < 3; ++k) {
          pos[3 * total + k] = c.pos[k];
          normal[3 * total + k] = c.normal[k];
        }
        depth[total] = c.depth;
      }
      ++total;
    }
  }
  return total;
}

// The contact part of intersect_Triangle for n triangle pairs (P: 9 doubles, Qm: 9
// doubles, Q already in P's frame): counts[i], pts (6), normal (3), depth (1).
void orc_tri_contact_batch(int64_t n, const double* P, const double* Qm, int* counts, double* pts,
                           double* normal, double* depth) {
  for (int64_t i = 0; i < n; ++i) {
    V3 a[3], b[3];
    for (int k = 0; k < 3; ++k) {
      a[k] = mk(P[9 * i + 3 * k], P[9 * i + 3 * k + 1], P[9 * i + 3 * k + 2]);
      b[k] = mk(Qm[9 * i + 3 * k], Qm[9 * i + 3 * k + 1], Qm[9 * i + 3 * k + 2]);
    }
    V3 cp[2], nrm;
    double d;
    int k = tri_contact_info(a, b, cp, nrm, d);
    counts[i] = k;
    for (int j = 0; j < 2; ++j)
      for (int c = 0; c < 3; ++c) pts[6 * i + 3 * j + c] = j < k ? cp[j][c] : 0.0;
    for (int c = 0; c < 3; ++c) normal[3 * i + c] = nrm[c];
    depth[i] = d;
  }
}

// Batched fcl::continuousCollide (naive solver; motion 0 translation, 1 linear, 2 screw) over n motions of
// one mesh pair: tf1_beg/tf1_end may be NULL (identity).  Outputs per motion: hit,
// time of contact, the transforms at the time of contact (12 doubles each; untouched
// when there is no collision).
void orc_ccd_batch(void* h1, void* h2, int64_t n, const double* a0, const double* a1, const double* b0,
                   const double* b1, int64_t num_max_iterations, double toc_err, int motion, int nthreads, int* hit,
                   double* toc, double* ctf1, double* ctf2) {
  const Mesh* m1 = static_cast<Mesh*>(h1);
  const Mesh* m2 = static_cast<Mesh*>(h2);
  parallel_for(n, nthreads, [&](int64_t i, int) {
    Tf ta0 = a0 ? load_tf(a0 + 12 * i) : identity_tf();
    Tf ta1 = a1 ? load_tf(a1 + 12 * i) : identity_tf();
    Tf tb0 = load_tf(b0 + 12 * i), tb1 = load_tf(b1 + 12 * i);
    Tf ca, cb;
    double t;
    bool h = continuous_collide_naive(*m1, ta0, ta1, *m2, tb0, tb1, (size_t)num_max_iterations, toc_err, motion, t,
                                      ca, cb);
    hit[i] = h ? 1 : 0;
    toc[i] = t;
    if (h) {
      for (int r = 0; r < 3; ++r) {
        for (int c = 0; c < 3; ++c) {
          ctf1[12 * i + 4 * r + c] = ca.R(r, c);
          ctf2[12 * i + 4 * r + c] = cb.R(r, c);
        }
        ctf1[12 * i + 4 * r + 3] = ca.t[r];
        ctf2[12 * i + 4 * r + 3] = cb.t[r];
      }
    }
  });
}

// Batched continuous collide with conservative advancement over n motions of one mesh
// pair (the oriented OBBRSS node); outputs as orc_ccd_batch plus the iteration count.
void orc_ca_batch(void* h1, void* h2, int64_t n, const double* a0, const double* a1, const double* b0,
                  const double* b1, int motion, int nthreads, int* hit, double* toc, double* ctf1, double* ctf2,
                  int64_t* iters) {
  const Mesh* m1 = static_cast<Mesh*>(h1);
  const Mesh* m2 = static_cast<Mesh*>(h2);
  parallel_for(n, nthreads, [&](int64_t i, int) {
    Tf ta0 = a0 ? load_tf(a0 + 12 * i) : identity_tf();
    Tf ta1 = a1 ? load_tf(a1 + 12 * i) : identity_tf();
    Tf tb0 = load_tf(b0 + 12 * i), tb1 = load_tf(b1 + 12 * i);
    Tf ca, cb;
    double t;
    bool h = continuous_collide_ca(*m1, ta0, ta1, *m2, tb0, tb1, motion, t, ca, cb, iters ? iters + i : nullptr);
    hit[i] = h ? 1 : 0;
    toc[i] = t;
    if (h) {
      for (int r = 0; r < 3; ++r) {
        for (int c = 0; c < 3; ++c) {
          ctf1[12 * i + 4 * r + c] = ca.R(r, c);
          ctf2[12 * i + 4 * r + c] = cb.R(r, c);
        }
        ctf1[12 * i + 4 * r + 3] = ca.t[r];
        ctf2[12 * i + 4 * r + 3] = cb.t[r];
      }
    }
  });
}

// Batched fcl::distance over n poses of one mesh pair.  Outputs per pose: dist,
// (b1,b2), and when nearest != 0 the two world-frame nearest points (6 doubles).
void orc_distance_batch(void* h1, void* h2, int64_t n, const double* tf1, const double* tf2,
                        int nearest, int nthreads, double* dist, int* ids, double* pts,
                        int64_t* nbv, int64_t* nleaf) {
  const Mesh* m1 = static_cast<Mesh*>(h1);
  const Mesh* m2 = static_cast<Mesh*>(h2);
  parallel_for(n, nthreads, [&](int64_t i, int) {
    Tf a = tf1 ? load_tf(tf1 + 12 * i) : identity_tf();
    Tf b = load_tf(tf2 + 12 * i);
    DistanceOut o;
    CollideStats st;
    distance_mesh(*m1, a, *m2, b, nearest != 0, o, &st);
    dist[i] = o.min_distance;
    if (ids) {
      ids[2 * i] = o.b1;
      ids[2 * i + 1] = o.b2;
    }
    if (pts) {
      for (int k = 0; k < 3; ++k) {
        pts[6 * i + k] = o.p1[k];
        pts[6 * i + 3 + k] = o.p2[k];
      }
    }
    if (nbv) nbv[i] = st.num_bv_tests;
    if (nleaf) nleaf[i] = st.num_leaf_tests;
  });
}

// --- single-primitive entry points used by the known-answer tests -------------------

// RSS given as axis (9 row-major), To (3), l (2), r (1) = 15 doubles.
static RSS load_rss(const double* p) {
  RSS r;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) r.axis(i, j) = p[3 * i + j];
  r.To = mk(p[9], p[10], p[11]);
  r.l[0] = p[12];
  r.l[1] = p[13];
  r.r = p[14];
  return r;
}
static void store_rss(const RSS& r, double* p) {
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) p[3 * i + j] = r.axis(i, j);
  p[9] = r.To[0]; p[10] = r.To[1]; p[11] = r.To[2];
  p[12] = r.l[0]; p[13] = r.l[1]; p[14] = r.r;
}

void orc_rss_fit3(const double* pts9, double* rss15) {
  V3 ps[3];
  for (int i = 0; i < 3; ++i) ps[i] = mk(pts9[3 * i], pts9[3 * i + 1], pts9[3 * i + 2]);
  RSS r;
  rss_fit3(ps, r);
  store_rss(r, rss15);
}

double orc_rss_member_distance(const double* a15, const double* b15) {
  return rss_member_distance(load_rss(a15), load_rss(b15));
}

// rss_distance(R0,T0,b1,b2): tf given as 3x4.
double orc_rss_distance(const double* tf12, const double* a15, const double* b15) {
  Tf f = load_tf(tf12);
  return rss_distance(f.R, f.t, load_rss(a15), load_rss(b15), nullptr, nullptr);
}

// OBB given as axis (9), To (3), extent (3) = 15 doubles.
int orc_obb_overlap(const double* tf12, const double* a15, const double* b15) {
  Tf f = load_tf(tf12);
  OBB a, b;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      a.axis(i, j) = a15[3 * i + j];
      b.axis(i, j) = b15[3 * i + j];
    }
  a.To = mk(a15[9], a15[10], a15[11]);
  b.To = mk(b15[9], b15[10], b15[11]);
  a.extent = mk(a15[12], a15[13], a15[14]);
  b.extent = mk(b15[12], b15[13], b15[14]);
  return obb_overlap(f.R, f.t, a, b) ? 1 : 0;
}

// Triangle pair tests on n pairs: P (9 doubles) and Q (9 doubles) per pair, Q moved
// by tf (3x4, shared).
void orc_tri_intersect_batch(int64_t n, const double* P, const double* Q, const double* tf12,
                             int* out) {
  Tf f = load_tf(tf12);
  for (int64_t i = 0; i < n; ++i) {
    const double* p = P + 9 * i;
    const double* q = Q + 9 * i;
    out[i] = tri_intersect(mk(p[0], p[1], p[2]), mk(p[3], p[4], p[5]), mk(p[6], p[7], p[8]),
                           mk(q[0], q[1], q[2]), mk(q[3], q[4], q[5]), mk(q[6], q[7], q[8]), f.R, f.t)
                 ? 1 : 0;
  }
}

void orc_tri_distance_batch(int64_t n, const double* P, const double* Q, double* dist, double* pts) {
  for (int64_t i = 0; i < n; ++i) {
    V3 A[3], B[3];
    for (int k = 0; k < 3; ++k) {
      A[k] = mk(P[9 * i + 3 * k], P[9 * i + 3 * k + 1], P[9 * i + 3 * k + 2]);
      B[k] = mk(Q[9 * i + 3 * k], Q[9 * i + 3 * k + 1], Q[9 * i + 3 * k + 2]);
    }
    V3 p, q;
    dist[i] = tri_distance(A, B, p, q);
    if (pts)
      for (int k = 0; k < 3; ++k) {
        pts[6 * i + k] = p[k];
        pts[6 * i + 3 + k] = q[k];
      }
  }
}

// Brute force over all triangle pairs (the reference tests' cross-check:
// test_fcl_collision.cpp compares every BV type, AABB included, on the same poses).
// Writes intersecting pairs (b1,b2) in row-major pair order; returns their number.
int64_t orc_brute_collide(void* h1, void* h2, const double* tf1, const double* tf2, int* out, int64_t cap) {
  const Mesh* m1 = static_cast<Mesh*>(h1);
  const Mesh* m2 = static_cast<Mesh*>(h2);
  Tf a = tf1 ? load_tf(tf1) : identity_tf();
  Tf b = load_tf(tf2);
  M3 R = mulT(a.R, b.R);
  V3 T = mulTv(a.R, sub(b.t, a.t));
  int64_t k = 0;
  for (size_t i = 0; i < m1->tris.size(); ++i) {
    const Tri& t1 = m1->tris[i];
    for (size_t j = 0; j < m2->tris.size(); ++j) {
      const Tri& t2 = m2->tris[j];
      if (tri_intersect(m1->verts[t1.v[0]], m1->verts[t1.v[1]], m1->verts[t1.v[2]], m2->verts[t2.v[0]],
                        m2->verts[t2.v[1]], m2->verts[t2.v[2]], R, T)) {
        if (k < cap) {
          out[2 * k] = (int)i;
          out[2 * k + 1] = (int)j;
        }
        ++k;
      }
    }
  }
  return k;
}

// Minimum triangle distance over all pairs (tf = tf1^-1 tf2 as in the distance path).
double orc_brute_distance(void* h1, void* h2, const double* tf1, const double* tf2) {
  const Mesh* m1 = static_cast<Mesh*>(h1);
  const Mesh* m2 = static_cast<Mesh*>(h2);
  Tf a = tf1 ? load_tf(tf1) : identity_tf();
  Tf b = load_tf(tf2);
  M3 Rinv = transpose(a.R);
  V3 tinv = neg(mulv(Rinv, a.t));
  M3 R = mul(Rinv, b.R);
  V3 T = add(mulv(Rinv, b.t), tinv);
  std::vector<V3> moved(m2->verts.size());
  for (size_t k = 0; k < moved.size(); ++k) moved[k] = add(mulv(R, m2->verts[k]), T);
  double best = std::numeric_limits<double>::max();
  for (size_t i = 0; i < m1->tris.size(); ++i) {
    const Tri& t1 = m1->tris[i];
    V3 A[3] = {m1->verts[t1.v[0]], m1->verts[t1.v[1]], m1->verts[t1.v[2]]};
    for (size_t j = 0; j < m2->tris.size(); ++j) {
      const Tri& t2 = m2->tris[j];
      V3 B[3] = {moved[t2.v[0]], moved[t2.v[1]], moved[t2.v[2]]};
      V3 P, Q;
      double d = tri_distance(A, B, P, Q);
      if (d < best) best = d;
    }
  }
  return best;
}

int orc_hardware_threads() {
  unsigned n = std::thread::hardware_concurrency();
  return n ? (int)n : 1;
}

}  // extern "C"

// ---------------------------------------------------------------------------------
// Convex shape pairs (GJKSolver_indep semantics, see oracle_gjk.cpp)
// ---------------------------------------------------------------------------------
#include "oracle_gjk.h"

extern "C" {

// Shapes: type[ns], params[3*ns], voff[ns], vcnt[ns] into verts[3*nv] (convex only).
// Queries: ia[n], ib[n], tf1[12n], tf2[12n].  Outputs: hit[n], normal[3n], point[3n],
// depth[n], dist[n], p1[3n], p2[3n], status[2n] (gjk, epa).
void orc_shape_batch(int ns, const int* type, const double* params, const int* voff, const int* vcnt,
                     const double* verts, int64_t n, const int* ia, const int* ib, const double* tf1,
                     const double* tf2, int nthreads, int* hit, double* normal, double* point, double* depth,
                     double* dist, double* p1, double* p2, int* status) {
  std::vector<V3> vv;
  int nv = 0;
  for (int i = 0; i < ns; ++i) nv = std::max(nv, voff[i] + vcnt[i]);
  vv.resize(nv);
  for (int i = 0; i < nv; ++i) vv[i] = mk(verts[3 * i], verts[3 * i + 1], verts[3 * i + 2]);
  std::vector<Shape> sh(ns);
  for (int i = 0; i < ns; ++i) {
    sh[i].type = type[i];
    for (int k = 0; k < 3; ++k) sh[i].p[k] = params[3 * i + k];
    sh[i].verts = vv.data() + voff[i];
    sh[i].nverts = vcnt[i];
  }
  parallel_for(n, nthreads, [&](int64_t q, int) {
    ShapeResult r;
    shape_pair(sh[ia[q]], load_tf(tf1 + 12 * q), sh[ib[q]], load_tf(tf2 + 12 * q), r);
    hit[q] = r.collide ? 1 : 0;
    for (int k = 0; k < 3; ++k) {
      normal[3 * q + k] = r.normal[k];
      point[3 * q + k] = r.point[k];
      p1[3 * q + k] = r.p1[k];
      p2[3 * q + k] = r.p2[k];
    }
    depth[q] = r.depth;
    dist[q] = r.distance;
    status[2 * q] = r.gjk_status;
    status[2 * q + 1] = r.epa_status;
  });
}

// Origin projections (math/detail/project-inl.h:183-306) for the known-answer tests.
// k = 2, 3 or 4 points (3k doubles); out: encode, sqr_distance, parameterization[4].
void orc_project_origin(int k, const double* pts, int* encode, double* out5) {
  V3 v[4];
  for (int i = 0; i < k; ++i) v[i] = mk(pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]);
  ProjectResult r = k == 2 ? project_line(v[0], v[1]) : (k == 3 ? project_triangle(v[0], v[1], v[2])
                                                                : project_tetra(v[0], v[1], v[2], v[3]));
  *encode = (int)r.encode;
  out5[0] = r.sqr_distance;
  for (int i = 0; i < 4; ++i) out5[1 + i] = r.parameterization[i];
}

// ------------------------------------------------------------------ broadphase ----
// A geometry registry: ids [0, ns) are convex shapes, [ns, ns + nm) meshes created by
// orc_mesh_create.  Scenes and queries name geometries by id.
struct OrcGeoms {
  std::vector<V3> verts;
  std::vector<BpGeom> g;
};
struct OrcScene {
  const OrcGeoms* geoms;
  std::vector<BpObject> objs;
  DynTree tree;
};

static BpObject make_object(const OrcGeoms& G, int gid, const double* tf) {
  BpObject o;
  o.geom = &G.g[gid];
  o.tf = load_tf(tf);
  o.aabb = compute_aabb(*o.geom, o.tf);
  return o;
}

void* orc_geoms_create(int ns, const int* type, const double* params, const int* voff, const int* vcnt,
                       const double* verts, int nm, void* const* meshes) {
  OrcGeoms* G = new OrcGeoms();
  int nv = 0;
  for (int i = 0; i < ns; ++i) nv = std::max(nv, voff[i] + vcnt[i]);
  G->verts.resize(nv);
  for (int i = 0; i < nv; ++i) G->verts[i] = mk(verts[3 * i], verts[3 * i + 1], verts[3 * i + 2]);
  G->g.resize(ns + nm);
  for (int i = 0; i < ns; ++i) {
    BpGeom& g = G->g[i];
    g.kind = 0;
    g.shape.type = type[i];
    for (int k = 0; k < 3; ++k) g.shape.p[k] = params[3 * i + k];
    g.shape.verts = G->verts.data() + voff[i];
    g.shape.nverts = vcnt[i];
    compute_local_aabb(g);
  }
  for (int i = 0; i < nm; ++i) {
    BpGeom& g = G->g[ns + i];
    g.kind = 1;
    g.mesh = static_cast<const Mesh*>(meshes[i]);
    compute_local_aabb(g);
  }
  return G;
}

void orc_geoms_free(void* h) { delete static_cast<OrcGeoms*>(h); }

// Per geometry: aabb_local min (3), max (3), aabb_center (3), aabb_radius.
void orc_geoms_local(void* h, double* out10) {
  const OrcGeoms* G = static_cast<OrcGeoms*>(h);
  for (size_t i = 0; i < G->g.size(); ++i) {
    const BpGeom& g = G->g[i];
    for (int k = 0; k < 3; ++k) {
      out10[10 * i + k] = g.local.mn[k];
      out10[10 * i + 3 + k] = g.local.mx[k];
      out10[10 * i + 6 + k] = g.center[k];
    }
    out10[10 * i + 9] = g.radius;
  }
}

void* orc_scene_create(void* geoms, int n, const int* gid, const double* tf) {
  OrcScene* S = new OrcScene();
  S->geoms = static_cast<OrcGeoms*>(geoms);
  S->objs.resize(n);
  std::vector<AABB> bv(n);
  for (int i = 0; i < n; ++i) {
    S->objs[i] = make_object(*S->geoms, gid[i], tf + 12 * i);
    bv[i] = S->objs[i].aabb;
  }
  S->tree.build(bv);
  return S;
}

void orc_scene_free(void* h) { delete static_cast<OrcScene*>(h); }

int orc_scene_num_tree_nodes(void* h) { return (int)static_cast<OrcScene*>(h)->tree.nodes.size(); }

// World AABBs of n objects (geometry ids + poses), 6 doubles each (min, max).
void orc_world_aabbs(void* geoms, int64_t n, const int* gid, const double* tf, double* out6) {
  const OrcGeoms* G = static_cast<OrcGeoms*>(geoms);
  for (int64_t i = 0; i < n; ++i) {
    const AABB b = compute_aabb(G->g[gid[i]], load_tf(tf + 12 * i));
    for (int k = 0; k < 3; ++k) {
      out6[6 * i + k] = b.mn[k];
      out6[6 * i + 3 + k] = b.mx[k];
    }
  }
}

// Exact AABB-overlap candidates of each query, brute force, in object order.
// Returns the total; writes object ids while they fit in cap.
int64_t orc_scene_candidates(void* h, int64_t nq, const int* qgid, const double* qtf, int64_t* counts, int* out,
                             int64_t cap) {
  const OrcScene* S = static_cast<OrcScene*>(h);
  int64_t total = 0;
  for (int64_t q = 0; q < nq; ++q) {
    const BpObject Q = make_object(*S->geoms, qgid[q], qtf + 12 * q);
    int64_t c = 0;
    for (int i = 0; i < (int)S->objs.size(); ++i)
      if (aabb_overlap(S->objs[i].aabb, Q.aabb)) {
        if (out && total < cap) out[total] = i;
        ++total;
        ++c;
      }
    counts[q] = c;
  }
  return total;
}

// manager.collide(query, DefaultCollisionFunction) per query with
// request.num_max_contacts = max_contacts; use_tree selects the dynamic AABB tree
// manager, else the naive one.  Per query: total contacts, number of scene objects
// that reported contact; their ids (callback order) go to hits while they fit.
int64_t orc_scene_collide(void* h, int64_t nq, const int* qgid, const double* qtf, int64_t max_contacts,
                          int use_tree, int nthreads, int64_t* num_contacts, int* num_hits, int* hits,
                          int64_t cap, int64_t* narrow_calls) {
  const OrcScene* S = static_cast<OrcScene*>(h);
  std::vector<std::vector<int>> per(nq);
  parallel_for(nq, nthreads, [&](int64_t q, int) {
    const BpObject Q = make_object(*S->geoms, qgid[q], qtf + 12 * q);
    BpCollideOut o;
    bp_collide(S->objs, use_tree ? &S->tree : nullptr, Q, max_contacts, o);
    num_contacts[q] = o.num_contacts;
    num_hits[q] = (int)o.hit_objects.size();
    if (narrow_calls) narrow_calls[q] = o.narrow_calls;
    per[q] = std::move(o.hit_objects);
  });
  int64_t total = 0;
  for (int64_t q = 0; q < nq; ++q)
    for (int id : per[q]) {
      if (hits && total < cap) hits[total] = id;
      ++total;
    }
  return total;
}

// Contact lists of the GPU broadphase contacts call per query (bp_collide_lists):
// counts[q], and the (object, b1, b2) triples of every query one after the other in
// trip when the total fits cap.  Returns the total.
int64_t orc_scene_collide_lists(void* h, int64_t nq, const int* qgid, const double* qtf, int64_t max_per_pair,
                                int nthreads, int64_t* counts, int* trip, int64_t cap) {
  const OrcScene* S = static_cast<OrcScene*>(h);
  std::vector<std::vector<int>> per(nq);
  parallel_for(nq, nthreads, [&](int64_t q, int) {
    const BpObject Q = make_object(*S->geoms, qgid[q], qtf + 12 * q);
    bp_collide_lists(S->objs, Q, max_per_pair, per[q]);
    counts[q] = (int64_t)(per[q].size() / 3);
  });
  int64_t total = 0;
  for (const auto& v : per) total += (int64_t)(v.size() / 3);
  if (total <= cap) {
    int64_t k = 0;
    for (const auto& v : per)
      for (int x : v) trip[k++] = x;
  }
  return total;
}

// GJKSolver_indep parameters for every later GJK / EPA of the oracle.
void orc_set_gjk_solver_params(double gjk_tol, double epa_tol, int64_t gjk_iter, int64_t epa_iter) {
  set_solver_params(gjk_tol, epa_tol, (size_t)gjk_iter, (size_t)epa_iter);
}

// Self-collision lists (bp_self_collide_lists): counts per o2 and (o1, b1, b2) triples.
int64_t orc_scene_self_collide_lists(void* h, int64_t max_per_pair, int64_t* counts, int* trip, int64_t cap) {
  const OrcScene* S = static_cast<OrcScene*>(h);
  std::vector<int64_t> c;
  std::vector<int> v;
  bp_self_collide_lists(S->objs, max_per_pair, c, v);
  for (size_t i = 0; i < c.size(); ++i) counts[i] = c[i];
  const int64_t total = (int64_t)(v.size() / 3);
  if (total <= cap)
    for (size_t i = 0; i < v.size(); ++i) trip[i] = v[i];
  return total;
}

// NaiveCollisionManager::collide(cdata, DefaultCollisionFunction): numContacts().
int64_t orc_scene_self_collide_naive(void* h, int64_t max_contacts) {
  return bp_self_collide_naive(static_cast<OrcScene*>(h)->objs, max_contacts);
}

// NaiveCollisionManager::distance(cdata, DefaultDistanceFunction): d[0] = distance,
// d[1..6] = witnesses (on o1, on o2); ids = (o1, o2, b1, b2).
void orc_scene_self_distance(void* h, double* d, int* ids) {
  BpSelfDistanceOut o;
  bp_self_distance_naive(static_cast<OrcScene*>(h)->objs, o);
  d[0] = o.min_distance;
  for (int k = 0; k < 3; ++k) {
    d[1 + k] = o.p1[k];
    d[4 + k] = o.p2[k];
  }
  ids[0] = o.o1;
  ids[1] = o.o2;
  ids[2] = o.b1;
  ids[3] = o.b2;
}

// manager.distance(query, DefaultDistanceFunction) per query.  Outputs: min distance,
// scene object, (b1, b2) triangle ids (-1 for shapes), world witnesses (6 doubles).
void orc_scene_distance(void* h, int64_t nq, const int* qgid, const double* qtf, int use_tree, int nthreads,
                        double* dist, int* obj, int* b12, double* pts, int64_t* narrow_calls) {
  const OrcScene* S = static_cast<OrcScene*>(h);
  parallel_for(nq, nthreads, [&](int64_t q, int) {
    const BpObject Q = make_object(*S->geoms, qgid[q], qtf + 12 * q);
    BpDistanceOut o;
    bp_distance(S->objs, use_tree ? &S->tree : nullptr, Q, o);
    dist[q] = o.min_distance;
    if (obj) obj[q] = o.object;
    if (b12) {
      b12[2 * q] = o.b1;
      b12[2 * q + 1] = o.b2;
    }
    if (pts)
      for (int k = 0; k < 3; ++k) {
        pts[6 * q + k] = o.p1[k];
        pts[6 * q + 3 + k] = o.p2[k];
      }
    if (narrow_calls) narrow_calls[q] = o.narrow_calls;
  });
}

}  // extern "C"

extern "C" {

// fcl::collide / fcl::distance of one mesh against a convex shape per query: mesh
// handle h, shape ids into the registry g, poses tfm (mesh) and tfs (shape).  Outputs
// per query: collide -> counts (contacts, at most max_contacts); distance -> dist,
// tri (b1), pts (mesh point, shape point: 6 doubles).  nbv / nleaf optional.
void orc_mesh_shape_batch(void* h, void* g, int64_t n, const int* sid, const double* tfm, const double* tfs,
                          int64_t max_contacts, int mode, int nthreads, int64_t* counts, double* dist, int* tri,
                          double* pts, int64_t* nbv, int64_t* nleaf) {
  const Mesh* m = static_cast<Mesh*>(h);
  const OrcGeoms* G = static_cast<OrcGeoms*>(g);
  parallel_for(n, nthreads, [&](int64_t q, int) {
    const Shape& s = G->g[sid[q]].shape;
    const Tf a = load_tf(tfm + 12 * q), b = load_tf(tfs + 12 * q);
    CollideStats st;
    if (mode == 0) {
      counts[q] = (int64_t)collide_mesh_shape(*m, a, s, b, (size_t)max_contacts, nullptr, &st);
    } else {
      DistanceOut o;
      distance_mesh_shape(*m, a, s, b, o, &st);
      dist[q] = o.min_distance;
      tri[q] = o.b1;
      for (int k = 0; k < 3; ++k) {
        pts[6 * q + k] = o.p1[k];
        pts[6 * q + 3 + k] = o.p2[k];
      }
    }
    if (nbv) nbv[q] = st.num_bv_tests;
    if (nleaf) nleaf[q] = st.num_leaf_tests;
  });
}

// fcl::collide(mesh, shape) per query with the contact list: the triangle ids of the
// contacts FCL adds (Contact b1), in order, at most max_contacts per query.  counts[q]
// per query; tris holds the lists one after the other when the total fits cap.
// Returns the total.
int64_t orc_mesh_shape_contacts(void* h, void* g, int64_t n, const int* sid, const double* tfm, const double* tfs,
                                int64_t max_contacts, int nthreads, int64_t* counts, int* tris, int64_t cap) {
  const Mesh* m = static_cast<Mesh*>(h);
  const OrcGeoms* G = static_cast<OrcGeoms*>(g);
  std::vector<std::vector<int>> lists((size_t)n);
  parallel_for(n, nthreads, [&](int64_t q, int) {
    const Shape& s = G->g[sid[q]].shape;
    const Tf a = load_tf(tfm + 12 * q), b = load_tf(tfs + 12 * q);
    counts[q] = (int64_t)collide_mesh_shape(*m, a, s, b, (size_t)max_contacts, &lists[(size_t)q], nullptr);
  });
  int64_t total = 0;
  for (const auto& l : lists) total += (int64_t)l.size();
  if (total <= cap) {
    int64_t k = 0;
    for (const auto& l : lists)
      for (int t : l) tris[k++] = t;
  }
  return total;
}

// Contact geometry of listed mesh-shape contacts: for contact k (pair sid[k], poses
// tfm/tfs of that contact, mesh triangle tri[k]) the position, normal and depth FCL's
// leaf records with enable_contact; ok[k] = 0 when the pair does not intersect.
void orc_mesh_shape_contact_geometry(void* h, void* g, int64_t n, const int* sid, const double* tfm,
                                     const double* tfs, const int* tri, double* pos, double* nrm, double* depth,
                                     int* ok) {
  const Mesh* m = static_cast<Mesh*>(h);
  const OrcGeoms* G = static_cast<OrcGeoms*>(g);
  for (int64_t k = 0; k < n; ++k) {
    const Tri& t = m->tris[tri[k]];
    V3 p, nv;
    double d = 0;
    ok[k] = shape_triangle_contact(G->g[sid[k]].shape, load_tf(tfs + 12 * k), m->verts[t.v[0]], m->verts[t.v[1]],
                                   m->verts[t.v[2]], load_tf(tfm + 12 * k), p, nv, d)
                ? 1
                : 0;
    for (int c = 0; c < 3; ++c) {
      pos[3 * k + c] = p[c];
      nrm[3 * k + c] = nv[c];
    }
    depth[k] = d;
  }
}

// Brute force over every triangle of the mesh (for the traversal tests): collide ->
// number of intersecting triangles; distance -> min over triangles.
void orc_mesh_shape_brute(void* h, void* g, int sid, const double* tfm, const double* tfs, int64_t* count,
                          double* dist) {
  const Mesh* m = static_cast<Mesh*>(h);
  const OrcGeoms* G = static_cast<OrcGeoms*>(g);
  const Shape& s = G->g[sid].shape;
  const Tf a = load_tf(tfm), b = load_tf(tfs);
  int64_t c = 0;
  double best = std::numeric_limits<double>::max();
  for (const Tri& t : m->tris) {
    const V3 &p1 = m->verts[t.v[0]], &p2 = m->verts[t.v[1]], &p3 = m->verts[t.v[2]];
    if (shape_triangle_intersect(s, b, p1, p2, p3, a)) ++c;
    double d;
    V3 ps, pt;
    shape_triangle_distance(s, b, p1, p2, p3, a, d, ps, pt);
    if (d < best) best = d;
  }
  *count = c;
  *dist = best;
}

// computeBV<OBBRSS>(shape, tf): obb axis (9, row-major), To, extent, rss axis, To, l[2], r (30).
void orc_shape_obbrss(void* g, int sid, const double* tf, double* out30) {
  const OrcGeoms* G = static_cast<OrcGeoms*>(g);
  OBB o;
  RSS r;
  shape_obbrss(G->g[sid].shape, load_tf(tf), o, r);
  int k = 0;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) out30[k++] = o.axis(i, j);
  for (int i = 0; i < 3; ++i) out30[k++] = o.To[i];
  for (int i = 0; i < 3; ++i) out30[k++] = o.extent[i];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) out30[k++] = r.axis(i, j);
  for (int i = 0; i < 3; ++i) out30[k++] = r.To[i];
  out30[k++] = r.l[0];
  out30[k++] = r.l[1];
  out30[k++] = r.r;
}

}  // extern "C"
