#include <algorithm>
// Test-only host build of the product's traversal code (collide_traverse.cuh) and
// BVH construction (bvh_build.cpp), so the kernel logic -- FP32 filters, FP64
// rechecks, visit order -- can be compared with the oracle without a GPU.  This
// library is built by the tests into tests/native/_build/ and is never shipped.
#include <vector>

#include "bvh_build.h"
#include "collide_traverse.cuh"
#include "distance_traverse.cuh"
#include "refit.cuh"
#include "shape_pair.cuh"
#include "tri_contact.cuh"
#include "motion.cuh"
#include "mesh_shape.cuh"

using namespace fclgpu;

namespace {

struct HostMesh {
  std::vector<double> verts;
  std::vector<int32_t> tris;
  HostBVH bvh;
  PackedF32 pk;
  DevMesh view;
};

void make_mesh(const double* v, int64_t nv, const int32_t* t, int64_t nt, HostMesh& m) {
  m.verts.assign(v, v + 3 * nv);
  m.tris.assign(t, t + 3 * nt);
  build_obbrss(m.verts.data(), nv, m.tris.data(), nt, m.bvh);
  pack_fp32(m.verts.data(), m.tris.data(), nt, m.bvh, m.pk);
  DevMesh& d = m.view;
  d.nodes64 = m.bvh.nodes.data();
  d.rss64 = m.bvh.rss.data();
  d.verts64 = m.verts.data();
  d.tris = m.tris.data();
  d.nodes32 = m.pk.nodes32.data();
  d.size64 = m.pk.size64.data();
  d.rss32 = m.pk.rss32.data();
  d.tri32 = m.pk.tri32.data();
  d.n_nodes = (int)m.bvh.nodes.size();
  d.n_tris = (int)nt;
  d.n_verts = (int)nv;
  d.max_depth = m.bvh.max_depth;
  double vmax = 0;
  for (int64_t i = 0; i < 3 * nv; ++i) vmax = std::max(vmax, std::fabs(v[i]));
  d.vmax = vmax * (1.0 + 1e-12);
  d.cmax = m.pk.cmax * (1.0 + 1e-12);
  d.rmax = m.pk.rmax * (1.0 + 1e-12);
  d.refitted = 0;
  d.pad2 = 0;
}

struct VecSink {
  std::vector<int>* out;
  void push(int, int, int b1, int b2) {
    out->push_back(b1);
    out->push_back(b2);
  }
};

// Host stand-in for the device split sink: contacts are (item, rank, b1, b2).
struct SplitHostSink {
  std::vector<int4>* rec;
  std::vector<int4>* items;
  std::vector<int>* cstart;
  std::vector<int>* ccount;
  bool dumped;
  void push(int item, int rank, int b1, int b2) { rec->push_back(make_int4(item, rank, b1, b2)); }
  void dump(long long item, long long qi, int2 cur, const int2* stk, int sp) {
    const int b = (int)items->size();
    items->push_back(make_int4((int)qi, cur.x, cur.y, 0));
    for (int j = 0; j < sp; ++j) items->push_back(make_int4((int)qi, stk[sp - 1 - j].x, stk[sp - 1 - j].y, 0));
    (*cstart)[item] = b;
    (*ccount)[item] = 1 + sp;
    dumped = true;
  }
};

}  // namespace

extern "C" {

// Certified FP32 distance traversal on the host (the device code of the FP32 form):
// per query distance, triangle ids, witness points (first mesh's frame: tf1 = I),
// statistics; returns -1 when a query fell back to FP64 or overflowed its stack.
int emu_distance_cert(const double* v1, int64_t nv1, const int32_t* t1, int64_t nt1, const double* v2, int64_t nv2,
                      const int32_t* t2, int64_t nt2, int64_t n, const double* tf2, double* dist, int32_t* ids,
                      double* pts, int64_t* nbv, int64_t* nleaf, int64_t* nrc) {
  HostMesh A, B;
  make_mesh(v1, nv1, t1, nt1, A);
  make_mesh(v2, nv2, t2, nt2, B);
  const double I[12] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0};
  for (int64_t q = 0; q < n; ++q) {
    M3<double> R;
    V3<double> T;
    rel_distance(I, tf2 + 12 * q, R, T);
    DistOut o;
    if (!distance_query_cert<256>(A.view, B.view, R, T, o) || o.status) return -1;
    dist[q] = o.d;
    ids[2 * q] = o.id1;
    ids[2 * q + 1] = o.id2;
    const double p[6] = {o.P.x, o.P.y, o.P.z, o.Q.x, o.Q.y, o.Q.z};
    for (int k = 0; k < 6; ++k) pts[6 * q + k] = p[k];
    nbv[q] = o.nbv;
    nleaf[q] = o.nleaf;
    nrc[q] = o.nrc;
  }
  return 0;
}

// Work-splitting batch on the host: same rounds, frontier dumps and item-tree
// assembly as the GPU path (budget = BV tests per item per round).
int64_t emu_collide_split(int prec, const double* v1, int64_t nv1, const int32_t* t1, int64_t nt1, const double* v2,
                          int64_t nv2, const int32_t* t2, int64_t nt2, int64_t n, const double* tf1,
                          const double* tf2, int maxc, int64_t budget, int32_t* counts, int32_t* out, int64_t cap,
                          int64_t* nbv, int64_t* nleaf, int64_t* nitems_out) {
  HostMesh A, B;
  make_mesh(v1, nv1, t1, nt1, A);
  make_mesh(v2, nv2, t2, nt2, B);
  DevMesh tab[2] = {A.view, B.view};
  int2 pair = make_int2(0, 1);
  CollideLaunch L{};
  L.meshes = tab;
  L.pairs = &pair;
  L.tf1 = tf1;
  L.tf2 = tf2;
  L.n = n;
  L.num_max_contacts = maxc;
  std::vector<int4> rec, items((size_t)n);
  for (int64_t q = 0; q < n; ++q) items[q] = make_int4((int)q, 0, 0, 0);
  std::vector<int> own, cstart, ccount;
  std::vector<std::pair<int64_t, int64_t>> rounds;
  for (int64_t q = 0; q < n; ++q) nbv[q] = nleaf[q] = 0;
  int64_t lo = 0, hi = n;
  while (hi > lo) {
    rounds.emplace_back(lo, hi);
    own.resize(items.size() + 70 * (hi - lo));
    cstart.resize(own.size());
    ccount.resize(own.size());
    for (int64_t it = lo; it < hi; ++it) {
      const int4 w = items[it];
      SplitHostSink sink{&rec, &items, &cstart, &ccount, false};
      QueryStats st;
      int k = prec == 0 ? collide_item<0, 256>(L, w.x, w.y, w.z, it, budget, maxc, sink, st)
                        : collide_item<1, 256>(L, w.x, w.y, w.z, it, budget, maxc, sink, st);
      if (st.status) return -1;
      own[it] = k;
      if (!sink.dumped) ccount[it] = 0;
      nbv[w.x] += st.nbv;
      nleaf[w.x] += st.nleaf;
      own.resize(std::max(own.size(), items.size() + 70));
      cstart.resize(own.size());
      ccount.resize(own.size());
    }
    lo = hi;
    hi = (int64_t)items.size();
  }
  const int64_t ni = (int64_t)items.size();
  std::vector<int64_t> total(ni), rel(ni, 0);
  for (size_t r = rounds.size(); r-- > 0;)
    for (int64_t i = rounds[r].first; i < rounds[r].second; ++i) {
      int64_t t = own[i];
      for (int j = 0; j < ccount[i]; ++j) t += total[cstart[i] + j];
      total[i] = t;
    }
  std::vector<int64_t> off(n + 1, 0);
  for (int64_t q = 0; q < n; ++q) {
    counts[q] = (int32_t)std::min<int64_t>(total[q], maxc);
    off[q + 1] = off[q] + counts[q];
  }
  for (size_t r = 0; r < rounds.size(); ++r)
    for (int64_t i = rounds[r].first; i < rounds[r].second; ++i) {
      int64_t run = rel[i] + own[i];
      for (int j = 0; j < ccount[i]; ++j) {
        rel[cstart[i] + j] = run;
        run += total[cstart[i] + j];
      }
    }
  const int64_t tot = off[n];
  for (const int4& r : rec) {
    const int64_t q = items[r.x].x;
    const int64_t pos = rel[r.x] + r.y;
    if (pos >= maxc) continue;
    const int64_t o = off[q] + pos;
    if (o < cap) {
      out[2 * o] = r.z;
      out[2 * o + 1] = r.w;
    }
  }
  *nitems_out = ni;
  return tot;
}

// Host run of the device refit math (refit.cuh): build from v0, then the bottom-up
// refit to each of the k frames in vs (k * nv * 3 doubles) in turn; nodes30 as emu_build.
void emu_refit(const double* v0, int64_t nv, const int32_t* t, int64_t nt, const double* vs, int k, double* nodes30,
               int32_t* fc, const int32_t* replace) {
  HostMesh m;
  make_mesh(v0, nv, t, nt, m);
  std::vector<double> prev;
  const int nn = (int)m.bvh.nodes.size();
  for (int f = 0; f < k; ++f) {
    prev = m.verts;
    m.verts.assign(vs + 3 * nv * f, vs + 3 * nv * (f + 1));
    for (int b = nn - 1; b >= 0; --b) {  // children follow their parent: reverse order is bottom up
      NodeD& nd = m.bvh.nodes[b];
      RssD& rs = m.bvh.rss[b];
      const int c = nd.child;
      if (c < 0 && replace && replace[f]) {  // replaced frame: fit3 of the new triangle
        const int tt = -(c + 1);
        D3v v[3];
        for (int i = 0; i < 3; ++i) {
          const double* q = m.verts.data() + 3 * m.tris[3 * tt + i];
          v[i] = v3(q[0], q[1], q[2]);
        }
        fit3_obbrss(v, nd, rs);
        nd.child = c;
      } else if (c < 0) {
        const int tt = -(c + 1);
        D3v v[6];
        for (int i = 0; i < 3; ++i) {
          const double* p = prev.data() + 3 * m.tris[3 * tt + i];
          const double* q = m.verts.data() + 3 * m.tris[3 * tt + i];
          v[i] = v3(p[0], p[1], p[2]);
          v[i + 3] = v3(q[0], q[1], q[2]);
        }
        auto pts = [&](int i) { return v[i]; };
        fit_points_bv(pts, 6, nd, rs.To, rs.l, rs.r);
        for (int j = 0; j < 9; ++j) rs.axis[j] = nd.axis[j];
        nd.child = c;
      } else {
        NodeD mg = obb_merge(m.bvh.nodes[c], m.bvh.nodes[c + 1]);
        mg.child = c;
        const RssD rm = rss_merge(m.bvh.rss[c], m.bvh.rss[c + 1]);
        nd = mg;
        rs = rm;
      }
    }
  }
  for (int i = 0; i < nn; ++i) {
    const NodeD& n = m.bvh.nodes[i];
    const RssD& r = m.bvh.rss[i];
    double* o = nodes30 + 30 * i;
    for (int j = 0; j < 9; ++j) o[j] = n.axis[j];
    for (int j = 0; j < 3; ++j) o[9 + j] = n.To[j];
    for (int j = 0; j < 3; ++j) o[12 + j] = n.ext[j];
    for (int j = 0; j < 9; ++j) o[15 + j] = r.axis[j];
    for (int j = 0; j < 3; ++j) o[24 + j] = r.To[j];
    o[27] = r.l[0];
    o[28] = r.l[1];
    o[29] = r.r;
    fc[i] = n.child;
  }
}

int emu_build(const double* v, int64_t nv, const int32_t* t, int64_t nt, double* nodes30, int32_t* fc,
              int32_t* max_depth) {
  HostMesh m;
  make_mesh(v, nv, t, nt, m);
  for (size_t i = 0; i < m.bvh.nodes.size(); ++i) {
    const NodeD& n = m.bvh.nodes[i];
    const RssD& r = m.bvh.rss[i];
    double* o = nodes30 + 30 * i;
    for (int k = 0; k < 9; ++k) o[k] = n.axis[k];
    for (int k = 0; k < 3; ++k) o[9 + k] = n.To[k];
    for (int k = 0; k < 3; ++k) o[12 + k] = n.ext[k];
    for (int k = 0; k < 9; ++k) o[15 + k] = r.axis[k];
    for (int k = 0; k < 3; ++k) o[24 + k] = r.To[k];
    o[27] = r.l[0];
    o[28] = r.l[1];
    o[29] = r.r;
    fc[i] = n.child;
  }
  *max_depth = m.bvh.max_depth;
  return (int)m.bvh.nodes.size();
}

// Runs n collide queries of one mesh pair with the product traversal on the host.
// Returns the total number of contacts written to out (cap pairs), or -1 on a stack
// overflow.
int64_t emu_collide(int prec, const double* v1, int64_t nv1, const int32_t* t1, int64_t nt1, const double* v2,
                    int64_t nv2, const int32_t* t2, int64_t nt2, int64_t n, const double* tf1, const double* tf2,
                    int maxc, int32_t* counts, int32_t* out, int64_t cap, int64_t* nbv, int64_t* nleaf,
                    int64_t* nrc) {
  HostMesh A, B;
  make_mesh(v1, nv1, t1, nt1, A);
  make_mesh(v2, nv2, t2, nt2, B);
  DevMesh tab[2] = {A.view, B.view};
  int2 pair = make_int2(0, 1);
  CollideLaunch L{};
  L.meshes = tab;
  L.pairs = &pair;
  L.pair_of_query = nullptr;
  L.tf1 = tf1;
  L.tf2 = tf2;
  L.n = n;
  L.num_max_contacts = maxc;
  std::vector<int> all;
  for (int64_t q = 0; q < n; ++q) {
    std::vector<int> cs;
    VecSink sink{&cs};
    QueryStats st;
    int k = prec == 0 ? collide_query<0, 256>(L, q, sink, st) : collide_query<1, 256>(L, q, sink, st);
    if (st.status) return -1;
    counts[q] = k;
    nbv[q] = st.nbv;
    nleaf[q] = st.nleaf;
    nrc[q] = st.nrecheck;
    all.insert(all.end(), cs.begin(), cs.end());
  }
  const int64_t total = (int64_t)all.size() / 2;
  for (int64_t i = 0; i < std::min(total, cap) * 2; ++i) out[i] = all[i];
  return total;
}

}  // extern "C"

// The shape registry as fclgpu_shapeset_create lays it out: the FP64 vertex pool, then
// the FP32 float4 copy the convex supports filter with; convex radii in p[0].
void make_shapes(int ns, const int* type, const double* params, const int* voff, const int* vcnt,
                 const double* verts, std::vector<double>& pool, std::vector<DevShape>& sh) {
  int64_t nv = 0;
  for (int i = 0; i < ns; ++i)
    if (type[i] == SHAPE_CONVEX) nv = std::max<int64_t>(nv, (int64_t)voff[i] + vcnt[i]);
  const int64_t off32 = (3 * nv + 1) & ~int64_t(1);
  pool.assign(off32 + 2 * nv + 2, 0.0);
  std::copy(verts, verts + 3 * nv, pool.begin());
  float* v32 = reinterpret_cast<float*>(pool.data() + off32);
  for (int64_t k = 0; k < nv; ++k)
    for (int c = 0; c < 3; ++c) v32[4 * k + c] = (float)verts[3 * k + c];
  sh.assign(ns, DevShape());
  for (int i = 0; i < ns; ++i) {
    sh[i].type = type[i];
    sh[i].voff = voff[i];
    sh[i].vcnt = vcnt[i];
    sh[i].pad = (type[i] == SHAPE_CONVEX && nv > 0) ? (int)off32 : 0;
    for (int k = 0; k < 3; ++k) sh[i].p[k] = params[3 * i + k];
    if (type[i] == SHAPE_CONVEX) {  // the radius fclgpu_shapeset_create stores
      double r = 0.0;
      for (int j = 0; j < vcnt[i]; ++j) {
        const double* v = verts + 3 * ((int64_t)voff[i] + j);
        r = std::max(r, std::sqrt((v[0] * v[0] + v[1] * v[1]) + v[2] * v[2]));
      }
      sh[i].p[0] = r * (1.0 + 1e-6);
    }
  }
}

extern "C" {

// Host run of the device shape-pair query (shape_pair.cuh) over n pairs.
void emu_shape_batch(int ns, const int* type, const double* params, const int* voff, const int* vcnt,
                     const double* verts, int64_t n, const int* ia, const int* ib, const double* tf1,
                     const double* tf2, int* hit, double* normal, double* point, double* depth, double* dist,
                     double* p1, double* p2, int* status) {
  std::vector<double> pool;
  std::vector<DevShape> sh;
  make_shapes(ns, type, params, voff, vcnt, verts, pool, sh);
  for (int64_t q = 0; q < n; ++q) {
    PairOut o;
    shape_pair_query(sh[ia[q]], sh[ib[q]], pool.data(), tf1 + 12 * q, tf2 + 12 * q, o);
    hit[q] = o.hit;
    const D3v* v[4] = {&o.normal, &o.point, &o.p1, &o.p2};
    double* d[4] = {normal, point, p1, p2};
    for (int k = 0; k < 4; ++k) {
      d[k][3 * q] = v[k]->x;
      d[k][3 * q + 1] = v[k]->y;
      d[k][3 * q + 2] = v[k]->z;
    }
    depth[q] = o.depth;
    dist[q] = o.dist;
    status[2 * q] = o.gstat;
    status[2 * q + 1] = o.estat;
  }
}

// The product's contact computation of an intersecting triangle pair (tri_contact.cuh),
// run on the host: P (9 doubles) and Qm (9 doubles, already in P's frame) per pair.
void emu_tri_contact_batch(int64_t n, const double* P, const double* Qm, int* counts, double* pts, double* normal,
                           double* depth) {
  for (int64_t i = 0; i < n; ++i) {
    V3<double> a[3], b[3];
    for (int k = 0; k < 3; ++k) {
      a[k] = v3<double>(P[9 * i + 3 * k], P[9 * i + 3 * k + 1], P[9 * i + 3 * k + 2]);
      b[k] = v3<double>(Qm[9 * i + 3 * k], Qm[9 * i + 3 * k + 1], Qm[9 * i + 3 * k + 2]);
    }
    V3<double> cp[2], nrm;
    double d;
    const int k = tri_contact(a, b, cp, nrm, d);
    counts[i] = k;
    for (int j = 0; j < 2; ++j) {
      pts[6 * i + 3 * j] = j < k ? cp[j].x : 0.0;
      pts[6 * i + 3 * j + 1] = j < k ? cp[j].y : 0.0;
      pts[6 * i + 3 * j + 2] = j < k ? cp[j].z : 0.0;
    }
    normal[3 * i] = nrm.x;
    normal[3 * i + 1] = nrm.y;
    normal[3 * i + 2] = nrm.z;
    depth[i] = d;
  }
}

// The product's motions (motion.cuh) on the host: n (beg, end, t) triples; type 0
// translation, 1 linear, 2 screw.
void emu_motion(int type, int64_t n, const double* beg, const double* end, const double* t, double* out) {
  for (int64_t i = 0; i < n; ++i) motion_at(type, beg + 12 * i, end + 12 * i, t[i], out + 12 * i);
}

// The certified FP32 bounds of the mesh-shape distance kernel (md_node_bound and
// leaf_cert_lb) checked against FCL's FP64 shapeTriangleDistance on the host: for every
// pair and every node, the node bound (along the nearest-point direction, and along
// the pair's direction dirs[3 * i]) must not exceed the smallest FP64 distance of the
// triangles below it by more than m64, and each triangle's bound not its own distance.
// Returns the number of violations; *checked receives the number of comparisons made
// and *positive how many bounds were above 0 (a bound that is never positive tests
// nothing).
int64_t emu_ms_bounds(int ns, const int* type, const double* params, const int* voff, const int* vcnt,
                      const double* verts, const double* mv, int64_t nv, const int32_t* mt, int64_t nt, int64_t n,
                      const int32_t* sidx, const double* tfm, const double* tfs, const float* dirs, int64_t* checked,
                      int64_t* positive) {
  std::vector<double> pool;
  std::vector<DevShape> sh;
  make_shapes(ns, type, params, voff, vcnt, verts, pool, sh);
  HostMesh hm;
  make_mesh(mv, nv, mt, nt, hm);
  const DevMesh& m = hm.view;
  const float4* rss32 = static_cast<const float4*>(m.rss32);
  int64_t bad = 0, nchk = 0, npos = 0;
  std::vector<double> dmin(m.n_nodes);
  for (int64_t i = 0; i < n; ++i) {
    ShapeRef A;
    A.s = sh[sidx[i]];
    A.verts = pool.data();
    M3<double> Rm, Rs;
    D3v tm, ts;
    load_tf(tfm + 12 * i, Rm, tm);
    load_tf(tfs + 12 * i, Rs, ts);
    MdPair q;
    md_pair(m, A, Rm, tm, Rs, ts, q);
    LeafCert32 cert;
    leaf_cert_init(A, Rs, ts, Rm, tm, cert);
    const double m64 = std::ldexp(1.0 + (double)q.rho + std::max(std::fabs(ts.x), std::max(std::fabs(ts.y), std::fabs(ts.z))) +
                                      std::max(std::fabs(tm.x), std::max(std::fabs(tm.y), std::fabs(tm.z))) + m.vmax + m.rmax,
                                  -36);
    const G3f dir = g3f(dirs[3 * i], dirs[3 * i + 1], dirs[3 * i + 2]);
    // children are stored after their parent: a reverse sweep sees them first
    for (int b = m.n_nodes - 1; b >= 0; --b) {
      const int c = m.nodes64[b].child;
      if (c < 0) {
        double P[9];
        load_tri_local(m, -(c + 1), P);
        SimplexVert V[kSimplexSlots];
        D3v ps, pt;
        double d;
        shape_triangle_distance(A, Rs, ts, P, Rm, tm, V, d, ps, pt);
        dmin[b] = d > 0.0 ? d : 0.0;
        if (A.s.type != SHAPE_SPHERE && d > 0.0) {
          G3f dd;
          const float lb = leaf_cert_lb(cert, P, dd);
          ++nchk;
          if (lb > 0.f) ++npos;
          if ((double)lb > d + m64) ++bad;
        }
      } else {
        dmin[b] = std::min(dmin[c], dmin[c + 1]);
      }
      for (int k = 0; k < 2; ++k) {
        const float lb = md_node_bound(rss32, b, A, q, k == 1, dir);
        ++nchk;
        if (lb > 0.f) ++npos;
        if ((double)lb > dmin[b] + m64) ++bad;
      }
    }
  }
  *checked = nchk;
  *positive = npos;
  return bad;
}

// The prepared leaf certificate (LeafCert32: poses and shape supports rounded once per
// pair) against the per-call certified_disjoint on n (shape, triangle) pairs of one
// posed mesh: returns the number of pairs where the two disagree; *disjoint receives
// how many the certificate proved disjoint.
int64_t emu_leaf_cert(int ns, const int* type, const double* params, const int* voff, const int* vcnt,
                      const double* verts, const double* mv, int64_t nv, const int32_t* mt, int64_t nt, int64_t n,
                      const int32_t* sidx, const double* tfm, const double* tfs, int64_t* disjoint) {
  std::vector<double> pool;
  std::vector<DevShape> sh;
  make_shapes(ns, type, params, voff, vcnt, verts, pool, sh);
  HostMesh hm;
  make_mesh(mv, nv, mt, nt, hm);
  const DevMesh& m = hm.view;
  int64_t diff = 0, dis = 0;
  for (int64_t i = 0; i < n; ++i) {
    ShapeRef A;
    A.s = sh[sidx[i]];
    A.verts = pool.data();
    M3<double> Rm, Rs;
    D3v tm, ts;
    load_tf(tfm + 12 * i, Rm, tm);
    load_tf(tfs + 12 * i, Rs, ts);
    LeafCert32 c;
    leaf_cert_init(A, Rs, ts, Rm, tm, c);
    for (int p = 0; p < m.n_tris; ++p) {
      double P[9];
      load_tri_local(m, p, P);
      const bool a = leaf_cert_disjoint(c, P);
      const bool b = certified_disjoint(A, Rs, ts, triangle_ref(P), Rm, tm);
      diff += a != b;
      dis += a;
    }
  }
  *disjoint = dis;
  return diff;
}

// The rule the warp mesh-shape distance applies to a pair with an intersecting triangle,
// run on the host over the whole tree: FCL's seed triangle 0 first, then the first
// triangle at distance < 0 in FCL's depth-first order (children ordered by its FP64
// bounds, the second first on d2 < d1), provided every bound on that triangle's path is
// exactly 0 and no triangle before it is at distance exactly 0.  tri[i] = the rule's
// triangle, or -1 where it does not apply (no intersecting triangle, or a condition
// fails: the kernel then runs FCL's serial traversal); dist[i] = that triangle's FP64
// distance.
void emu_ms_contact_rule(int ns, const int* type, const double* params, const int* voff, const int* vcnt,
                         const double* verts, const double* mv, int64_t nv, const int32_t* mt, int64_t nt, int64_t n,
                         const int32_t* sidx, const double* tfm, const double* tfs, int32_t* tri, double* dist) {
  std::vector<double> pool;
  std::vector<DevShape> sh;
  make_shapes(ns, type, params, voff, vcnt, verts, pool, sh);
  HostMesh hm;
  make_mesh(mv, nv, mt, nt, hm);
  const DevMesh& m = hm.view;
  for (int64_t i = 0; i < n; ++i) {
    ShapeRef A;
    A.s = sh[sidx[i]];
    A.verts = pool.data();
    M3<double> Rm, Rs;
    D3v tm, ts;
    load_tf(tfm + 12 * i, Rm, tm);
    load_tf(tfs + 12 * i, Rs, ts);
    ShapeBV bv;
    shape_obbrss(A.s, A.verts, Rs, ts, bv);
    M3<double> Ab;
    for (int k = 0; k < 9; ++k) Ab.m[k] = bv.obb.axis[k];
    const D3v Tob = v3(bv.rTo[0], bv.rTo[1], bv.rTo[2]);
    auto bvd = [&](int b) {
      const RssD& rs = m.rss64[b];
      M3<double> A2;
      for (int k = 0; k < 9; ++k) A2.m[k] = rs.axis[k];
      return rss_distance<double>(Rm, tm, Ab, Tob, bv.rl, bv.rr, A2, v3(rs.To[0], rs.To[1], rs.To[2]), rs.l, rs.r);
    };
    auto leaf_d = [&](int prim) {
      double P[9];
      load_tri_local(m, prim, P);
      SimplexVert V[kSimplexSlots];
      D3v ps, pt;
      double d;
      shape_triangle_distance(A, Rs, ts, P, Rm, tm, V, d, ps, pt);
      return d;
    };
    tri[i] = -1;
    dist[i] = 0.0;
    const double d0 = leaf_d(0);
    if (d0 < 0.0) {
      tri[i] = 0;
      dist[i] = d0;
      continue;
    }
    if (d0 == 0.0) continue;
    // depth-first in FCL's order: (node, all bounds on its path are 0)
    std::vector<std::pair<int, bool>> stack{{0, true}};
    bool zero_before = false;
    while (!stack.empty()) {
      const auto [b, zero] = stack.back();
      stack.pop_back();
      const int c = m.nodes64[b].child;
      if (c < 0) {
        const double d = leaf_d(-(c + 1));
        if (d == 0.0) zero_before = true;
        if (d < 0.0) {
          if (zero && !zero_before) {
            tri[i] = -(c + 1);
            dist[i] = d;
          }
          break;
        }
        continue;
      }
      const double d1 = bvd(c), d2 = bvd(c + 1);
      if (d2 < d1) {  // c + 1 first: pushed last
        stack.push_back({c, zero && d1 == 0.0});
        stack.push_back({c + 1, zero && d2 == 0.0});
      } else {
        stack.push_back({c + 1, zero && d2 == 0.0});
        stack.push_back({c, zero && d1 == 0.0});
      }
    }
  }
}

// The rule the warp mesh-shape distance applies to a pair without an intersecting
// triangle, run on the host over every triangle: the distance is the smallest FP64
// shapeTriangleDistance, and of the triangles at that distance FCL's first -- triangle 0
// (the seed) if it is one, otherwise the one on the side FCL enters first at their
// deepest common node (children ordered by its FP64 bounds, the second first on
// d2 < d1).  tri[i] = -1 where some triangle is at distance <= 0; ties[i] = the number
// of triangles at the minimum.
void emu_ms_min_rule(int ns, const int* type, const double* params, const int* voff, const int* vcnt,
                     const double* verts, const double* mv, int64_t nv, const int32_t* mt, int64_t nt, int64_t n,
                     const int32_t* sidx, const double* tfm, const double* tfs, int32_t* tri, double* dist,
                     int32_t* ties) {
  std::vector<double> pool;
  std::vector<DevShape> sh;
  make_shapes(ns, type, params, voff, vcnt, verts, pool, sh);
  HostMesh hm;
  make_mesh(mv, nv, mt, nt, hm);
  const DevMesh& m = hm.view;
  // parent of every node (children are allocated after their parent)
  std::vector<int> parent(m.n_nodes, -1), leaf_of(m.n_tris, -1);
  for (int b = 0; b < m.n_nodes; ++b) {
    const int c = m.nodes64[b].child;
    if (c >= 0) {
      parent[c] = b;
      parent[c + 1] = b;
    } else {
      leaf_of[-(c + 1)] = b;
    }
  }
  for (int64_t i = 0; i < n; ++i) {
    ShapeRef A;
    A.s = sh[sidx[i]];
    A.verts = pool.data();
    M3<double> Rm, Rs;
    D3v tm, ts;
    load_tf(tfm + 12 * i, Rm, tm);
    load_tf(tfs + 12 * i, Rs, ts);
    ShapeBV bv;
    shape_obbrss(A.s, A.verts, Rs, ts, bv);
    M3<double> Ab;
    for (int k = 0; k < 9; ++k) Ab.m[k] = bv.obb.axis[k];
    const D3v Tob = v3(bv.rTo[0], bv.rTo[1], bv.rTo[2]);
    auto bvd = [&](int b) {
      const RssD& rs = m.rss64[b];
      M3<double> A2;
      for (int k = 0; k < 9; ++k) A2.m[k] = rs.axis[k];
      return rss_distance<double>(Rm, tm, Ab, Tob, bv.rl, bv.rr, A2, v3(rs.To[0], rs.To[1], rs.To[2]), rs.l, rs.r);
    };
    double best = DBL_MAX;
    std::vector<int> at;
    bool contact = false;
    for (int p = 0; p < m.n_tris; ++p) {
      double P[9];
      load_tri_local(m, p, P);
      SimplexVert V[kSimplexSlots];
      D3v ps, pt;
      double d;
      shape_triangle_distance(A, Rs, ts, P, Rm, tm, V, d, ps, pt);
      if (!(d > 0.0)) contact = true;
      if (d < best) {
        best = d;
        at.assign(1, p);
      } else if (d == best) {
        at.push_back(p);
      }
    }
    ties[i] = (int32_t)at.size();
    dist[i] = best;
    tri[i] = -1;
    if (contact) continue;
    // FCL's first of the tied triangles
    auto path = [&](int p) {
      std::vector<int> up;
      for (int b = leaf_of[p]; b >= 0; b = parent[b]) up.push_back(b);
      return std::vector<int>(up.rbegin(), up.rend());  // root first
    };
    auto first = [&](int a, int b) {
      if (a == 0) return a;
      if (b == 0) return b;
      const std::vector<int> pa = path(a), pb = path(b);
      size_t k = 0;
      while (pa[k + 1] == pb[k + 1]) ++k;  // pa[k] is the deepest common node
      const int c = m.nodes64[pa[k]].child;
      const bool second_first = bvd(c + 1) < bvd(c);
      const bool a_second = pa[k + 1] == c + 1;
      return a_second == second_first ? a : b;
    };
    int w = at[0];
    for (size_t j = 1; j < at.size(); ++j) w = first(w, at[j]);
    tri[i] = w;
  }
}

}  // extern "C"
