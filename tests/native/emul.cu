// Test-only host build of the product's traversal code (collide_traverse.cuh) and
// BVH construction (bvh_build.cpp), so the kernel logic -- FP32 filters, FP64
// rechecks, visit order -- can be compared with the oracle without a GPU.  This
// library is built by the tests into tests/native/_build/ and is never shipped.
#include <vector>

#include "bvh_build.h"
#include "collide_traverse.cuh"

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
}

struct VecSink {
  std::vector<int>* out;
  void push(int, int, int b1, int b2) {
    out->push_back(b1);
    out->push_back(b2);
  }
};

}  // namespace

extern "C" {

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
    for (int k = 0; k < 9; ++k) o[15 + k] = n.axis[k];
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
