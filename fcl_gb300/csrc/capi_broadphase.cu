// C ABI of the device broadphase (include/fclgpu.h): scene registration and update,
// batched per-object collide and distance queries with FCL's default callbacks.
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <chrono>
#include <cmath>
#include <cstring>
#include <limits>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/fclgpu.h"
#include "broadphase.h"
#include "kernels.h"
#include "mesh_handle.h"
#include "mesh_shape.cuh"
#include "mesh_shape.h"
#include "shape_pair.cuh"
#include "shapeset_handle.h"

using namespace fclgpu;

struct fclgpu_broadphase_s {
  fclgpu_shapeset shapes = nullptr;
  std::vector<fclgpu_mesh> meshes;
  std::vector<int32_t> mesh_pairs;  // nm x nm table, pair p = a * nm + b -> (a, b)
  int32_t ns = 0, nm = 0, n = 0, root = -1;
  GeomRec* geoms = nullptr;
  int32_t* gid = nullptr;
  double* tf = nullptr;
  double* aabb64 = nullptr;
  float* aabb32 = nullptr;
  BpNode* nodes = nullptr;
  void* build_scratch = nullptr;
  DevMesh* dmeshes = nullptr;  // device table of the meshes, for mesh-shape pairs
  int max_depth = 0;
  void* sbv = nullptr;         // the objects' shape BVs at their current poses (ShapeBV)
  int32_t* sbv_ok = nullptr;   // per object: sbv holds its BV (reset by every pose update)
};

namespace {

std::mutex g_bp_mu;

int bp_fail(int code, const std::string& why) {
  set_error_detail(why);
  return code;
}
int bp_cuda(cudaError_t e, const char* where) {
  set_error_detail(std::string(where) + ": " + cudaGetErrorString(e));
  return e == cudaErrorMemoryAllocation ? FCLGPU_ERR_OUT_OF_MEMORY : FCLGPU_ERR_CUDA;
}
#define CKB(expr, where)                            \
  do {                                              \
    cudaError_t e_ = (expr);                        \
    if (e_ != cudaSuccess) return bp_cuda(e_, where); \
  } while (0)
#define RCB(expr)         \
  do {                    \
    int r_ = (expr);      \
    if (r_) return r_;    \
  } while (0)

struct Buf {
  void* p = nullptr;
  size_t cap = 0;
  cudaError_t ensure(size_t bytes) {
    if (bytes <= cap) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
    const size_t want = std::max<size_t>(bytes + bytes / 4, 256);
    cudaError_t e = cudaMalloc(&p, want);
    if (e == cudaSuccess) cap = want;
    return e;
  }
  template <class T>
  T* as() const {
    return static_cast<T*>(p);
  }
};

// query-side scratch (one set, calls are serialised by g_bp_mu)
struct BpScratch {
  Buf ctr, qgid, q64, q32, counts, offsets, scan_tmp, ub;
  Buf pairs, kind, hit, dist, b12, pts, list;
  Buf m_pair, m_tf1, m_tf2, m_counts, m_dist, m_ids, m_pts;
  Buf x_midx, x_sidx, x_counts, x_tri, qdone, x_bvsrc, x_need, x_bvtab, x_group, x_gcount;
  // contact lists: mesh-shape lists and slot index, mesh-mesh lists and slot index,
  // the per-query order of the slots and the scanned contact counts
  Buf x_loff, x_ltris, x_index, mm_off, mm_cont, mm_index, perm, ccount, coff, c_out;
  Buf h_refs, h_tf, h_out1, h_out2, h_out3, h_out4;
};
BpScratch g_bs;

// Phase times of collide (row 0) and distance (row 1) calls, accumulated until read, ms:
// [0] query prep + candidate passes, [1] shape-shape pairs, [2] mesh-shape pairs,
// [3] mesh-mesh pairs, [4] reduction; [5] candidates, [6] mesh-shape and [7] mesh-mesh
// pairs evaluated.
double g_phase[2][8];
int64_t g_last_mixed = 0;

struct PhaseClock {
  int row;
  cudaStream_t s;
  std::chrono::steady_clock::time_point t;
  PhaseClock(int r, cudaStream_t st) : row(r), s(st), t(std::chrono::steady_clock::now()) {
    (void)r;
  }
  void tick(int k) {
    cudaStreamSynchronize(s);
    const auto now = std::chrono::steady_clock::now();
    g_phase[row][k] += std::chrono::duration<double, std::milli>(now - t).count();
    t = now;
  }
};

// device counters block
struct BpCounters {
  unsigned status;
  unsigned pad;
  unsigned long long list_count;
  int64_t visits;
};

// Shape::computeLocalAABB per type, in FCL's operation order (see oracle restatement)
void shape_record(const DevShape& s, const double* verts, GeomRec& g) {
  g.kind = GEOM_SHAPE;
  for (int k = 0; k < 3; ++k) g.ref[k] = 0.0;
  double d[3];
  switch (s.type) {
    case FCLGPU_SHAPE_BOX:  // box-inl.h:80-88: 0.5 * side
      for (int k = 0; k < 3; ++k) d[k] = 0.5 * s.p[k];
      break;
    case FCLGPU_SHAPE_SPHERE:  // sphere-inl.h:62-69
      d[0] = d[1] = d[2] = s.p[0];
      break;
    case FCLGPU_SHAPE_CAPSULE:  // capsule-inl.h:64-72
      d[0] = d[1] = s.p[0];
      d[2] = 0.5 * s.p[1] + s.p[0];
      break;
    case FCLGPU_SHAPE_CYLINDER:  // cylinder-inl.h:64-72
    case FCLGPU_SHAPE_CONE:      // cone-inl.h:64-72
      d[0] = d[1] = s.p[0];
      d[2] = 0.5 * s.p[1];
      break;
    default: {  // convex-inl.h:86-96
      double lo[3], hi[3];
      for (int k = 0; k < 3; ++k) {
        lo[k] = std::numeric_limits<double>::max();
        hi[k] = -std::numeric_limits<double>::max();
      }
      for (int i = 0; i < s.vcnt; ++i)
        for (int k = 0; k < 3; ++k) {
          lo[k] = std::min(lo[k], verts[3 * (s.voff + i) + k]);
          hi[k] = std::max(hi[k], verts[3 * (s.voff + i) + k]);
        }
      double m[3];
      for (int k = 0; k < 3; ++k) {
        g.lo[k] = lo[k];
        g.hi[k] = hi[k];
        g.center[k] = (lo[k] + hi[k]) * 0.5;
        m[k] = lo[k] - g.center[k];
        g.ref[k] = verts[3 * s.voff + k];
      }
      g.radius = std::sqrt((m[0] * m[0] + m[1] * m[1]) + m[2] * m[2]);
      return;
    }
  }
  double m[3];
  for (int k = 0; k < 3; ++k) {
    g.hi[k] = d[k];
    g.lo[k] = -d[k];
    g.center[k] = (g.lo[k] + g.hi[k]) * 0.5;
    m[k] = g.lo[k] - g.center[k];
  }
  g.radius = s.type == FCLGPU_SHAPE_SPHERE ? s.p[0] : std::sqrt((m[0] * m[0] + m[1] * m[1]) + m[2] * m[2]);
}

BpSceneView scene_view(const fclgpu_broadphase_s* bp) {
  BpSceneView S;
  S.geoms = bp->geoms;
  S.shapes = bp->shapes ? bp->shapes->shapes : nullptr;
  S.sverts = bp->shapes ? bp->shapes->verts : nullptr;
  S.meshes = nullptr;
  S.n = bp->n;
  S.root = bp->root;
  S.gid = bp->gid;
  S.tf = bp->tf;
  S.aabb64 = bp->aabb64;
  S.nodes = bp->nodes;
  S.bv_cache = bp->sbv;
  S.bv_ok = bp->sbv_ok;
  return S;
}

// AABBs + tree for the current poses
int rebuild(fclgpu_broadphase_s* bp, cudaStream_t s) {
  if (bp->n == 0) return FCLGPU_OK;
  if (bp->sbv_ok) CKB(cudaMemsetAsync(bp->sbv_ok, 0, 4 * (size_t)bp->n, s), "shape BV cache");
  CKB(launch_world_aabbs(bp->geoms, bp->n, bp->gid, bp->tf, bp->aabb64, bp->aabb32, s), "world aabbs");
  if (bp->n >= 2) {
    CKB(launch_lbvh_build(bp->n, bp->aabb32, bp->nodes, bp->build_scratch, s), "lbvh build");
    bp->root = 0;
  } else {
    bp->root = ~0;
  }
  CKB(cudaStreamSynchronize(s), "broadphase build");
  return FCLGPU_OK;
}

void free_bp(fclgpu_broadphase_s* bp) {
  for (void* p : {(void*)bp->geoms, (void*)bp->gid, (void*)bp->tf, (void*)bp->aabb64, (void*)bp->aabb32,
                  (void*)bp->nodes, bp->build_scratch, (void*)bp->dmeshes, bp->sbv, (void*)bp->sbv_ok})
    if (p) cudaFree(p);
  delete bp;
}

// Query preparation: registry ids, world AABBs.
int prepare_queries(const fclgpu_broadphase_s* bp, const fclgpu_geometry_ref* refs, int64_t nq, const double* tf,
                    BpQueryView& Q, BpCounters* dctr, cudaStream_t s) {
  CKB(g_bs.qgid.ensure(4 * nq), "query scratch");
  CKB(g_bs.q64.ensure(48 * nq), "query scratch");
  CKB(g_bs.q32.ensure(24 * nq), "query scratch");
  CKB(launch_bp_query_gids(reinterpret_cast<const int2*>(refs), nq, bp->ns, bp->nm, g_bs.qgid.as<int32_t>(),
                           &dctr->status, s),
      "query refs");
  CKB(launch_world_aabbs(bp->geoms, nq, g_bs.qgid.as<int32_t>(), tf, g_bs.q64.as<double>(), g_bs.q32.as<float>(), s),
      "query aabbs");
  Q.nq = nq;
  Q.gid = g_bs.qgid.as<int32_t>();
  Q.tf = tf;
  Q.aabb64 = g_bs.q64.as<double>();
  Q.aabb32 = g_bs.q32.as<float>();
  return FCLGPU_OK;
}

int check_status(const BpCounters& c) {
  if (c.status & BP_ERR_REF) return bp_fail(FCLGPU_ERR_INVALID_ARGUMENT, "query geometry ref out of range");
  if (c.status & BP_ERR_STACK) return bp_fail(FCLGPU_ERR_STACK_DEPTH, "broadphase traversal stack overflow");
  if (c.status) return bp_fail(FCLGPU_ERR_DEVICE_STATUS, "broadphase status word set");
  return FCLGPU_OK;
}

// counts -> offsets -> total; returns the total through *total (host sync)
int scan_counts(int64_t nq, BpCounters* dctr, BpCounters* hctr, int64_t* total, cudaStream_t s) {
  CKB(g_bs.offsets.ensure(8 * (nq + 1)), "offsets");
  CKB(g_bs.scan_tmp.ensure(8 * ((nq + 4095) / 4096 + 2)), "scan scratch");
  CKB(launch_exclusive_scan(g_bs.counts.as<int32_t>(), nq, g_bs.offsets.as<int64_t>(), g_bs.scan_tmp.as<int64_t>(),
                            s),
      "scan");
  CKB(cudaMemcpyAsync(total, g_bs.offsets.as<int64_t>() + nq, 8, cudaMemcpyDeviceToHost, s), "read total");
  CKB(cudaMemcpyAsync(hctr, dctr, sizeof(BpCounters), cudaMemcpyDeviceToHost, s), "read counters");
  CKB(cudaStreamSynchronize(s), "candidate pass");
  return check_status(*hctr);
}

int ensure_pair_buffers(int64_t total) {
  const size_t t = (size_t)std::max<int64_t>(total, 1);
  CKB(g_bs.pairs.ensure(8 * t), "pairs");
  CKB(g_bs.kind.ensure(4 * t), "pairs");
  CKB(g_bs.list.ensure(8 * t), "pairs");
  return FCLGPU_OK;
}

// list of candidates of one kind; returns its length (host sync)
int list_kind(int64_t total, int32_t want, BpCounters* dctr, int64_t* nlist, cudaStream_t s,
              const int32_t* qdone = nullptr) {
  CKB(cudaMemsetAsync(&dctr->list_count, 0, 8, s), "list");
  CKB(launch_bp_list(g_bs.kind.as<int32_t>(), total, want, g_bs.pairs.as<int2>(), qdone, g_bs.list.as<int64_t>(),
                     &dctr->list_count, s),
      "list");
  unsigned long long c = 0;
  CKB(cudaMemcpyAsync(&c, &dctr->list_count, 8, cudaMemcpyDeviceToHost, s), "list");
  CKB(cudaStreamSynchronize(s), "list");
  *nlist = (int64_t)c;
  return FCLGPU_OK;
}

// Mesh-shape candidates (kind 2): BVH-shape collide (mode 0, contacts into hit) or
// distance (mode 1, into the distance slots), mesh first as FCL calls it.
// With lists (collide only): every listed pair's triangle list (g_bs.x_loff,
// g_bs.x_ltris) and index[slot] = its list position (g_bs.x_index).
int run_mixed(const fclgpu_broadphase_s* bp, const BpSceneView& S, const BpQueryView& Q, int64_t total, int mode,
              int64_t max_contacts, BpCounters* dctr, cudaStream_t s, const int32_t* qdone = nullptr,
              bool lists = false, bool witness = true) {
  int64_t nl = 0;
  RCB(list_kind(total, 2, dctr, &nl, s, qdone));
  g_last_mixed = nl;
  if (nl == 0) return FCLGPU_OK;
  if (!bp->shapes || !bp->dmeshes) return bp_fail(FCLGPU_ERR_INVALID_ARGUMENT, "mesh-shape pair without registry");
  CKB(g_bs.x_midx.ensure(4 * nl), "mixed scratch");
  CKB(g_bs.x_sidx.ensure(4 * nl), "mixed scratch");
  CKB(g_bs.m_tf1.ensure(96 * nl), "mixed scratch");
  CKB(g_bs.m_tf2.ensure(96 * nl), "mixed scratch");
  CKB(g_bs.x_counts.ensure(4 * nl), "mixed scratch");
  CKB(g_bs.m_dist.ensure(8 * nl), "mixed scratch");
  CKB(g_bs.x_tri.ensure(4 * nl), "mixed scratch");
  CKB(g_bs.m_pts.ensure(48 * nl), "mixed scratch");
  // one shape BV per (shape, pose) source, shared by all its mesh-shape pairs (sources
  // are int32 indices; beyond that every pair fits its own)
  const int64_t nsrc = Q.nq + S.n;
  const bool table = nsrc < INT32_MAX;
  if (table) {
    CKB(g_bs.x_bvsrc.ensure(4 * nl), "mixed scratch");
    CKB(g_bs.x_need.ensure(4 * nsrc), "mixed scratch");
    CKB(g_bs.x_bvtab.ensure(sizeof(ShapeBV) * nsrc), "mixed scratch");
    CKB(cudaMemsetAsync(g_bs.x_need.p, 0, 4 * nsrc, s), "mixed scratch");
  }
  // collide without exhaustive search: a query's mesh-shape pairs stop together once
  // the query has num_max_contacts contacts (FCL's manager stops visiting objects then)
  const bool grouped = mode == 0 && qdone != nullptr;
  if (grouped) {
    CKB(g_bs.x_group.ensure(4 * nl), "mixed scratch");
    CKB(g_bs.x_gcount.ensure(8 * Q.nq), "mixed scratch");
    CKB(cudaMemsetAsync(g_bs.x_gcount.p, 0, 8 * Q.nq, s), "mixed scratch");
  }
  CKB(launch_bp_gather_mixed(S, Q, g_bs.pairs.as<int2>(), g_bs.list.as<int64_t>(), nl, g_bs.x_midx.as<int32_t>(),
                             g_bs.x_sidx.as<int32_t>(), g_bs.m_tf1.as<double>(), g_bs.m_tf2.as<double>(),
                             table ? g_bs.x_bvsrc.as<int32_t>() : nullptr,
                             table ? g_bs.x_need.as<int32_t>() : nullptr, grouped ? g_bs.x_group.as<int32_t>() : nullptr,
                             s),
      "mixed gather");
  if (table) CKB(launch_bp_shape_bvs(S, Q, g_bs.x_need.as<int32_t>(), g_bs.x_bvtab.p, s), "shape BVs");
  MeshShapeLaunch L;
  L.meshes = bp->dmeshes;
  L.shapes = bp->shapes->shapes;
  L.sverts = bp->shapes->verts;
  L.n = nl;
  L.mesh_idx = g_bs.x_midx.as<int32_t>();
  L.shape_idx = g_bs.x_sidx.as<int32_t>();
  L.tfm = g_bs.m_tf1.as<double>();
  L.tfs = g_bs.m_tf2.as<double>();
  L.mode = mode;
  L.max_contacts = (int32_t)std::min<int64_t>(max_contacts, INT32_MAX);
  L.counts = g_bs.x_counts.as<int32_t>();
  L.dist = g_bs.m_dist.as<double>();
  L.tri = g_bs.x_tri.as<int32_t>();
  L.pts = g_bs.m_pts.as<double>();
  if (mode == 1 && !witness) {  // values only: the triangle ids and points stay unset
    CKB(cudaMemsetAsync(g_bs.x_tri.p, 0xff, 4 * nl, s), "mixed scratch");
    CKB(cudaMemsetAsync(g_bs.m_pts.p, 0, 48 * nl, s), "mixed scratch");
    L.tri = nullptr;
    L.pts = nullptr;
  }
  L.nbv = nullptr;
  L.nleaf = nullptr;
  L.status = &dctr->status;
  L.bv_table = table ? g_bs.x_bvtab.p : nullptr;
  L.bv_src = table ? g_bs.x_bvsrc.as<int32_t>() : nullptr;
  if (grouped) {
    L.group = g_bs.x_group.as<int32_t>();
    L.group_count = (unsigned long long*)g_bs.x_gcount.p;
    L.group_max = max_contacts;
  }
  if (lists) {
    CKB(g_bs.x_loff.ensure(8 * (nl + 1)), "mixed lists");
    CKB(g_bs.x_ltris.ensure(4 * std::max<int64_t>(nl, 1024)), "mixed lists");
    CKB(g_bs.x_index.ensure(4 * std::max<int64_t>(total, 1)), "mixed lists");
    L.list_offsets = g_bs.x_loff.as<int64_t>();
    L.list_tris = g_bs.x_ltris.as<int32_t>();
    L.list_cap = (int64_t)(g_bs.x_ltris.cap / 4);
    int64_t ltotal = 0;
    L.list_total = &ltotal;
    CKB(run_mesh_shape_split(L, bp->max_depth + 2, s), "mesh-shape narrowphase");
    if (ltotal > L.list_cap) {  // the lists did not fit: once more with room for all of them
      CKB(g_bs.x_ltris.ensure(4 * (size_t)ltotal), "mixed lists");
      L.list_tris = g_bs.x_ltris.as<int32_t>();
      L.list_cap = (int64_t)(g_bs.x_ltris.cap / 4);
      CKB(run_mesh_shape_split(L, bp->max_depth + 2, s), "mesh-shape narrowphase");
    }
    CKB(launch_bp_inverse_index(g_bs.list.as<int64_t>(), nl, g_bs.x_index.as<int32_t>(), s), "mixed index");
  } else {
    CKB(run_mesh_shape_split(L, bp->max_depth + 2, s), "mesh-shape narrowphase");
  }
  if (mode == 0) {
    CKB(launch_bp_scatter_hits(g_bs.list.as<int64_t>(), nl, g_bs.x_counts.as<int32_t>(), g_bs.hit.as<int32_t>(), s),
        "mixed scatter");
  } else {
    CKB(launch_bp_scatter_mixed_dist(g_bs.list.as<int64_t>(), nl, g_bs.m_dist.as<double>(), g_bs.x_tri.as<int32_t>(),
                                     g_bs.m_pts.as<double>(), g_bs.dist.as<double>(), g_bs.b12.as<int32_t>(),
                                     g_bs.pts.as<double>(), s),
        "mixed scatter");
  }
  return FCLGPU_OK;
}

}  // namespace

extern "C" {

int fclgpu_broadphase_create(fclgpu_shapeset shapes, const fclgpu_mesh* meshes, int32_t num_meshes,
                             const fclgpu_geometry_ref* objects, int32_t num_objects, const double* tf,
                             fclgpu_broadphase* out) {
  if (!out) return bp_fail(FCLGPU_ERR_INVALID_ARGUMENT, "out is null");
  *out = nullptr;
  if (num_meshes < 0 || num_objects < 0 || (num_meshes > 0 && !meshes) || (num_objects > 0 && (!objects || !tf)))
    return bp_fail(FCLGPU_ERR_INVALID_ARGUMENT, "bad broadphase arguments");
  const int32_t ns = shapes ? shapes->n : 0;
  for (int32_t i = 0; i < num_meshes; ++i)
    if (!meshes[i]) return bp_fail(FCLGPU_ERR_INVALID_ARGUMENT, "null mesh handle");
  if ((int64_t)num_meshes * num_meshes > (1 << 22)) return bp_fail(FCLGPU_ERR_UNSUPPORTED, "too many meshes");
  std::vector<int32_t> gid(num_objects);
  for (int32_t i = 0; i < num_objects; ++i) {
    const fclgpu_geometry_ref r = objects[i];
    if (r.kind == FCLGPU_GEOM_SHAPE && r.index >= 0 && r.index < ns)
      gid[i] = r.index;
    else if (r.kind == FCLGPU_GEOM_MESH && r.index >= 0 && r.index < num_meshes)
      gid[i] = ns + r.index;
    else
      return bp_fail(FCLGPU_ERR_INVALID_ARGUMENT, "scene geometry ref out of range");
  }
  std::vector<GeomRec> geoms(ns + num_meshes);
  for (int32_t i = 0; i < ns; ++i) {
    std::memset(&geoms[i], 0, sizeof(GeomRec));
    shape_record(shapes->host[i], shapes->host_verts.data(), geoms[i]);
    geoms[i].index = i;
  }
  for (int32_t i = 0; i < num_meshes; ++i) {
    GeomRec& g = geoms[ns + i];
    std::memset(&g, 0, sizeof(GeomRec));
    g.kind = GEOM_MESH;
    g.index = i;
    for (int k = 0; k < 3; ++k) {
      g.lo[k] = meshes[i]->aabb_local[k];
      g.hi[k] = meshes[i]->aabb_local[3 + k];
      g.center[k] = meshes[i]->aabb_center[k];
      g.ref[k] = meshes[i]->first_vertex[k];
    }
    g.radius = meshes[i]->aabb_radius;
  }
  std::lock_guard<std::mutex> lk(g_bp_mu);
  fclgpu_broadphase_s* bp = new fclgpu_broadphase_s();
  bp->shapes = shapes;
  bp->meshes.assign(meshes, meshes + num_meshes);
  bp->ns = ns;
  bp->nm = num_meshes;
  bp->n = num_objects;
  bp->mesh_pairs.resize(2 * (size_t)num_meshes * num_meshes);
  for (int32_t a = 0; a < num_meshes; ++a)
    for (int32_t b = 0; b < num_meshes; ++b) {
      bp->mesh_pairs[2 * ((size_t)a * num_meshes + b)] = a;
      bp->mesh_pairs[2 * ((size_t)a * num_meshes + b) + 1] = b;
    }
  const size_t n = (size_t)std::max(num_objects, 1);
  cudaError_t e = cudaMalloc(&bp->geoms, sizeof(GeomRec) * std::max<size_t>(geoms.size(), 1));
  if (e == cudaSuccess) e = cudaMalloc(&bp->gid, 4 * n);
  if (e == cudaSuccess) e = cudaMalloc(&bp->tf, 96 * n);
  if (e == cudaSuccess) e = cudaMalloc(&bp->aabb64, 48 * n);
  if (e == cudaSuccess) e = cudaMalloc(&bp->aabb32, 24 * n);
  if (e == cudaSuccess) e = cudaMalloc(&bp->nodes, sizeof(BpNode) * n);
  if (e == cudaSuccess) e = cudaMalloc(&bp->build_scratch, bp_build_scratch_bytes((int64_t)n));
  if (e == cudaSuccess && shapes) e = cudaMalloc(&bp->sbv, sizeof(ShapeBV) * n);
  if (e == cudaSuccess && shapes) e = cudaMalloc(&bp->sbv_ok, 4 * n);
  if (e == cudaSuccess && !geoms.empty())
    e = cudaMemcpy(bp->geoms, geoms.data(), sizeof(GeomRec) * geoms.size(), cudaMemcpyHostToDevice);
  if (e == cudaSuccess && num_objects > 0) e = cudaMemcpy(bp->gid, gid.data(), 4 * n, cudaMemcpyHostToDevice);
  if (e == cudaSuccess && num_objects > 0) e = cudaMemcpy(bp->tf, tf, 96 * n, cudaMemcpyHostToDevice);
  if (e == cudaSuccess && num_meshes > 0) {
    std::vector<DevMesh> table(num_meshes);
    for (int32_t i = 0; i < num_meshes; ++i) {
      table[i] = meshes[i]->dev;
      bp->max_depth = std::max(bp->max_depth, (int)meshes[i]->dev.max_depth);
    }
    e = cudaMalloc(&bp->dmeshes, sizeof(DevMesh) * num_meshes);
    if (e == cudaSuccess)
      e = cudaMemcpy(bp->dmeshes, table.data(), sizeof(DevMesh) * num_meshes, cudaMemcpyHostToDevice);
  }
  if (e != cudaSuccess) {
    free_bp(bp);
    return bp_cuda(e, "broadphase upload");
  }
  const int rc = rebuild(bp, nullptr);
  if (rc) {
    free_bp(bp);
    return rc;
  }
  *out = bp;
  return FCLGPU_OK;
}

int fclgpu_broadphase_update(fclgpu_broadphase bp, const double* tf, int32_t tf_on_device, void* stream) {
  if (!bp || (bp->n > 0 && !tf)) return bp_fail(FCLGPU_ERR_INVALID_ARGUMENT, "bad update arguments");
  std::lock_guard<std::mutex> lk(g_bp_mu);
  cudaStream_t s = (cudaStream_t)stream;
  if (bp->n > 0)
    CKB(cudaMemcpyAsync(bp->tf, tf, 96 * (size_t)bp->n, tf_on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                        s),
        "update poses");
  return rebuild(bp, s);
}

int fclgpu_broadphase_destroy(fclgpu_broadphase bp) {
  if (!bp) return FCLGPU_OK;
  std::lock_guard<std::mutex> lk(g_bp_mu);
  cudaDeviceSynchronize();
  free_bp(bp);
  return FCLGPU_OK;
}

int fclgpu_broadphase_get_aabbs(fclgpu_broadphase bp, double* aabb6) {
  if (!bp || (bp->n > 0 && !aabb6)) return bp_fail(FCLGPU_ERR_INVALID_ARGUMENT, "bad arguments");
  std::lock_guard<std::mutex> lk(g_bp_mu);
  if (bp->n > 0) CKB(cudaMemcpy(aabb6, bp->aabb64, 48 * (size_t)bp->n, cudaMemcpyDeviceToHost), "read aabbs");
  return FCLGPU_OK;
}

int fclgpu_broadphase_collide_device(fclgpu_broadphase bp, const fclgpu_geometry_ref* queries, int64_t nq,
                                     const double* tf, const fclgpu_broadphase_collide_request* req,
                                     fclgpu_broadphase_collide_result* res, void* stream) {
  if (!bp || !req || !res || nq < 0 || (nq > 0 && (!queries || !tf || !res->num_contacts)))
    return bp_fail(FCLGPU_ERR_INVALID_ARGUMENT, "missing broadphase collide argument");
  if (req->num_max_contacts < 1) return bp_fail(FCLGPU_ERR_INVALID_ARGUMENT, "num_max_contacts must be >= 1");
  if (req->precision != FCLGPU_PLAIN_FP64 && req->precision != FCLGPU_FP32_RECHECK)
    return bp_fail(FCLGPU_ERR_INVALID_ARGUMENT, "unknown precision");
  if (nq >= ((int64_t)1 << 31)) return bp_fail(FCLGPU_ERR_INVALID_ARGUMENT, "too many queries");
  std::lock_guard<std::mutex> lk(g_bp_mu);
  cudaStream_t s = (cudaStream_t)stream;
  res->total_candidates = 0;
  res->total_node_visits = 0;
  if (nq == 0) return FCLGPU_OK;
  PhaseClock pc(0, s);
  g_last_mixed = 0;
  CKB(g_bs.ctr.ensure(sizeof(BpCounters)), "counters");
  BpCounters* dctr = g_bs.ctr.as<BpCounters>();
  CKB(cudaMemsetAsync(dctr, 0, sizeof(BpCounters), s), "counters");
  BpQueryView Q;
  RCB(prepare_queries(bp, queries, nq, tf, Q, dctr, s));
  const BpSceneView S = scene_view(bp);
  CKB(g_bs.counts.ensure(4 * nq), "counts");
  CKB(launch_bp_overlap(S, Q, g_bs.counts.as<int32_t>(), nullptr, nullptr, &dctr->visits, &dctr->status, s),
      "overlap count");
  BpCounters hc;
  int64_t total = 0;
  RCB(scan_counts(nq, dctr, &hc, &total, s));
  res->total_candidates = total;
  res->total_node_visits = hc.visits;
  g_phase[0][5] += (double)total;
  RCB(ensure_pair_buffers(total));
  CKB(g_bs.hit.ensure(4 * (size_t)std::max<int64_t>(total, 1)), "hits");
  const int64_t* off = g_bs.offsets.as<int64_t>();
  int2* pairs = g_bs.pairs.as<int2>();
  int32_t* hit = g_bs.hit.as<int32_t>();
  if (total > 0) {
    CKB(launch_bp_overlap(S, Q, nullptr, off, pairs, nullptr, &dctr->status, s), "overlap write");
    CKB(launch_bp_classify(S, Q, pairs, total, g_bs.kind.as<int32_t>(), s), "classify");
    CKB(cudaMemsetAsync(hit, 0, 4 * (size_t)total, s), "hits");
    pc.tick(0);
    CKB(launch_bp_shape_narrow(S, Q, pairs, total, g_bs.kind.as<int32_t>(), PAIR_INTERSECT, hit, nullptr, nullptr,
                               s),
        "shape narrowphase");
    pc.tick(1);
    // without exhaustive evaluation a query stops once it has num_max_contacts
    // contacts, as DefaultCollisionFunction stops FCL's traversal: cheaper pair kinds
    // run first and later kinds skip finished queries
    int32_t* qdone = nullptr;
    if (!req->exhaustive) {
      CKB(g_bs.qdone.ensure(4 * nq), "query flags");
      qdone = g_bs.qdone.as<int32_t>();
      CKB(launch_bp_query_done(nq, off, hit, req->num_max_contacts, qdone, s), "query flags");
    }
    RCB(run_mixed(bp, S, Q, total, 0, req->num_max_contacts, dctr, s, qdone));
    g_phase[0][6] += (double)g_last_mixed;
    pc.tick(2);
    if (qdone) CKB(launch_bp_query_done(nq, off, hit, req->num_max_contacts, qdone, s), "query flags");
    int64_t nl = 0;
    RCB(list_kind(total, 1, dctr, &nl, s, qdone));
    g_phase[0][7] += (double)nl;
    if (nl > 0) {
      CKB(g_bs.m_pair.ensure(4 * nl), "mesh scratch");
      CKB(g_bs.m_tf1.ensure(96 * nl), "mesh scratch");
      CKB(g_bs.m_tf2.ensure(96 * nl), "mesh scratch");
      CKB(g_bs.m_counts.ensure(4 * nl), "mesh scratch");
      CKB(launch_bp_gather_mesh(S, Q, pairs, g_bs.list.as<int64_t>(), nl, bp->nm, g_bs.m_pair.as<int32_t>(),
                                g_bs.m_tf1.as<double>(), g_bs.m_tf2.as<double>(), s),
          "mesh gather");
      fclgpu_collide_request mr = {(int32_t)std::min<int64_t>(req->num_max_contacts, INT32_MAX), req->precision, 0,
                                   0};
      fclgpu_collide_result mres = {g_bs.m_counts.as<int32_t>(), nullptr, nullptr, 0, nullptr, nullptr, nullptr, 0};
      const int rc = fclgpu_collide_batch_device(bp->meshes.data(), bp->nm, bp->mesh_pairs.data(), bp->nm * bp->nm,
                                                 nl, g_bs.m_pair.as<int32_t>(), g_bs.m_tf1.as<double>(),
                                                 g_bs.m_tf2.as<double>(), &mr, &mres, stream);
      if (rc) return rc;
      CKB(launch_bp_scatter_hits(g_bs.list.as<int64_t>(), nl, g_bs.m_counts.as<int32_t>(), hit, s), "mesh scatter");
    }
    pc.tick(3);
  }
  CKB(launch_bp_reduce_collide(nq, off, pairs, hit, req->num_max_contacts, res->num_contacts, res->num_objects,
                               res->first_object, s),
      "reduce");
  CKB(cudaMemcpyAsync(&hc, dctr, sizeof(BpCounters), cudaMemcpyDeviceToHost, s), "read counters");
  CKB(cudaStreamSynchronize(s), "broadphase collide");
  pc.tick(4);
  return check_status(hc);
}

}  // extern "C"

namespace {

// The broadphase distance of the queries Q (per query: the nearest scene object among
// the candidates, its triangle ids and world witness points).
int distance_core(fclgpu_broadphase_s* bp, const BpQueryView& Q, const fclgpu_broadphase_distance_request* req,
                  fclgpu_broadphase_distance_result* res, BpCounters* dctr, cudaStream_t s, PhaseClock& pc) {
  const int64_t nq = Q.nq;
  const BpSceneView S = scene_view(bp);
  CKB(g_bs.ub.ensure(8 * nq), "bounds");
  CKB(g_bs.counts.ensure(4 * nq), "counts");
  CKB(launch_bp_dist_bound(S, Q, g_bs.ub.as<double>(), &dctr->status, s), "distance bound");
  CKB(launch_bp_dist_candidates(S, Q, g_bs.ub.as<double>(), g_bs.counts.as<int32_t>(), nullptr, nullptr,
                                &dctr->visits, &dctr->status, s),
      "distance count");
  BpCounters hc;
  int64_t total = 0;
  RCB(scan_counts(nq, dctr, &hc, &total, s));
  res->total_candidates = total;
  res->total_node_visits = hc.visits;
  g_phase[1][5] += (double)total;
  RCB(ensure_pair_buffers(total));
  const size_t t = (size_t)std::max<int64_t>(total, 1);
  CKB(g_bs.dist.ensure(8 * t), "distances");
  CKB(g_bs.b12.ensure(8 * t), "distances");
  CKB(g_bs.pts.ensure(48 * t), "distances");
  const int64_t* off = g_bs.offsets.as<int64_t>();
  int2* pairs = g_bs.pairs.as<int2>();
  double* dist = g_bs.dist.as<double>();
  int32_t* b12 = g_bs.b12.as<int32_t>();
  double* pts = g_bs.pts.as<double>();
  if (total > 0) {
    CKB(launch_bp_dist_candidates(S, Q, g_bs.ub.as<double>(), nullptr, off, pairs, nullptr, &dctr->status, s),
        "distance write");
    CKB(launch_bp_classify(S, Q, pairs, total, g_bs.kind.as<int32_t>(), s), "classify");
    CKB(cudaMemsetAsync(b12, 0xff, 8 * (size_t)total, s), "ids");
    pc.tick(0);
    CKB(launch_bp_shape_narrow(S, Q, pairs, total, g_bs.kind.as<int32_t>(), PAIR_DISTANCE, nullptr, dist, pts, s),
        "shape narrowphase");
    pc.tick(1);
    // the per-pair triangle and points matter only for ids or nearest points
    const bool witness = res->ids || (req->enable_nearest_points && res->nearest_points);
    RCB(run_mixed(bp, S, Q, total, 1, 0, dctr, s, nullptr, false, witness));
    g_phase[1][6] += (double)g_last_mixed;
    pc.tick(2);
    int64_t nl = 0;
    RCB(list_kind(total, 1, dctr, &nl, s));
    g_phase[1][7] += (double)nl;
    if (nl > 0) {
      CKB(g_bs.m_pair.ensure(4 * nl), "mesh scratch");
      CKB(g_bs.m_tf1.ensure(96 * nl), "mesh scratch");
      CKB(g_bs.m_tf2.ensure(96 * nl), "mesh scratch");
      CKB(g_bs.m_dist.ensure(8 * nl), "mesh scratch");
      CKB(g_bs.m_ids.ensure(8 * nl), "mesh scratch");
      CKB(g_bs.m_pts.ensure(48 * nl), "mesh scratch");
      CKB(launch_bp_gather_mesh(S, Q, pairs, g_bs.list.as<int64_t>(), nl, bp->nm, g_bs.m_pair.as<int32_t>(),
                                g_bs.m_tf1.as<double>(), g_bs.m_tf2.as<double>(), s),
          "mesh gather");
      // without witnesses the mesh pairs report their distances alone (ids and points
      // of the scatter below stay unset)
      fclgpu_distance_request mr = {witness ? 1 : 0, req->precision, 0, 0};
      fclgpu_distance_result mres = {g_bs.m_dist.as<double>(), witness ? g_bs.m_ids.as<int32_t>() : nullptr,
                                     witness ? g_bs.m_pts.as<double>() : nullptr, nullptr, nullptr, nullptr, nullptr,
                                     nullptr};
      if (!witness) {
        CKB(cudaMemsetAsync(g_bs.m_ids.p, 0xff, 8 * nl, s), "mesh scratch");
        CKB(cudaMemsetAsync(g_bs.m_pts.p, 0, 48 * nl, s), "mesh scratch");
      }
      const int rc = fclgpu_distance_batch_device(bp->meshes.data(), bp->nm, bp->mesh_pairs.data(),
                                                  bp->nm * bp->nm, nl, g_bs.m_pair.as<int32_t>(),
                                                  g_bs.m_tf1.as<double>(), g_bs.m_tf2.as<double>(), &mr, &mres,
                                                  (void*)s);
      if (rc) return rc;
      CKB(launch_bp_scatter_dist(g_bs.list.as<int64_t>(), nl, g_bs.m_dist.as<double>(), g_bs.m_ids.as<int32_t>(),
                                 g_bs.m_pts.as<double>(), dist, b12, pts, s),
          "mesh scatter");
    }
    pc.tick(3);
  }
  CKB(launch_bp_reduce_distance(nq, off, pairs, dist, b12, pts, res->min_distance, res->object, res->ids,
                                req->enable_nearest_points ? res->nearest_points : nullptr, s),
      "reduce");
  CKB(cudaMemcpyAsync(&hc, dctr, sizeof(BpCounters), cudaMemcpyDeviceToHost, s), "read counters");
  CKB(cudaStreamSynchronize(s), "broadphase distance");
  pc.tick(4);
  return check_status(hc);
}

}  // namespace

extern "C" {

int fclgpu_broadphase_distance_device(fclgpu_broadphase bp, const fclgpu_geometry_ref* queries, int64_t nq,
                                      const double* tf, const fclgpu_broadphase_distance_request* req,
                                      fclgpu_broadphase_distance_result* res, void* stream) {
  if (!bp || !req || !res || nq < 0 || (nq > 0 && (!queries || !tf || !res->min_distance)))
    return bp_fail(FCLGPU_ERR_INVALID_ARGUMENT, "missing broadphase distance argument");
  if (req->precision != FCLGPU_PLAIN_FP64 && req->precision != FCLGPU_FP32_RECHECK)
    return bp_fail(FCLGPU_ERR_INVALID_ARGUMENT, "unknown precision");
  if (nq >= ((int64_t)1 << 31)) return bp_fail(FCLGPU_ERR_INVALID_ARGUMENT, "too many queries");
  std::lock_guard<std::mutex> lk(g_bp_mu);
  cudaStream_t s = (cudaStream_t)stream;
  res->total_candidates = 0;
  res->total_node_visits = 0;
  if (nq == 0) return FCLGPU_OK;
  PhaseClock pc(1, s);
  g_last_mixed = 0;
  CKB(g_bs.ctr.ensure(sizeof(BpCounters)), "counters");
  BpCounters* dctr = g_bs.ctr.as<BpCounters>();
  CKB(cudaMemsetAsync(dctr, 0, sizeof(BpCounters), s), "counters");
  BpQueryView Q;
  RCB(prepare_queries(bp, queries, nq, tf, Q, dctr, s));
  return distance_core(bp, Q, req, res, dctr, s, pc);
}

int fclgpu_broadphase_collide(fclgpu_broadphase bp, const fclgpu_geometry_ref* queries, int64_t nq, const double* tf,
                              const fclgpu_broadphase_collide_request* req, fclgpu_broadphase_collide_result* res,
                              void* stream) {
  if (!bp || !req || !res || nq < 0 || (nq > 0 && (!queries || !tf || !res->num_contacts)))
    return bp_fail(FCLGPU_ERR_INVALID_ARGUMENT, "missing broadphase collide argument");
  if (nq == 0) return fclgpu_broadphase_collide_device(bp, queries, 0, tf, req, res, stream);
  cudaStream_t s = (cudaStream_t)stream;
  Buf refs, tfd, nc, no, fo;  // per-call staging (the device entry point owns the shared scratch)
  CKB(refs.ensure(8 * nq), "staging");
  CKB(tfd.ensure(96 * nq), "staging");
  CKB(nc.ensure(8 * nq), "staging");
  CKB(no.ensure(4 * nq), "staging");
  CKB(fo.ensure(4 * nq), "staging");
  CKB(cudaMemcpyAsync(refs.p, queries, 8 * nq, cudaMemcpyHostToDevice, s), "h2d");
  CKB(cudaMemcpyAsync(tfd.p, tf, 96 * nq, cudaMemcpyHostToDevice, s), "h2d");
  fclgpu_broadphase_collide_result dr = {nc.as<int64_t>(), no.as<int32_t>(), fo.as<int32_t>(), 0, 0};
  int rc = fclgpu_broadphase_collide_device(bp, refs.as<fclgpu_geometry_ref>(), nq, tfd.as<double>(), req, &dr,
                                            stream);
  if (rc == FCLGPU_OK) {
    res->total_candidates = dr.total_candidates;
    res->total_node_visits = dr.total_node_visits;
    cudaError_t e = cudaMemcpyAsync(res->num_contacts, nc.p, 8 * nq, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess && res->num_objects)
      e = cudaMemcpyAsync(res->num_objects, no.p, 4 * nq, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess && res->first_object)
      e = cudaMemcpyAsync(res->first_object, fo.p, 4 * nq, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) rc = bp_cuda(e, "d2h");
  }
  for (Buf* b : {&refs, &tfd, &nc, &no, &fo}) cudaFree(b->p);
  return rc;
}

int fclgpu_broadphase_distance(fclgpu_broadphase bp, const fclgpu_geometry_ref* queries, int64_t nq,
                               const double* tf, const fclgpu_broadphase_distance_request* req,
                               fclgpu_broadphase_distance_result* res, void* stream) {
  if (!bp || !req || !res || nq < 0 || (nq > 0 && (!queries || !tf || !res->min_distance)))
    return bp_fail(FCLGPU_ERR_INVALID_ARGUMENT, "missing broadphase distance argument");
  if (nq == 0) return fclgpu_broadphase_distance_device(bp, queries, 0, tf, req, res, stream);
  cudaStream_t s = (cudaStream_t)stream;
  Buf refs, tfd, d, ob, ids, pts;
  CKB(refs.ensure(8 * nq), "staging");
  CKB(tfd.ensure(96 * nq), "staging");
  CKB(d.ensure(8 * nq), "staging");
  CKB(ob.ensure(4 * nq), "staging");
  CKB(ids.ensure(8 * nq), "staging");
  CKB(pts.ensure(48 * nq), "staging");
  CKB(cudaMemcpyAsync(refs.p, queries, 8 * nq, cudaMemcpyHostToDevice, s), "h2d");
  CKB(cudaMemcpyAsync(tfd.p, tf, 96 * nq, cudaMemcpyHostToDevice, s), "h2d");
  // witnesses staged only when the caller asked for them (without, the mesh-shape
  // pairs take the value-only path)
  const bool want_pts = res->nearest_points && req->enable_nearest_points;
  fclgpu_broadphase_distance_result dr = {d.as<double>(), ob.as<int32_t>(), res->ids ? ids.as<int32_t>() : nullptr,
                                          want_pts ? pts.as<double>() : nullptr, 0, 0};
  int rc = fclgpu_broadphase_distance_device(bp, refs.as<fclgpu_geometry_ref>(), nq, tfd.as<double>(), req, &dr,
                                             stream);
  if (rc == FCLGPU_OK) {
    res->total_candidates = dr.total_candidates;
    res->total_node_visits = dr.total_node_visits;
    cudaError_t e = cudaMemcpyAsync(res->min_distance, d.p, 8 * nq, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess && res->object) e = cudaMemcpyAsync(res->object, ob.p, 4 * nq, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess && res->ids) e = cudaMemcpyAsync(res->ids, ids.p, 8 * nq, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess && res->nearest_points && req->enable_nearest_points)
      e = cudaMemcpyAsync(res->nearest_points, pts.p, 48 * nq, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) rc = bp_cuda(e, "d2h");
  }
  for (Buf* b : {&refs, &tfd, &d, &ob, &ids, &pts}) cudaFree(b->p);
  return rc;
}

}  // extern "C"

namespace {

// Contact lists of the candidate pairs of Q (every pair evaluated, each capped at
// num_max_contacts): per query, its contacts ordered by scene-object index, each
// object's in the order FCL's traversal of that pair adds them.  Device outputs.
int contacts_core(fclgpu_broadphase_s* bp, const BpQueryView& Q, const fclgpu_broadphase_contacts_request* req,
                  fclgpu_broadphase_contacts_result* res, BpCounters* dctr, cudaStream_t s) {
  const int64_t nq = Q.nq;
  const BpSceneView S = scene_view(bp);
  CKB(g_bs.counts.ensure(4 * nq), "counts");
  CKB(launch_bp_overlap(S, Q, g_bs.counts.as<int32_t>(), nullptr, nullptr, &dctr->visits, &dctr->status, s),
      "overlap count");
  BpCounters hc;
  int64_t total = 0;
  RCB(scan_counts(nq, dctr, &hc, &total, s));
  res->total_candidates = total;
  RCB(ensure_pair_buffers(total));
  const size_t t1 = (size_t)std::max<int64_t>(total, 1);
  CKB(g_bs.hit.ensure(4 * t1), "hits");
  const int64_t* off = g_bs.offsets.as<int64_t>();
  int2* pairs = g_bs.pairs.as<int2>();
  int32_t* hit = g_bs.hit.as<int32_t>();
  CKB(g_bs.mm_index.ensure(4 * t1), "mesh index");
  CKB(g_bs.x_index.ensure(4 * t1), "mixed index");
  if (total > 0) {
    CKB(launch_bp_overlap(S, Q, nullptr, off, pairs, nullptr, &dctr->status, s), "overlap write");
    CKB(launch_bp_classify(S, Q, pairs, total, g_bs.kind.as<int32_t>(), s), "classify");
    CKB(cudaMemsetAsync(hit, 0, 4 * (size_t)total, s), "hits");
    CKB(launch_bp_shape_narrow(S, Q, pairs, total, g_bs.kind.as<int32_t>(), PAIR_INTERSECT, hit, nullptr, nullptr,
                               s),
        "shape narrowphase");
    RCB(run_mixed(bp, S, Q, total, 0, req->num_max_contacts, dctr, s, nullptr, true));
    int64_t nl = 0;
    RCB(list_kind(total, 1, dctr, &nl, s, nullptr));
    if (nl > 0) {
      CKB(g_bs.m_pair.ensure(4 * nl), "mesh scratch");
      CKB(g_bs.m_tf1.ensure(96 * nl), "mesh scratch");
      CKB(g_bs.m_tf2.ensure(96 * nl), "mesh scratch");
      CKB(g_bs.m_counts.ensure(4 * nl), "mesh scratch");
      CKB(g_bs.mm_off.ensure(8 * (nl + 1)), "mesh scratch");
      CKB(g_bs.mm_cont.ensure(8 * std::max<int64_t>(nl, 1024)), "mesh scratch");
      CKB(launch_bp_gather_mesh(S, Q, pairs, g_bs.list.as<int64_t>(), nl, bp->nm, g_bs.m_pair.as<int32_t>(),
                                g_bs.m_tf1.as<double>(), g_bs.m_tf2.as<double>(), s),
          "mesh gather");
      fclgpu_collide_request mr = {(int32_t)std::min<int64_t>(req->num_max_contacts, INT32_MAX), req->precision, 0,
                                   0};
      for (int attempt = 0; attempt < 2; ++attempt) {
        fclgpu_collide_result mres = {g_bs.m_counts.as<int32_t>(), g_bs.mm_off.as<int64_t>(),
                                      g_bs.mm_cont.as<int32_t>(), (int64_t)(g_bs.mm_cont.cap / 8), nullptr, nullptr,
                                      nullptr, 0};
        const int rc = fclgpu_collide_batch_device(bp->meshes.data(), bp->nm, bp->mesh_pairs.data(),
                                                   bp->nm * bp->nm, nl, g_bs.m_pair.as<int32_t>(),
                                                   g_bs.m_tf1.as<double>(), g_bs.m_tf2.as<double>(), &mr, &mres,
                                                   (void*)s);
        if (rc == FCLGPU_ERR_CAPACITY && attempt == 0) {
          CKB(g_bs.mm_cont.ensure(8 * (size_t)mres.total_contacts), "mesh scratch");
          continue;
        }
        if (rc) return rc;
        break;
      }
      CKB(launch_bp_scatter_hits(g_bs.list.as<int64_t>(), nl, g_bs.m_counts.as<int32_t>(), hit, s), "mesh scatter");
      CKB(launch_bp_inverse_index(g_bs.list.as<int64_t>(), nl, g_bs.mm_index.as<int32_t>(), s), "mesh index");
    }
  }
  // order: per query by object index; scan of the per-slot contact counts
  CKB(g_bs.perm.ensure(8 * t1), "lists");
  CKB(g_bs.ccount.ensure(4 * t1), "lists");
  CKB(g_bs.coff.ensure(8 * (t1 + 1)), "lists");
  CKB(g_bs.scan_tmp.ensure(8 * ((total + 4095) / 4096 + 2)), "scan scratch");
  CKB(launch_bp_sort_segments(nq, off, pairs, g_bs.perm.as<int64_t>(), s), "sort");
  CKB(launch_bp_gather_counts(g_bs.perm.as<int64_t>(), total, hit, g_bs.ccount.as<int32_t>(), s), "counts");
  CKB(launch_exclusive_scan(g_bs.ccount.as<int32_t>(), total, g_bs.coff.as<int64_t>(), g_bs.scan_tmp.as<int64_t>(),
                            s),
      "scan");
  CKB(launch_bp_query_contacts(nq, off, g_bs.coff.as<int64_t>(), res->counts, res->offsets, s), "query counts");
  int64_t nc = 0;
  CKB(cudaMemcpyAsync(&nc, g_bs.coff.as<int64_t>() + total, 8, cudaMemcpyDeviceToHost, s), "read total");
  CKB(cudaMemcpyAsync(&hc, dctr, sizeof(BpCounters), cudaMemcpyDeviceToHost, s), "read counters");
  CKB(cudaStreamSynchronize(s), "broadphase contacts");
  res->total_contacts = nc;
  res->total_node_visits = hc.visits;
  RCB(check_status(hc));
  if (nc > res->capacity) return bp_fail(FCLGPU_ERR_CAPACITY, "contacts buffer too small");
  CKB(launch_bp_fill_contacts(g_bs.perm.as<int64_t>(), total, pairs, g_bs.kind.as<int32_t>(), hit,
                              g_bs.coff.as<int64_t>(), g_bs.mm_index.as<int32_t>(), g_bs.mm_off.as<int64_t>(),
                              g_bs.mm_cont.as<int32_t>(), g_bs.x_index.as<int32_t>(), g_bs.x_loff.as<int64_t>(),
                              g_bs.x_ltris.as<int32_t>(), res->contacts, s),
      "fill");
  CKB(cudaStreamSynchronize(s), "broadphase contacts");
  return FCLGPU_OK;
}

// The scene's own objects as queries (object q against the objects below it).
BpQueryView self_queries(const fclgpu_broadphase_s* bp) {
  BpQueryView Q;
  Q.nq = bp->n;
  Q.gid = bp->gid;
  Q.tf = bp->tf;
  Q.aabb64 = bp->aabb64;
  Q.aabb32 = bp->aabb32;
  Q.self = 1;
  return Q;
}

int check_contacts_args(const fclgpu_broadphase_contacts_request* req, const fclgpu_broadphase_contacts_result* res,
                        int64_t nq) {
  if (!req || !res || !res->offsets || (nq > 0 && !res->counts) || res->capacity < 0 ||
      (res->capacity > 0 && !res->contacts))
    return bp_fail(FCLGPU_ERR_INVALID_ARGUMENT, "missing broadphase contacts argument");
  if (req->num_max_contacts < 1) return bp_fail(FCLGPU_ERR_INVALID_ARGUMENT, "num_max_contacts must be >= 1");
  if (req->precision != FCLGPU_PLAIN_FP64 && req->precision != FCLGPU_FP32_RECHECK)
    return bp_fail(FCLGPU_ERR_INVALID_ARGUMENT, "unknown precision");
  return FCLGPU_OK;
}

// Host form of a contacts call: device outputs staged per call, then copied back.
template <class F>
int contacts_host(int64_t nq, fclgpu_broadphase_contacts_result* res, cudaStream_t s, F&& run_device) {
  Buf c, o, l;
  CKB(c.ensure(8 * (size_t)std::max<int64_t>(nq, 1)), "staging");
  CKB(o.ensure(8 * (size_t)(nq + 1)), "staging");
  CKB(l.ensure(12 * (size_t)std::max<int64_t>(res->capacity, 1)), "staging");
  fclgpu_broadphase_contacts_result dr = {c.as<int64_t>(), o.as<int64_t>(), l.as<int32_t>(), res->capacity, 0, 0, 0};
  int rc = run_device(&dr);
  res->total_contacts = dr.total_contacts;
  res->total_candidates = dr.total_candidates;
  res->total_node_visits = dr.total_node_visits;
  if (rc == FCLGPU_OK || rc == FCLGPU_ERR_CAPACITY) {
    cudaError_t e = cudaSuccess;
    if (nq > 0) e = cudaMemcpyAsync(res->counts, dr.counts, 8 * (size_t)nq, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(res->offsets, dr.offsets, 8 * (size_t)(nq + 1), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess && rc == FCLGPU_OK && dr.total_contacts > 0)
      e = cudaMemcpyAsync(res->contacts, dr.contacts, 12 * (size_t)dr.total_contacts, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) rc = bp_cuda(e, "d2h");
  }
  for (Buf* b : {&c, &o, &l}) cudaFree(b->p);
  return rc;
}

}  // namespace

extern "C" {

int fclgpu_broadphase_collide_contacts_device(fclgpu_broadphase bp, const fclgpu_geometry_ref* queries, int64_t nq,
                                              const double* tf, const fclgpu_broadphase_contacts_request* req,
                                              fclgpu_broadphase_contacts_result* res, void* stream) {
  if (!bp || nq < 0 || (nq > 0 && (!queries || !tf)))
    return bp_fail(FCLGPU_ERR_INVALID_ARGUMENT, "missing broadphase contacts argument");
  RCB(check_contacts_args(req, res, nq));
  if (nq >= ((int64_t)1 << 31)) return bp_fail(FCLGPU_ERR_INVALID_ARGUMENT, "too many queries");
  std::lock_guard<std::mutex> lk(g_bp_mu);
  cudaStream_t s = (cudaStream_t)stream;
  res->total_contacts = res->total_candidates = res->total_node_visits = 0;
  CKB(g_bs.ctr.ensure(sizeof(BpCounters)), "counters");
  BpCounters* dctr = g_bs.ctr.as<BpCounters>();
  CKB(cudaMemsetAsync(dctr, 0, sizeof(BpCounters), s), "counters");
  if (nq == 0) {
    CKB(cudaMemsetAsync(res->offsets, 0, 8, s), "offsets");
    CKB(cudaStreamSynchronize(s), "offsets");
    return FCLGPU_OK;
  }
  BpQueryView Q;
  RCB(prepare_queries(bp, queries, nq, tf, Q, dctr, s));
  return contacts_core(bp, Q, req, res, dctr, s);
}

int fclgpu_broadphase_collide_contacts(fclgpu_broadphase bp, const fclgpu_geometry_ref* queries, int64_t nq,
                                       const double* tf, const fclgpu_broadphase_contacts_request* req,
                                       fclgpu_broadphase_contacts_result* res, void* stream) {
  if (!bp || nq < 0 || (nq > 0 && (!queries || !tf)))
    return bp_fail(FCLGPU_ERR_INVALID_ARGUMENT, "missing broadphase contacts argument");
  RCB(check_contacts_args(req, res, nq));
  cudaStream_t s = (cudaStream_t)stream;
  // inputs to the device (the device entry point takes the lock)
  void* dq = nullptr;
  void* dt = nullptr;
  if (nq > 0) {
    CKB(cudaMalloc(&dq, 8 * (size_t)nq), "staging");
    cudaError_t e = cudaMalloc(&dt, 96 * (size_t)nq);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dq, queries, 8 * (size_t)nq, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dt, tf, 96 * (size_t)nq, cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) {
      cudaFree(dq);
      if (dt) cudaFree(dt);
      return bp_cuda(e, "staging");
    }
  }
  const int rc = contacts_host(nq, res, s, [&](fclgpu_broadphase_contacts_result* dr) {
    return fclgpu_broadphase_collide_contacts_device(bp, (const fclgpu_geometry_ref*)dq, nq, (const double*)dt, req,
                                                     dr, stream);
  });
  if (dq) cudaFree(dq);
  if (dt) cudaFree(dt);
  return rc;
}

int fclgpu_broadphase_self_collide_contacts_device(fclgpu_broadphase bp,
                                                   const fclgpu_broadphase_contacts_request* req,
                                                   fclgpu_broadphase_contacts_result* res, void* stream) {
  if (!bp) return bp_fail(FCLGPU_ERR_INVALID_ARGUMENT, "missing broadphase");
  RCB(check_contacts_args(req, res, bp->n));
  std::lock_guard<std::mutex> lk(g_bp_mu);
  cudaStream_t s = (cudaStream_t)stream;
  res->total_contacts = res->total_candidates = res->total_node_visits = 0;
  CKB(g_bs.ctr.ensure(sizeof(BpCounters)), "counters");
  BpCounters* dctr = g_bs.ctr.as<BpCounters>();
  CKB(cudaMemsetAsync(dctr, 0, sizeof(BpCounters), s), "counters");
  if (bp->n == 0) {
    CKB(cudaMemsetAsync(res->offsets, 0, 8, s), "offsets");
    CKB(cudaStreamSynchronize(s), "offsets");
    return FCLGPU_OK;
  }
  const BpQueryView Q = self_queries(bp);
  return contacts_core(bp, Q, req, res, dctr, s);
}

int fclgpu_broadphase_self_collide_contacts(fclgpu_broadphase bp, const fclgpu_broadphase_contacts_request* req,
                                            fclgpu_broadphase_contacts_result* res, void* stream) {
  if (!bp) return bp_fail(FCLGPU_ERR_INVALID_ARGUMENT, "missing broadphase");
  RCB(check_contacts_args(req, res, bp->n));
  return contacts_host(bp->n, res, (cudaStream_t)stream, [&](fclgpu_broadphase_contacts_result* dr) {
    return fclgpu_broadphase_self_collide_contacts_device(bp, req, dr, stream);
  });
}

int fclgpu_broadphase_self_distance(fclgpu_broadphase bp, const fclgpu_broadphase_distance_request* req,
                                    fclgpu_broadphase_self_distance_result* out, void* stream) {
  if (!bp || !req || !out) return bp_fail(FCLGPU_ERR_INVALID_ARGUMENT, "missing broadphase self-distance argument");
  if (req->precision != FCLGPU_PLAIN_FP64 && req->precision != FCLGPU_FP32_RECHECK)
    return bp_fail(FCLGPU_ERR_INVALID_ARGUMENT, "unknown precision");
  out->min_distance = std::numeric_limits<double>::max();
  out->o1 = out->o2 = out->b1 = out->b2 = -1;
  for (double& p : out->nearest_points) p = 0.0;
  out->total_candidates = 0;
  const int64_t n = bp->n;
  if (n < 2) return FCLGPU_OK;
  cudaStream_t s = (cudaStream_t)stream;
  Buf d, o, ids, pts;  // per-object results (object q against the objects below it)
  CKB(d.ensure(8 * n), "staging");
  CKB(o.ensure(4 * n), "staging");
  CKB(ids.ensure(8 * n), "staging");
  CKB(pts.ensure(48 * n), "staging");
  fclgpu_broadphase_distance_result dr = {d.as<double>(), o.as<int32_t>(), ids.as<int32_t>(), pts.as<double>(), 0, 0};
  int rc;
  {
    std::lock_guard<std::mutex> lk(g_bp_mu);
    PhaseClock pc(1, s);
    g_last_mixed = 0;
    rc = g_bs.ctr.ensure(sizeof(BpCounters)) == cudaSuccess ? FCLGPU_OK : FCLGPU_ERR_OUT_OF_MEMORY;
    if (rc == FCLGPU_OK) {
      BpCounters* dctr = g_bs.ctr.as<BpCounters>();
      const cudaError_t e = cudaMemsetAsync(dctr, 0, sizeof(BpCounters), s);
      rc = e == cudaSuccess ? distance_core(bp, self_queries(bp), req, &dr, dctr, s, pc) : bp_cuda(e, "counters");
    }
  }
  if (rc == FCLGPU_OK) {
    std::vector<double> hd(n), hp(6 * n);
    std::vector<int32_t> ho(n), hi(2 * n);
    cudaError_t e = cudaMemcpyAsync(hd.data(), d.p, 8 * n, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(ho.data(), o.p, 4 * n, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(hi.data(), ids.p, 8 * n, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(hp.data(), pts.p, 48 * n, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
      rc = bp_cuda(e, "d2h");
    } else {
      // the smallest distance over all pairs; ties to the smaller o2, then o1
      int64_t best = -1;
      for (int64_t q = 1; q < n; ++q)
        if (ho[q] >= 0 && (best < 0 || hd[q] < hd[best])) best = q;
      out->total_candidates = dr.total_candidates;
      if (best >= 0) {
        out->min_distance = hd[best];
        out->o1 = ho[best];
        out->o2 = (int32_t)best;
        out->b1 = hi[2 * best];
        out->b2 = hi[2 * best + 1];
        for (int k = 0; k < 6; ++k) out->nearest_points[k] = req->enable_nearest_points ? hp[6 * best + k] : 0.0;
      }
    }
  }
  for (Buf* b : {&d, &o, &ids, &pts}) cudaFree(b->p);
  return rc;
}

int fclgpu_broadphase_last_phase_ms(double* out16) {
  if (!out16) return FCLGPU_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lk(g_bp_mu);
  for (int r = 0; r < 2; ++r)
    for (int k = 0; k < 8; ++k) {
      out16[8 * r + k] = g_phase[r][k];
      g_phase[r][k] = 0.0;
    }
  return FCLGPU_OK;
}

}  // extern "C"
