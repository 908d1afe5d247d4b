// Batched BVHModel<OBBRSS> x convex shape collide / distance (one pair per thread) and
// its C ABI (fclgpu_mesh_shape_batch*).
#include <cuda_runtime.h>
#include <math_constants.h>

#include <algorithm>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/fclgpu.h"
#include "kernels.h"
#include "mesh_handle.h"
#include "mesh_shape.cuh"
#include "mesh_shape.h"
#include "shapeset_handle.h"

namespace fclgpu {
namespace {

template <int STACK>
__global__ void __launch_bounds__(128) k_mesh_shape(MeshShapeLaunch L) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < L.n; i += stride) {
    const DevMesh m = L.meshes[L.mesh_idx[i]];
    ShapeRef A;
    A.s = L.shapes[L.shape_idx[i]];
    A.verts = L.sverts;
    M3<double> Rm, Rs;
    D3v tm, ts;
    load_tf(L.tfm + 12 * i, Rm, tm);
    load_tf(L.tfs + 12 * i, Rs, ts);
    MeshShapeOut o;
    o.count = 0;
    o.tri = -1;
    o.dist = 0;
    o.pmesh = o.pshape = v3(0.0, 0.0, 0.0);
    o.nbv = o.nleaf = 0;
    o.status = 0;
    if (L.mode == 0) {
      mesh_shape_collide<STACK>(m, Rm, tm, A, Rs, ts, L.max_contacts, o);
      L.counts[i] = o.count;
    } else {
      mesh_shape_distance<STACK>(m, Rm, tm, A, Rs, ts, o);
      L.dist[i] = o.dist;
      if (L.tri) L.tri[i] = o.tri;
      if (L.pts) {
        double* p = L.pts + 6 * i;
        p[0] = o.pmesh.x;
        p[1] = o.pmesh.y;
        p[2] = o.pmesh.z;
        p[3] = o.pshape.x;
        p[4] = o.pshape.y;
        p[5] = o.pshape.z;
      }
    }
    if (L.nbv) L.nbv[i] = o.nbv;
    if (L.nleaf) L.nleaf[i] = o.nleaf;
    if (o.status) atomicOr(L.status, 1u);
  }
}

// ------------------------------------------------------------------ split form ----

struct PairGeom {
  DevMesh m;
  ShapeRef A;
  M3<double> Rm, Rs;
  D3v tm, ts;
};

__device__ __forceinline__ void pair_geom(const MeshShapeLaunch& L, long long i, PairGeom& g) {
  g.m = L.meshes[L.mesh_idx[i]];
  g.A.s = L.shapes[L.shape_idx[i]];
  g.A.verts = L.sverts;
  load_tf(L.tfm + 12 * i, g.Rm, g.tm);
  load_tf(L.tfs + 12 * i, g.Rs, g.ts);
}

// distance: leaves of each pair that may hold the minimum, count pass (offsets == null)
// or write pass
template <int STACK>
__global__ void __launch_bounds__(128) k_ms_collect(MeshShapeLaunch L, int32_t* counts, const int64_t* offsets,
                                                    int32_t* leaf_pair, int32_t* leaf_prim, double* leaf_lb,
                                                    double* ub) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < L.n; i += stride) {
    PairGeom g;
    pair_geom(L, i, g);
    ShapeBV bv;
    if (L.bv_src)
      bv = static_cast<const ShapeBV*>(L.bv_table)[L.bv_src[i]];
    else
      shape_obbrss(g.A.s, g.A.verts, g.Rs, g.ts, bv);
    const long long base = offsets ? offsets[i] : 0;
    int cnt = 0;
    auto emit = [&](int prim, double lb) {
      if (offsets) {
        leaf_pair[base + cnt] = (int32_t)i;
        leaf_prim[base + cnt] = prim;
        if (leaf_lb) leaf_lb[base + cnt] = lb;
      }
      ++cnt;
    };
    double u = DBL_MAX;
    const int st = mesh_shape_collect_distance<STACK>(g.m, g.Rm, g.tm, g.A, g.Rs, g.ts, bv, &u, emit);
    if (ub) ub[i] = u;
    if (st) atomicOr(L.status, 1u);
    if (counts) counts[i] = cnt;
  }
}

__global__ void __launch_bounds__(128) k_ms_leaf_tests(MeshShapeLaunch L, long long nl, const int32_t* leaf_pair,
                                                       const int32_t* leaf_prim, const double* leaf_lb,
                                                       const double* ub, double* dist, double* pts) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x; j < nl; j += stride) {
    const long long i = leaf_pair[j];
    if (leaf_lb[j] > ub[i]) {  // cannot hold the minimum
      dist[j] = DBL_MAX;
      continue;
    }
    PairGeom g;
    pair_geom(L, i, g);
    double P[9];
    load_tri_local(g.m, leaf_prim[j], P);
    SimplexVert V[kSimplexSlots];
    double d;
    D3v ps, pt;
    shape_triangle_distance(g.A, g.Rs, g.ts, P, g.Rm, g.tm, V, d, ps, pt);
    dist[j] = d;
    double* p = pts + 6 * j;
    p[0] = pt.x;
    p[1] = pt.y;
    p[2] = pt.z;
    p[3] = ps.x;
    p[4] = ps.y;
    p[5] = ps.z;
  }
}

// per pair: distance = the first minimum in collection order (the seed triangle first,
// as FCL's strict update)
__global__ void k_ms_reduce(MeshShapeLaunch L, const int64_t* off, const int32_t* leaf_prim, const double* dist,
                            const double* pts) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < L.n; i += stride) {
    double best = DBL_MAX;
    long long bj = -1;
    for (long long j = off[i]; j < off[i + 1]; ++j)
      if (best > dist[j]) {
        best = dist[j];
        bj = j;
      }
    L.dist[i] = best;
    if (L.tri) L.tri[i] = bj >= 0 ? leaf_prim[bj] : -1;
    if (L.pts)
      for (int k = 0; k < 6; ++k) L.pts[6 * i + k] = bj >= 0 ? pts[6 * bj + k] : 0.0;
  }
}

// Collide in rounds.  Each unfinished pair resumes its DFS (stack kept in global
// memory) until it has K_r more overlapping leaves or has tested 128 * 2^min(r, 3)
// nodes this round; stage 1 of the leaf test runs one
// leaf per thread (sphere closed form, FP32 GJK with the FP64 disjointness
// certificate), then one thread per pair walks its leaves in DFS order, running the
// FP64 GJK on undecided leaves, and stops once it has max_contacts intersecting leaves
// -- FCL's early stop (the rest of the DFS is not visited either).  K_r = 16 * 2^r (at most 1024): colliding pairs usually
// stop in the first round, long contact-free traversals need few rounds.
struct MsPairState {
  ShapeBV bv;
  ShapeBV32 b32;
};

__global__ void __launch_bounds__(128) k_msr_init(MeshShapeLaunch L, MsPairState* ps, int32_t* stack, int cap,
                                                  int32_t* sp, int32_t* act) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < L.n; i += stride) {
    PairGeom g;
    pair_geom(L, i, g);
    MsPairState st;
    if (L.bv_src)
      st.bv = static_cast<const ShapeBV*>(L.bv_table)[L.bv_src[i]];
    else
      shape_obbrss(g.A.s, g.A.verts, g.Rs, g.ts, st.bv);
    make_shape_bv32(g.Rm, g.tm, st.bv, g.m, st.b32);
    ps[i] = st;
    stack[i * (long long)cap] = 0;
    sp[i] = 1;
    L.counts[i] = 0;
    act[i] = (int32_t)i;
  }
}

__global__ void __launch_bounds__(128) k_msr_dfs(MeshShapeLaunch L, const int32_t* act, long long nact, int K,
                                                 int max_visits, const MsPairState* ps, int32_t* stack, int cap,
                                                 int32_t* sp, int32_t* leaf, int32_t* nleaf) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long a = (long long)blockIdx.x * blockDim.x + threadIdx.x; a < nact; a += stride) {
    const long long i = act[a];
    if (L.group && L.group_count[L.group[i]] >= (unsigned long long)L.group_max) {  // the query has its contacts
      sp[i] = 0;
      nleaf[a] = 0;
      continue;
    }
    const DevMesh m = L.meshes[L.mesh_idx[i]];
    M3<double> Rm;
    D3v tm;
    load_tf(L.tfm + 12 * i, Rm, tm);
    const ShapeBV bv = ps[i].bv;
    const ShapeBV32 b32 = ps[i].b32;
    int s = sp[i];
    int32_t* out = leaf + a * (long long)K;
    const int ne = mesh_shape_dfs_resume(m, Rm, tm, bv, b32, stack + i * (long long)cap, s, cap, K, max_visits,
                                         [&](int k, int prim) { out[k] = prim; });
    if (ne < 0) {
      atomicOr(L.status, 1u);
      sp[i] = 0;
      nleaf[a] = 0;
    } else {
      sp[i] = s;
      nleaf[a] = ne;
    }
  }
}

__global__ void __launch_bounds__(128) k_msr_tests(MeshShapeLaunch L, const int32_t* act, long long nact, int K,
                                                   const int32_t* leaf, const int32_t* nleaf, int32_t* hit) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < nact * K; t += stride) {
    const long long a = t / K;
    if (t % K >= nleaf[a]) continue;
    PairGeom g;
    pair_geom(L, act[a], g);
    double P[9];
    load_tri_local(g.m, leaf[t], P);
    hit[t] = shape_triangle_stage1(g.A, g.Rs, g.ts, P, g.Rm, g.tm);
  }
}

// Walks a pair's leaves in DFS order and counts intersections until it has max_contacts:
// stage-1 hits count at once, undecided leaves run the FP64 GJK in this thread -- at
// most kSerialGjk of them; the pair's further undecided leaves are deferred to one
// thread each (k_msr_deferred) and the pair is recounted after them (k_msr_recount).
// The count is min(max_contacts, intersecting leaves) either way.  The serial part would
// keep the early stop for a pair whose first undecided leaf intersects, but one FP64 GJK
// per thread leaves most lanes of a warp idle at GB300's FP64 rate; deferring every
// undecided leaf (one full warp of GJKs at a time) measured faster on the motion-checking
// server (256-request burst 2,099 -> 2,405 requests/s, 16-request burst's mesh-shape
// phase 71 -> 56 ms for budgets 4 -> 0), so the budget is 0.
constexpr int kSerialGjk = 0;

// Lists the pair's contacts c0..c-1: its first intersecting leaves of this round in
// DFS order, as (pair, rank, triangle) records.
__device__ __forceinline__ void emit_contacts(const MeshShapeLaunch& L, long long i, long long a, int K,
                                              const int32_t* leaf, const int32_t* nleaf, const int32_t* hit, int c0,
                                              int c) {
  if (!L.rec || c <= c0) return;
  int r = c0;
  const int nl = nleaf[a];
  for (int k = 0; k < nl && r < c; ++k) {
    const long long slot = a * (long long)K + k;
    if (hit[slot] == 2) {
      L.rec[atomicAdd(L.nrec, 1ull)] = make_int4((int)i, r, leaf[slot], 0);
      ++r;
    }
  }
}

// adds a pair's new contacts to its group; false once the group has group_max (the
// pair's query needs no more contacts, so its traversal can stop)
__device__ __forceinline__ bool group_open(const MeshShapeLaunch& L, long long i, int delta) {
  if (!L.group) return true;
  const unsigned long long t = (delta > 0 ? atomicAdd(&L.group_count[L.group[i]], (unsigned long long)delta)
                                          : L.group_count[L.group[i]]) +
                               (unsigned long long)delta;
  return t < (unsigned long long)L.group_max;
}

__global__ void __launch_bounds__(128) k_msr_update(MeshShapeLaunch L, const int32_t* act, long long nact, int K,
                                                    const int32_t* leaf, const int32_t* nleaf, int32_t* hit,
                                                    const int32_t* sp, int32_t* next, unsigned long long* nnext,
                                                    int32_t* defer_leaf, unsigned long long* ndefer,
                                                    int32_t* defer_pair, unsigned long long* ndefer_pair) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long a = (long long)blockIdx.x * blockDim.x + threadIdx.x; a < nact; a += stride) {
    const long long i = act[a];
    int c = L.counts[i];
    const int nl = nleaf[a];
    int budget = kSerialGjk;
    bool deferred = false;
    for (int k = 0; k < nl && c < L.max_contacts; ++k) {
      const long long slot = a * (long long)K + k;
      const int h = hit[slot];
      if (h == 2) {
        ++c;
      } else if (h == 1) {
        if (budget > 0) {
          --budget;
          PairGeom g;
          pair_geom(L, i, g);
          double P[9];
          load_tri_local(g.m, leaf[slot], P);
          SimplexVert V[kSimplexSlots];
          const bool in = shape_triangle_gjk64(g.A, g.Rs, g.ts, P, g.Rm, g.tm, V);
          hit[slot] = in ? 2 : 0;
          if (in) ++c;
        } else {
          defer_leaf[atomicAdd(ndefer, 1ull)] = (int32_t)slot;
          deferred = true;
        }
      }
    }
    if (deferred) {
      defer_pair[atomicAdd(ndefer_pair, 1ull)] = (int32_t)a;
      continue;
    }
    const int c0 = L.counts[i];
    L.counts[i] = c;
    emit_contacts(L, i, a, K, leaf, nleaf, hit, c0, c);
    if (c < L.max_contacts && sp[i] > 0 && group_open(L, i, c - c0)) next[atomicAdd(nnext, 1ull)] = (int32_t)i;
  }
}

__global__ void __launch_bounds__(128) k_msr_deferred(MeshShapeLaunch L, const int32_t* act, int K,
                                                      const int32_t* leaf, int32_t* hit, const int32_t* defer_leaf,
                                                      const unsigned long long* ndefer) {
  const long long n = (long long)*ndefer;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += stride) {
    const long long slot = defer_leaf[t];
    PairGeom g;
    pair_geom(L, act[slot / K], g);
    double P[9];
    load_tri_local(g.m, leaf[slot], P);
    SimplexVert V[kSimplexSlots];
    hit[slot] = shape_triangle_gjk64(g.A, g.Rs, g.ts, P, g.Rm, g.tm, V) ? 2 : 0;
  }
}

__global__ void __launch_bounds__(128) k_msr_recount(MeshShapeLaunch L, const int32_t* act, int K,
                                                     const int32_t* leaf, const int32_t* nleaf, const int32_t* hit,
                                                     const int32_t* sp, const int32_t* defer_pair,
                                                     const unsigned long long* ndefer_pair, int32_t* next,
                                                     unsigned long long* nnext) {
  const long long n = (long long)*ndefer_pair;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += stride) {
    const long long a = defer_pair[t];
    const long long i = act[a];
    int c = L.counts[i];
    const int nl = nleaf[a];
    for (int k = 0; k < nl && c < L.max_contacts; ++k) c += hit[a * (long long)K + k] == 2 ? 1 : 0;
    const int c0 = L.counts[i];
    L.counts[i] = c;
    emit_contacts(L, i, a, K, leaf, nleaf, hit, c0, c);
    if (c < L.max_contacts && sp[i] > 0 && group_open(L, i, c - c0)) next[atomicAdd(nnext, 1ull)] = (int32_t)i;
  }
}

// Collide counts without a contact list: FCL's count is min(max_contacts, intersecting
// leaves), whatever order the leaves are met in, so one warp works a pair, testing up to
// 32 of its frontier nodes (a LIFO stack in shared memory) and leaves at a time, and stops
// at max_contacts or once the pair's group is full.  With pops of 32 and pushes of at most
// 64 per step the stack stays below 32 (depth + 2) entries.
constexpr int kMsWarps = 4;
constexpr int kMsFront = 2048;
constexpr int kMsWarpMaxDepth = kMsFront / 32 - 4;
// (register caps of 168 and 128 for more resident warps were measured slower: spills)

__global__ void __launch_bounds__(32 * kMsWarps) k_ms_count_warp(MeshShapeLaunch L) {
  __shared__ int32_t front[kMsWarps][kMsFront];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const long long i = (long long)blockIdx.x * kMsWarps + w;
  if (i >= L.n) return;
  const unsigned full = 0xffffffffu;
  const unsigned lt = (1u << lane) - 1u;
  PairGeom g;
  pair_geom(L, i, g);
  ShapeBV bv;
  if (L.bv_src)
    bv = static_cast<const ShapeBV*>(L.bv_table)[L.bv_src[i]];
  else
    shape_obbrss(g.A.s, g.A.verts, g.Rs, g.ts, bv);
  ShapeBV32 b32;
  make_shape_bv32(g.Rm, g.tm, bv, g.m, b32);
  LeafCert32 cert;
  if (g.A.s.type != SHAPE_SPHERE) leaf_cert_init(g.A, g.Rs, g.ts, g.Rm, g.tm, cert);
  const int M = L.max_contacts;
  if (lane == 0) front[w][0] = 0;
  int size = 1, count = 0;
  __syncwarp();
  while (size > 0 && count < M) {
    if (L.group) {
      unsigned long long gc = 0;
      if (lane == 0) gc = *(volatile unsigned long long*)&L.group_count[L.group[i]];
      gc = __shfl_sync(full, gc, 0);
      if (gc >= (unsigned long long)L.group_max) break;  // the query has its contacts
    }
    const int take = size < 32 ? size : 32;
    const int b = lane < take ? front[w][size - 1 - lane] : -1;
    size -= take;
    __syncwarp();
    bool ov = false;
    int child = 0;
    if (b >= 0) ov = shape_node_overlap(g.m, g.Rm, g.tm, bv, b32, b, &child);
    const bool inner = ov && child >= 0;
    const unsigned pm = __ballot_sync(full, inner);
    if (size + 2 * __popc(pm) > kMsFront) {  // not reached for trees within kMsWarpMaxDepth
      if (lane == 0) atomicOr(L.status, 1u);  // reported as a stack overflow
      break;
    }
    if (inner) {
      const int pos = size + 2 * __popc(pm & lt);
      front[w][pos] = child + 1;
      front[w][pos + 1] = child;
    }
    size += 2 * __popc(pm);
    bool hit = false;
    if (ov && child < 0) {
      double P[9];
      load_tri_local(g.m, -(child + 1), P);
      int h = shape_triangle_stage1(cert, g.A, g.ts, P, g.Rm, g.tm);
      if (h == 1) {
        SimplexVert V[kSimplexSlots];
        if (L.group)  // a long GJK gives up once the query has its contacts from other pairs
          h = shape_triangle_gjk64_until(g.A, g.Rs, g.ts, P, g.Rm, g.tm, V, [&] {
                return *(volatile unsigned long long*)&L.group_count[L.group[i]] >=
                       (unsigned long long)L.group_max;
              })
                  ? 2
                  : 0;
        else
          h = shape_triangle_gjk64(g.A, g.Rs, g.ts, P, g.Rm, g.tm, V) ? 2 : 0;
      }
      hit = h == 2;
    }
    const int nh = __popc(__ballot_sync(full, hit));
    if (nh) {
      count += nh;
      if (L.group && lane == 0) atomicAdd(&L.group_count[L.group[i]], (unsigned long long)nh);
    }
    __syncwarp();
  }
  if (lane == 0) L.counts[i] = count < M ? count : M;
}

// Mesh-shape distance, one warp per pair.  FCL's traversal (distanceRecurse with
// triangle 0 as the seed, mesh_shape_distance_traversal_node-inl.h) reports the first
// leaf in its visit order with the smallest distance it meets, and prunes a subtree
// whose bound is at least its running minimum; so its distance is the minimum over the
// mesh's triangles (up to a triangle whose FP64 distance falls below its node's FP64
// bound by rounding), and its triangle is the first of the triangles at that minimum
// in its depth-first order, whatever order they are found in here.
//
// The warp keeps a stack of (node, bound, path) in shared memory and takes up to 32
// entries a step; the children it adds are sorted by bound (a bitonic network over the
// warp) and pushed nearest on top, so the nearest leaves come first.  Bounds are FP32
// lower bounds with a derived error (below): a node is dropped, and a leaf's FP64
// distance skipped, only when its bound exceeds the running minimum by more than
// m64 = 2^-36 S (S the pair's coordinate scale), which covers FCL's FP64 volumes
// containing their triangles up to rounding and its FP64 distances being within
// rounding of the exact ones.  So every triangle whose FP64 distance can reach the
// minimum -- including every triangle tied at it -- is evaluated with FCL's FP64
// shapeTriangleDistance.  Of tied triangles the first in FCL's order wins: triangle 0
// (the seed) first, otherwise the one on the side FCL enters first at the two leaves'
// deepest common node (FCL's FP64 bounds of that node's children, the nearer first,
// the second child on d2 < d1).  A triangle at distance <= 0 (touching or
// intersecting, where FCL's first-met rule decides the value) switches the pair to the
// search described below the main loop; a pair whose mesh was refitted (FCL's merged
// volumes then need not bound their triangles), or where that search's conditions
// fail, is handed to k_ms_dist_serial, which runs FCL's own traversal.
//
// Node bounds: md_node_bound (mesh_shape.cuh, with its error derivation), along two
// directions: from the RSS rectangle's point nearest to the shape's origin to that
// origin, and the separating direction of the best triangle so far (its FP32 GJK
// direction).  Leaf bound: leaf_cert_lb (gjk32.cuh): FP32 GJK on (shape, triangle) to
// convergence, then the support gap along its direction (under 40u ||D||_1 S of error;
// 64u is subtracted).
constexpr int kMdWarps = 2;
constexpr int kMdFront = 1024;
constexpr int kMdWarpMaxDepth = kMdFront / 32 - 4;

// one compare-exchange network sorting 64 entries held two per lane (entry e = lane +
// 32 * slot) by (key, node), ascending; pay travels with its entry
template <class K>
__device__ __forceinline__ bool md_less(K ka, int na, K kb, int nb) {
  return ka < kb || (ka == kb && na < nb);
}
template <class K>
__device__ __forceinline__ void md_sort64(K& k0, int& n0, unsigned& p0, K& k1, int& n1, unsigned& p1, int lane) {
  const unsigned full = 0xffffffffu;
#pragma unroll
  for (int k = 2; k <= 64; k <<= 1) {
#pragma unroll
    for (int j = k >> 1; j > 0; j >>= 1) {
      if (j == 32) {  // partner in the other slot of the same lane (k == 64: ascending)
        if (md_less(k1, n1, k0, n0)) {
          const K tk = k0;
          const int tn = n0;
          const unsigned tp = p0;
          k0 = k1;
          n0 = n1;
          p0 = p1;
          k1 = tk;
          n1 = tn;
          p1 = tp;
        }
        continue;
      }
#pragma unroll
      for (int slot = 0; slot < 2; ++slot) {
        K& kk = slot ? k1 : k0;
        int& nn = slot ? n1 : n0;
        unsigned& pp = slot ? p1 : p0;
        const int e = lane + 32 * slot;
        const K pk = __shfl_xor_sync(full, kk, j);
        const int pn = __shfl_xor_sync(full, nn, j);
        const unsigned ppay = __shfl_xor_sync(full, pp, j);
        const bool up = (e & k) == 0;
        const bool lower = (e & j) == 0;
        const bool p_first = md_less(pk, pn, kk, nn);  // the partner orders before this entry
        // the lower position keeps the first of the two in the sort direction
        const bool take = lower ? (up ? p_first : !p_first) : (up ? !p_first : p_first);
        if (take) {
          kk = pk;
          nn = pn;
          pp = ppay;
        }
      }
    }
  }
}

// path of a node below the root: one bit per level from bit 31 down (0 = first child,
// 1 = second), then a marker bit
__device__ __forceinline__ unsigned md_child_path(unsigned path, int which) {
  const int m = __ffs(path) - 1;
  return (path & ~(1u << m)) | ((unsigned)which << m) | (1u << (m - 1));
}

template <bool WIT>
__global__ void __launch_bounds__(32 * kMdWarps) k_ms_dist_warp(MeshShapeLaunch L) {
  __shared__ int32_t fnode[kMdWarps][kMdFront];
  __shared__ float flb[kMdWarps][kMdFront];
  __shared__ unsigned fpath[kMdWarps][kMdFront];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const long long i = (long long)blockIdx.x * kMdWarps + w;
  if (i >= L.n) return;
  const unsigned full = 0xffffffffu;
  PairGeom g;
  pair_geom(L, i, g);
  if (g.m.refitted) {  // FCL's traversal order decides: k_ms_dist_serial
    if (lane == 0) L.dist[i] = CUDART_NAN;
    return;
  }
  const float4* rss32 = static_cast<const float4*>(g.m.rss32);
  MdPair q;
  md_pair(g.m, g.A, g.Rm, g.tm, g.Rs, g.ts, q);
  const bool sphere = g.A.s.type == SHAPE_SPHERE;
  LeafCert32 cert;
  if (!sphere) leaf_cert_init(g.A, g.Rs, g.ts, g.Rm, g.tm, cert);
  const double m64 = ldexp(1.0 + (double)q.rho + fmax(fabs(g.ts.x), fmax(fabs(g.ts.y), fabs(g.ts.z))) +
                               fmax(fabs(g.tm.x), fmax(fabs(g.tm.y), fabs(g.tm.z))) + g.m.vmax + g.m.rmax,
                           -36);
  ShapeBV bv;  // FCL's model2_bv, for its FP64 bounds when two triangles tie
  if (L.bv_src)
    bv = static_cast<const ShapeBV*>(L.bv_table)[L.bv_src[i]];
  else
    shape_obbrss(g.A.s, g.A.verts, g.Rs, g.ts, bv);
  auto bvd = [&](int b) {  // as mesh_shape_distance's node bound
    const RssD& rs = g.m.rss64[b];
    M3<double> A2, Ab;
    for (int k = 0; k < 9; ++k) {
      A2.m[k] = rs.axis[k];
      Ab.m[k] = bv.obb.axis[k];
    }
    return rss_distance<double>(g.Rm, g.tm, Ab, v3(bv.rTo[0], bv.rTo[1], bv.rTo[2]), bv.rl, bv.rr, A2,
                                v3(rs.To[0], rs.To[1], rs.To[2]), rs.l, rs.r);
  };
  // true when leaf (pa, ka) comes before leaf (pb_, kb) in FCL's order
  auto fcl_first = [&](int prim_a, unsigned ka, int prim_b, unsigned kb) {
    if (prim_a == 0) return true;
    if (prim_b == 0) return false;
    const int lca = __clz(ka ^ kb);
    int x = 0;
    for (int t = 0; t < lca; ++t) x = g.m.nodes64[x].child + (int)((ka >> (31 - t)) & 1u);
    const int c = g.m.nodes64[x].child;
    const double d1 = bvd(c), d2 = bvd(c + 1);
    const bool a_second = ((ka >> (31 - lca)) & 1u) != 0;
    return a_second == (d2 < d1);
  };
  double ub = DBL_MAX;
  int best = -1;
  unsigned best_path = 0;
  bool have_dir = false;
  G3f dir = g3f(0.f, 0.f, 0.f);
  bool serial = false;
  if (lane == 0) {
    fnode[w][0] = 0;
    flb[w][0] = -CUDART_INF_F;
    fpath[w][0] = 0x80000000u;
  }
  int size = 1;
  __syncwarp();
  while (size > 0) {
    const int take = size < 32 ? size : 32;
    int b = -1;
    float lb = 0.f;
    unsigned path = 0;
    if (lane < take) {
      b = fnode[w][size - 1 - lane];
      lb = flb[w][size - 1 - lane];
      path = fpath[w][size - 1 - lane];
    }
    size -= take;
    __syncwarp();
    if (b >= 0 && (double)lb > ub + m64) b = -1;  // no triangle below can reach the minimum
    int child = 0;
    if (b >= 0) child = g.m.nodes64[b].child;
    const bool inner = b >= 0 && child >= 0;
    float k0 = CUDART_INF_F, k1 = CUDART_INF_F;  // the children to push (sorted below); infinity = none
    int n0 = -1, n1 = -1;
    unsigned p0 = 0, p1 = 0;
    if (inner) {
      const float l1 = md_node_bound(rss32, child, g.A, q, have_dir, dir);
      const float l2 = md_node_bound(rss32, child + 1, g.A, q, have_dir, dir);
      if ((double)l1 <= ub + m64) {
        k0 = l1;
        n0 = child;
        p0 = md_child_path(path, 0);
      }
      if ((double)l2 <= ub + m64) {
        k1 = l2;
        n1 = child + 1;
        p1 = md_child_path(path, 1);
      }
    }
    double d = DBL_MAX;
    bool has_dir = false;
    G3f ldir = g3f(0.f, 0.f, 0.f);
    if (b >= 0 && child < 0) {
      double P[9];
      load_tri_local(g.m, -(child + 1), P);
      bool eval = true;
      if (!sphere) {
        const float lbl = leaf_cert_lb(cert, P, ldir);
        has_dir = lbl > -CUDART_INF_F;
        eval = !((double)lbl > ub + m64);
      }
      if (eval) {
        SimplexVert V[kSimplexSlots];
        D3v ps, pt;
        shape_triangle_distance(g.A, g.Rs, g.ts, P, g.Rm, g.tm, V, d, ps, pt);
        if (!(d > 0.0)) serial = true;
      }
    }
    if (__any_sync(full, serial)) {
      serial = true;
      break;
    }
    // the step's smallest distance; of equal ones FCL's first
    double dm = d;
    for (int off = 16; off > 0; off >>= 1) dm = fmin(dm, __shfl_xor_sync(full, dm, off));
    if (dm < DBL_MAX && dm <= ub) {
      unsigned at = __ballot_sync(full, d == dm);
      const int prim = -(child + 1);
      int win = -1;
      if (dm < ub) {
        win = __ffs(at) - 1;
        at &= at - 1;
        best = __shfl_sync(full, prim, win);
        best_path = __shfl_sync(full, path, win);
        ub = dm;
      }
      if (WIT) {
        while (at) {  // ties: keep the first in FCL's order
          const int l = __ffs(at) - 1;
          at &= at - 1;
          const int pl = __shfl_sync(full, prim, l);
          const unsigned kl = __shfl_sync(full, path, l);
          if (fcl_first(pl, kl, best, best_path)) {
            best = pl;
            best_path = kl;
            win = l;
          }
        }
      }
      if (win >= 0) {  // the separating direction of the new best, for the node bounds
        const bool hd = __shfl_sync(full, has_dir, win);
        const float dx = __shfl_sync(full, ldir.x, win), dy = __shfl_sync(full, ldir.y, win),
                    dz = __shfl_sync(full, ldir.z, win);
        if (hd) {
          dir = rot32(q.Rr, g3f(dx, dy, dz));
          have_dir = true;
        }
      }
    }
    // push the children nearest on top; those no longer within reach stay out
    if ((double)k0 > ub + m64) n0 = -1, k0 = CUDART_INF_F;
    if ((double)k1 > ub + m64) n1 = -1, k1 = CUDART_INF_F;
    const int np = __popc(__ballot_sync(full, n0 >= 0)) + __popc(__ballot_sync(full, n1 >= 0));
    if (np == 0) continue;
    if (size + np > kMdFront) {  // not reached for trees within kMdWarpMaxDepth
      if (lane == 0) atomicOr(L.status, 1u);
      break;
    }
    md_sort64(k0, n0, p0, k1, n1, p1, lane);
    // ascending order: entry e (valid for e < np) goes to size + np - 1 - e
    if (lane < np) {
      fnode[w][size + np - 1 - lane] = n0;
      flb[w][size + np - 1 - lane] = k0;
      fpath[w][size + np - 1 - lane] = p0;
    }
    if (lane + 32 < np) {
      fnode[w][size + np - 33 - lane] = n1;
      flb[w][size + np - 33 - lane] = k1;
      fpath[w][size + np - 33 - lane] = p1;
    }
    size += np;
    __syncwarp();
  }
  if (serial) {
    // A triangle at distance <= 0.  FCL's traversal then ends at the first intersecting
    // triangle (-1) it meets: bounds are >= 0, so nothing passes canStop after it.  That
    // is the first intersecting triangle in its depth-first order (children ordered by
    // its FP64 bounds, the second first on d2 < d1) whenever every volume on that
    // triangle's path has the FP64 bound 0 (an intersecting triangle's volumes overlap
    // the shape's, and FCL's RSS distance clamps at 0) and no triangle before it is at
    // distance exactly 0 (the running minimum then stays above 0, so those volumes pass
    // canStop).  The warp searches the volumes whose certified FP32 bound is within m64
    // of 0 in that order, 32 at a time (stack sorted by order path, earliest on top),
    // drops every volume after the best intersecting triangle found, and hands the pair
    // to FCL's serial traversal when a condition fails (a triangle at exactly 0, a
    // positive bound on the winner's path, triangle 0 at 0).
    bool cm_ok = true;
    int cbest = -1;
    {
      double d0 = 0.0;
      if (lane == 0) {
        double P[9];
        load_tri_local(g.m, 0, P);
        SimplexVert V[kSimplexSlots];
        D3v ps, pt;
        shape_triangle_distance(g.A, g.Rs, g.ts, P, g.Rm, g.tm, V, d0, ps, pt);
      }
      d0 = __shfl_sync(full, d0, 0);
      if (d0 < 0.0)
        cbest = 0;  // FCL's seed intersects: its result at once
      else if (d0 == 0.0)
        cm_ok = false;
    }
    if (cm_ok && cbest < 0) {
      // order path: bits from 31 down (0 = the child FCL enters first), a marker bit after
      // them, bit 0 = every FP64 bound on the path so far is 0
      unsigned best_key = 0xffffffffu;
      bool best_zero = false;
      __syncwarp();
      if (lane == 0) {
        fnode[w][0] = 0;
        fpath[w][0] = 0x80000000u | 1u;
      }
      int csize = 1;
      __syncwarp();
      while (csize > 0) {
        const int take = csize < 32 ? csize : 32;
        int b = -1;
        unsigned key = 0;
        if (lane < take) {
          b = fnode[w][csize - 1 - lane];
          key = fpath[w][csize - 1 - lane];
        }
        csize -= take;
        __syncwarp();
        if (b >= 0 && (key & ~31u) > (best_key & ~31u)) b = -1;  // after the best in FCL's order
        int child = 0;
        if (b >= 0) child = g.m.nodes64[b].child;
        const bool inner = b >= 0 && child >= 0;
        unsigned k0 = 0xffffffffu, k1 = 0xffffffffu;
        int n0 = -1, n1 = -1;
        unsigned p0 = 0, p1 = 0;
        if (inner) {
          const float l1 = md_node_bound(rss32, child, g.A, q, false, dir);
          const float l2 = md_node_bound(rss32, child + 1, g.A, q, false, dir);
          const double d1 = bvd(child), d2 = bvd(child + 1);
          const unsigned second_first = d2 < d1 ? 1u : 0u;
          const unsigned base = key & ~31u, zero = key & 1u;
          if ((double)l1 <= m64) {
            k0 = md_child_path(base, (int)second_first) | (zero & (d1 == 0.0 ? 1u : 0u));
            n0 = child;
          }
          if ((double)l2 <= m64) {
            k1 = md_child_path(base, (int)(second_first ^ 1u)) | (zero & (d2 == 0.0 ? 1u : 0u));
            n1 = child + 1;
          }
        }
        double d = 1.0;
        if (b >= 0 && child < 0) {
          double P[9];
          load_tri_local(g.m, -(child + 1), P);
          bool eval = true;
          if (!sphere) {
            G3f dd;
            eval = !((double)leaf_cert_lb(cert, P, dd) > m64);
          }
          if (eval) {
            SimplexVert V[kSimplexSlots];
            D3v ps, pt;
            shape_triangle_distance(g.A, g.Rs, g.ts, P, g.Rm, g.tm, V, d, ps, pt);
            if (d == 0.0) cm_ok = false;
          }
        }
        if (__any_sync(full, !cm_ok)) {
          cm_ok = false;
          break;
        }
        // the earliest intersecting triangle of the step
        unsigned kc = d < 0.0 ? (key & ~31u) : 0xffffffffu;
        for (int off = 16; off > 0; off >>= 1) kc = min(kc, __shfl_xor_sync(full, kc, off));
        if (kc < (best_key & ~31u)) {
          const int l = __ffs(__ballot_sync(full, d < 0.0 && (key & ~31u) == kc)) - 1;
          cbest = __shfl_sync(full, -(child + 1), l);
          best_key = __shfl_sync(full, key, l);
          best_zero = (best_key & 1u) != 0;
        }
        if ((k0 & ~31u) > (best_key & ~31u)) n0 = -1, k0 = 0xffffffffu;
        if ((k1 & ~31u) > (best_key & ~31u)) n1 = -1, k1 = 0xffffffffu;
        const int np = __popc(__ballot_sync(full, n0 >= 0)) + __popc(__ballot_sync(full, n1 >= 0));
        if (np == 0) continue;
        if (csize + np > kMdFront) {
          cm_ok = false;
          break;
        }
        md_sort64(k0, n0, p0, k1, n1, p1, lane);
        if (lane < np) {
          fnode[w][csize + np - 1 - lane] = n0;
          fpath[w][csize + np - 1 - lane] = k0;
        }
        if (lane + 32 < np) {
          fnode[w][csize + np - 33 - lane] = n1;
          fpath[w][csize + np - 33 - lane] = k1;
        }
        csize += np;
        __syncwarp();
      }
      if (cbest < 0 || !best_zero) cm_ok = false;
    }
    if (!cm_ok) {
      if (lane == 0) L.dist[i] = CUDART_NAN;
      return;
    }
    ub = -1.0;
    best = cbest;
  }
  if (lane == 0) {
    L.dist[i] = ub;
    if (WIT) {
      D3v ps = v3(0.0, 0.0, 0.0), pt = ps;
      if (best >= 0) {
        double P[9];
        load_tri_local(g.m, best, P);
        SimplexVert V[kSimplexSlots];
        double d;
        shape_triangle_distance(g.A, g.Rs, g.ts, P, g.Rm, g.tm, V, d, ps, pt);
      }
      if (L.tri) L.tri[i] = best;
      if (L.pts) {
        double* p = L.pts + 6 * i;
        p[0] = pt.x;
        p[1] = pt.y;
        p[2] = pt.z;
        p[3] = ps.x;
        p[4] = ps.y;
        p[5] = ps.z;
      }
    }
  }
}

// FCL's traversal, one thread per pair, for the pairs the order-free forms hand over
// (distance NaN) and the pairs with a refitted mesh
template <int STACK>
__global__ void __launch_bounds__(128) k_ms_dist_serial(MeshShapeLaunch L) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < L.n; i += stride) {
    if (!isnan(L.dist[i]) && !L.meshes[L.mesh_idx[i]].refitted) continue;
    PairGeom g;
    pair_geom(L, i, g);
    MeshShapeOut o;
    o.count = 0;
    o.tri = -1;
    o.dist = 0;
    o.pmesh = o.pshape = v3(0.0, 0.0, 0.0);
    o.nbv = o.nleaf = 0;
    o.status = 0;
    mesh_shape_distance<STACK>(g.m, g.Rm, g.tm, g.A, g.Rs, g.ts, o);
    if (o.status) atomicOr(L.status, 1u);
    L.dist[i] = o.dist;
    if (L.tri) L.tri[i] = o.tri;
    if (L.pts) {
      double* p = L.pts + 6 * i;
      p[0] = o.pmesh.x;
      p[1] = o.pmesh.y;
      p[2] = o.pmesh.z;
      p[3] = o.pshape.x;
      p[4] = o.pshape.y;
      p[5] = o.pshape.z;
    }
  }
}

// tris[offsets[pair] + rank] = triangle for every record
__global__ void k_msr_scatter(const int4* rec, const unsigned long long* nrec, const int64_t* offsets, int32_t* tris) {
  const long long n = (long long)*nrec;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += stride) {
    const int4 r = rec[t];
    tris[offsets[r.x] + r.y] = r.z;
  }
}

// contact geometry of every record (enable_contact), written beside its triangle; one
// thread per contact, each running the shape-triangle intersection with EPA in FP64
__global__ void __launch_bounds__(128) k_msr_geometry(MeshShapeLaunch L, const int4* rec,
                                                      const unsigned long long* nrec) {
  const long long n = (long long)*nrec;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += stride) {
    const int4 r = rec[t];
    PairGeom g;
    pair_geom(L, r.x, g);
    double P[9];
    load_tri_local(g.m, r.z, P);
    SimplexVert V[kSimplexSlots];
    EpaState epa;
    D3v pos, nrm;
    double depth = 0;
    if (!shape_triangle_contact(g.A, g.Rs, g.ts, P, g.Rm, g.tm, V, &epa, pos, nrm, depth)) {
      // the record came from the same tests, so this does not happen; keep it visible
      const double q = __longlong_as_double(0x7ff8000000000000ll);
      pos = nrm = v3(q, q, q);
      depth = q;
    }
    const long long o = L.list_offsets[r.x] + r.y;
    L.list_pos[3 * o] = pos.x;
    L.list_pos[3 * o + 1] = pos.y;
    L.list_pos[3 * o + 2] = pos.z;
    L.list_normal[3 * o] = nrm.x;
    L.list_normal[3 * o + 1] = nrm.y;
    L.list_normal[3 * o + 2] = nrm.z;
    L.list_depth[o] = depth;
  }
}

int grid128(long long n) { return (int)std::min<long long>(std::max<long long>((n + 127) / 128, 1), 152 * 32); }

}  // namespace

cudaError_t launch_exclusive_scan(const int32_t* counts, int64_t n, int64_t* offsets, int64_t* tmp, cudaStream_t s);

namespace {
struct SplitScratch {
  void* p[16] = {nullptr};
  size_t cap[16] = {0};
  cudaError_t ensure(int k, size_t bytes) {
    if (bytes <= cap[k]) return cudaSuccess;
    if (p[k]) cudaFree(p[k]);
    p[k] = nullptr;
    cap[k] = 0;
    const size_t want = std::max<size_t>(bytes + bytes / 4, 256);
    cudaError_t e = cudaMalloc(&p[k], want);
    if (e == cudaSuccess) cap[k] = want;
    return e;
  }
};
SplitScratch g_split_ms;
std::mutex g_split_mu;
}  // namespace

namespace {

cudaError_t run_collide_rounds(const MeshShapeLaunch& L, int stack_entries, cudaStream_t s, SplitScratch& S) {
  const long long n = L.n;
  const int cap = stack_entries;
  cudaError_t e;
  if ((e = S.ensure(0, sizeof(MsPairState) * n)) || (e = S.ensure(1, 4ull * cap * n)) || (e = S.ensure(2, 4 * n)) ||
      (e = S.ensure(3, 4 * n)) || (e = S.ensure(4, 4 * n)) || (e = S.ensure(5, 32)))
    return e;
  // contact list: records (pair, rank, triangle) in slot 11, counter nnext[3]
  MeshShapeLaunch Lr = L;
  const bool listing = L.list_offsets != nullptr;
  unsigned long long nrec_host = 0;
  if (listing) {
    Lr.nrec = (unsigned long long*)S.p[5] + 3;
    if ((e = cudaMemsetAsync(Lr.nrec, 0, 8, s))) return e;
  }
  MsPairState* ps = (MsPairState*)S.p[0];
  int32_t* stack = (int32_t*)S.p[1];
  int32_t* sp = (int32_t*)S.p[2];
  int32_t* act = (int32_t*)S.p[3];
  int32_t* next = (int32_t*)S.p[4];
  unsigned long long* nnext = (unsigned long long*)S.p[5];
  k_msr_init<<<grid128(n), 128, 0, s>>>(Lr, ps, stack, cap, sp, act);
  ++g_kernel_launches;
  long long nact = n;
  for (int r = 0; nact > 0; ++r) {
    const int K = 16 << std::min(r, 6);
    const long long nl = nact * K;
    if ((e = S.ensure(6, 4 * nl)) || (e = S.ensure(7, 4 * nact)) || (e = S.ensure(8, 4 * nl))) return e;
    if (listing) {  // a round adds at most one record per leaf it lists; grow keeping the records
      const size_t need = sizeof(int4) * (size_t)(nrec_host + nl);
      if (need > S.cap[11]) {
        void* np = nullptr;
        const size_t want = std::max<size_t>(need + need / 2, 4096);
        if ((e = cudaMalloc(&np, want))) return e;
        if (nrec_host && (e = cudaMemcpyAsync(np, S.p[11], sizeof(int4) * nrec_host, cudaMemcpyDeviceToDevice, s)))
          return e;
        if ((e = cudaStreamSynchronize(s))) return e;
        if (S.p[11]) cudaFree(S.p[11]);
        S.p[11] = np;
        S.cap[11] = want;
      }
      Lr.rec = (int4*)S.p[11];
    }
    int32_t* leaf = (int32_t*)S.p[6];
    int32_t* nleaf = (int32_t*)S.p[7];
    int32_t* hit = (int32_t*)S.p[8];
    if ((e = S.ensure(9, 4 * nl)) || (e = S.ensure(10, 4 * nact))) return e;
    int32_t* defer_leaf = (int32_t*)S.p[9];
    int32_t* defer_pair = (int32_t*)S.p[10];
    // nnext, then the deferred-leaf and deferred-pair counters
    if ((e = cudaMemsetAsync(nnext, 0, 24, s))) return e;
    // node tests per pair per round are capped too, so that one pair with a long
    // traversal does not hold every round up
    const int max_visits = 128 << std::min(r, 3);
    k_msr_dfs<<<grid128(nact), 128, 0, s>>>(Lr, act, nact, K, max_visits, ps, stack, cap, sp, leaf, nleaf);
    k_msr_tests<<<grid128(nl), 128, 0, s>>>(Lr, act, nact, K, leaf, nleaf, hit);
    k_msr_update<<<grid128(nact), 128, 0, s>>>(Lr, act, nact, K, leaf, nleaf, hit, sp, next, nnext, defer_leaf,
                                               nnext + 1, defer_pair, nnext + 2);
    k_msr_deferred<<<grid128(nl), 128, 0, s>>>(Lr, act, K, leaf, hit, defer_leaf, nnext + 1);
    k_msr_recount<<<grid128(nact), 128, 0, s>>>(Lr, act, K, leaf, nleaf, hit, sp, defer_pair, nnext + 2, next,
                                                nnext);
    g_kernel_launches += 5;
    unsigned long long nn[4] = {0, 0, 0, 0};
    if ((e = cudaGetLastError()) || (e = cudaMemcpyAsync(nn, nnext, 32, cudaMemcpyDeviceToHost, s)) ||
        (e = cudaStreamSynchronize(s)))
      return e;
    nact = (long long)nn[0];
    nrec_host = nn[3];
    std::swap(act, next);
  }
  if (listing) {
    if ((e = S.ensure(12, 8 * ((n + 4095) / 4096 + 2)))) return e;
    if ((e = launch_exclusive_scan(L.counts, n, L.list_offsets, (int64_t*)S.p[12], s))) return e;
    int64_t total = 0;
    if ((e = cudaMemcpyAsync(&total, L.list_offsets + n, 8, cudaMemcpyDeviceToHost, s)) ||
        (e = cudaStreamSynchronize(s)))
      return e;
    if (L.list_total) *L.list_total = total;
    if (total <= L.list_cap && nrec_host > 0) {
      k_msr_scatter<<<grid128((long long)nrec_host), 128, 0, s>>>(Lr.rec, Lr.nrec, L.list_offsets, L.list_tris);
      ++g_kernel_launches;
      if (L.list_pos) {
        k_msr_geometry<<<grid128((long long)nrec_host), 128, 0, s>>>(Lr, Lr.rec, Lr.nrec);
        ++g_kernel_launches;
      }
    }
  }
  return cudaGetLastError();
}

cudaError_t run_distance_split(const MeshShapeLaunch& L, int stack_entries, cudaStream_t s, SplitScratch& S) {
  const long long n = L.n;
  cudaError_t e;
  if ((e = S.ensure(0, 4 * n)) || (e = S.ensure(1, 8 * (n + 1))) || (e = S.ensure(2, 8 * ((n + 4095) / 4096 + 2))) ||
      (e = S.ensure(3, 8 * n)))
    return e;
  int32_t* counts = (int32_t*)S.p[0];
  int64_t* off = (int64_t*)S.p[1];
  double* ub = (double*)S.p[3];
  const bool big = stack_entries > 64;
  if (big)
    k_ms_collect<256><<<grid128(n), 128, 0, s>>>(L, counts, nullptr, nullptr, nullptr, nullptr, ub);
  else
    k_ms_collect<64><<<grid128(n), 128, 0, s>>>(L, counts, nullptr, nullptr, nullptr, nullptr, ub);
  ++g_kernel_launches;
  if ((e = cudaGetLastError())) return e;
  if ((e = launch_exclusive_scan(counts, n, off, (int64_t*)S.p[2], s))) return e;
  int64_t nl = 0;
  if ((e = cudaMemcpyAsync(&nl, off + n, 8, cudaMemcpyDeviceToHost, s)) || (e = cudaStreamSynchronize(s))) return e;
  if (nl > 0) {
    if ((e = S.ensure(4, 4 * nl)) || (e = S.ensure(5, 4 * nl)) || (e = S.ensure(6, 8 * nl)) ||
        (e = S.ensure(7, 56 * nl)))
      return e;
    int32_t* leaf_pair = (int32_t*)S.p[4];
    int32_t* leaf_prim = (int32_t*)S.p[5];
    double* leaf_lb = (double*)S.p[6];
    double* dist = (double*)S.p[7];
    double* pts = dist + nl;
    if (big)
      k_ms_collect<256><<<grid128(n), 128, 0, s>>>(L, nullptr, off, leaf_pair, leaf_prim, leaf_lb, nullptr);
    else
      k_ms_collect<64><<<grid128(n), 128, 0, s>>>(L, nullptr, off, leaf_pair, leaf_prim, leaf_lb, nullptr);
    k_ms_leaf_tests<<<grid128(nl), 128, 0, s>>>(L, nl, leaf_pair, leaf_prim, leaf_lb, ub, dist, pts);
    k_ms_reduce<<<grid128(n), 128, 0, s>>>(L, off, leaf_prim, dist, pts);
    g_kernel_launches += 3;
  } else {
    k_ms_reduce<<<grid128(n), 128, 0, s>>>(L, off, nullptr, nullptr, nullptr);
    ++g_kernel_launches;
  }
  return cudaGetLastError();
}

}  // namespace

cudaError_t run_mesh_shape_split(const MeshShapeLaunch& L, int stack_entries, cudaStream_t s) {
  if (L.n <= 0) return cudaSuccess;
  const cudaError_t ep = upload_solver_params(s);
  if (ep != cudaSuccess) return ep;
  std::lock_guard<std::mutex> lk(g_split_mu);
  if (L.mode == 0 && !L.list_offsets && stack_entries <= kMsWarpMaxDepth) {  // counts only
    k_ms_count_warp<<<(unsigned)((L.n + kMsWarps - 1) / kMsWarps), 32 * kMsWarps, 0, s>>>(L);
    ++g_kernel_launches;
    return cudaGetLastError();
  }
  if (L.mode == 1 && stack_entries <= kMdWarpMaxDepth) {  // distance: warp per pair, then the handed-over pairs
    const unsigned blocks = (unsigned)((L.n + kMdWarps - 1) / kMdWarps);
    if (L.tri || L.pts)
      k_ms_dist_warp<true><<<blocks, 32 * kMdWarps, 0, s>>>(L);
    else
      k_ms_dist_warp<false><<<blocks, 32 * kMdWarps, 0, s>>>(L);
    k_ms_dist_serial<64><<<(unsigned)std::min<long long>((L.n + 127) / 128, 152 * 32), 128, 0, s>>>(L);
    g_kernel_launches += 2;
    return cudaGetLastError();
  }
  if (L.mode == 0) return run_collide_rounds(L, stack_entries, s, g_split_ms);
  const cudaError_t e = run_distance_split(L, stack_entries, s, g_split_ms);
  if (e != cudaSuccess) return e;
  const unsigned grid = (unsigned)std::min<long long>((L.n + 127) / 128, 152 * 32);
  if (stack_entries <= 64)
    k_ms_dist_serial<64><<<grid, 128, 0, s>>>(L);
  else
    k_ms_dist_serial<256><<<grid, 128, 0, s>>>(L);
  ++g_kernel_launches;
  return cudaGetLastError();
}

cudaError_t launch_mesh_shape(const MeshShapeLaunch& L, int stack_entries, cudaStream_t s) {
  if (L.n <= 0) return cudaSuccess;
  const cudaError_t ep = upload_solver_params(s);
  if (ep != cudaSuccess) return ep;
  const long long want = (L.n + 127) / 128;
  const int grid = (int)std::min<long long>(std::max<long long>(want, 1), 152 * 32);
  if (stack_entries <= 64)
    k_mesh_shape<64><<<grid, 128, 0, s>>>(L);
  else
    k_mesh_shape<256><<<grid, 128, 0, s>>>(L);
  ++g_kernel_launches;
  return cudaGetLastError();
}

}  // namespace fclgpu

using namespace fclgpu;

namespace {

std::mutex g_ms_mu;

struct MsBuf {
  void* p = nullptr;
  size_t cap = 0;
  cudaError_t ensure(size_t bytes) {
    if (bytes <= cap) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
    const size_t want = std::max<size_t>(bytes, 256);
    cudaError_t e = cudaMalloc(&p, want);
    if (e == cudaSuccess) cap = want;
    return e;
  }
};
MsBuf g_ms_meshes, g_ms_status;

int ms_fail(int code, const std::string& why) {
  set_error_detail(why);
  return code;
}
int ms_cuda(cudaError_t e, const char* where) {
  set_error_detail(std::string(where) + ": " + cudaGetErrorString(e));
  return e == cudaErrorMemoryAllocation ? FCLGPU_ERR_OUT_OF_MEMORY : FCLGPU_ERR_CUDA;
}

}  // namespace

extern "C" {

int fclgpu_mesh_shape_batch_device(const fclgpu_mesh* meshes, int32_t num_meshes, fclgpu_shapeset shapes, int64_t n,
                                   const int32_t* mesh_idx, const int32_t* shape_idx, const double* tf_mesh,
                                   const double* tf_shape, const fclgpu_mesh_shape_request* req,
                                   fclgpu_mesh_shape_result* res, void* stream) {
  if (!req || !res || n < 0 || !meshes || num_meshes <= 0 || !shapes)
    return ms_fail(FCLGPU_ERR_INVALID_ARGUMENT, "missing mesh-shape argument");
  if (req->mode != FCLGPU_MESH_SHAPE_COLLIDE && req->mode != FCLGPU_MESH_SHAPE_DISTANCE)
    return ms_fail(FCLGPU_ERR_INVALID_ARGUMENT, "unknown mode");
  if (n > 0 && (!mesh_idx || !shape_idx || !tf_mesh || !tf_shape ||
                (req->mode == FCLGPU_MESH_SHAPE_COLLIDE ? !res->counts : !res->min_distance)))
    return ms_fail(FCLGPU_ERR_INVALID_ARGUMENT, "missing mesh-shape input or output");
  if (req->mode == FCLGPU_MESH_SHAPE_COLLIDE && req->num_max_contacts < 1)
    return ms_fail(FCLGPU_ERR_INVALID_ARGUMENT, "num_max_contacts must be >= 1");
  std::vector<DevMesh> table(num_meshes);
  int depth = 0;
  for (int32_t i = 0; i < num_meshes; ++i) {
    if (!meshes[i]) return ms_fail(FCLGPU_ERR_INVALID_ARGUMENT, "null mesh handle");
    table[i] = meshes[i]->dev;
    depth = std::max(depth, (int)meshes[i]->dev.max_depth);
  }
  if (depth + 2 > 256) return ms_fail(FCLGPU_ERR_STACK_DEPTH, "BVH deeper than the traversal stack");
  if (n == 0) return FCLGPU_OK;
  std::lock_guard<std::mutex> lk(g_ms_mu);
  cudaStream_t s = (cudaStream_t)stream;
  cudaError_t e = g_ms_meshes.ensure(sizeof(DevMesh) * num_meshes);
  if (e == cudaSuccess) e = g_ms_status.ensure(sizeof(unsigned));
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(g_ms_meshes.p, table.data(), sizeof(DevMesh) * num_meshes, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(g_ms_status.p, 0, sizeof(unsigned), s);
  if (e != cudaSuccess) return ms_cuda(e, "mesh-shape setup");
  MeshShapeLaunch L;
  L.meshes = static_cast<const DevMesh*>(g_ms_meshes.p);
  L.shapes = shapes->shapes;
  L.sverts = shapes->verts;
  L.n = n;
  L.mesh_idx = mesh_idx;
  L.shape_idx = shape_idx;
  L.tfm = tf_mesh;
  L.tfs = tf_shape;
  L.mode = req->mode;
  L.max_contacts = (int32_t)std::min<int64_t>(req->num_max_contacts, INT32_MAX);
  L.counts = res->counts;
  L.dist = res->min_distance;
  L.tri = res->tri;
  L.pts = res->nearest_points;
  L.nbv = res->num_bv_tests;
  L.nleaf = res->num_leaf_tests;
  L.status = static_cast<unsigned*>(g_ms_status.p);
  // statistics need the serial traversal; otherwise the leaf tests run one per thread
  e = (L.nbv || L.nleaf) ? launch_mesh_shape(L, depth + 2, s) : run_mesh_shape_split(L, depth + 2, s);
  unsigned st = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&st, g_ms_status.p, sizeof(unsigned), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return ms_cuda(e, "mesh-shape kernel");
  if (st) return ms_fail(FCLGPU_ERR_STACK_DEPTH, "mesh-shape traversal stack overflow");
  return FCLGPU_OK;
}

int fclgpu_mesh_shape_batch(const fclgpu_mesh* meshes, int32_t num_meshes, fclgpu_shapeset shapes, int64_t n,
                            const int32_t* mesh_idx, const int32_t* shape_idx, const double* tf_mesh,
                            const double* tf_shape, const fclgpu_mesh_shape_request* req,
                            fclgpu_mesh_shape_result* res, void* stream) {
  if (!req || !res || n < 0) return ms_fail(FCLGPU_ERR_INVALID_ARGUMENT, "missing mesh-shape argument");
  if (n == 0)
    return fclgpu_mesh_shape_batch_device(meshes, num_meshes, shapes, 0, mesh_idx, shape_idx, tf_mesh, tf_shape, req,
                                          res, stream);
  cudaStream_t s = (cudaStream_t)stream;
  const size_t nn = (size_t)n;
  // one staging block: inputs, then outputs
  const size_t bytes = nn * (4 + 4 + 96 + 96 + 4 + 8 + 4 + 48 + 8 + 8) + 16;  // + alignment padding
  char* d = nullptr;
  cudaError_t e = cudaMalloc(&d, bytes);
  if (e != cudaSuccess) return ms_cuda(e, "staging");
  int32_t* dm = (int32_t*)d;
  int32_t* ds = dm + nn;
  double* dtm = (double*)(ds + nn);
  double* dts = dtm + 12 * nn;
  int32_t* dc = (int32_t*)(dts + 12 * nn);
  double* dd = (double*)(dc + nn + (nn & 1));
  int32_t* dt = (int32_t*)(dd + nn);
  double* dp = (double*)(dt + nn + (nn & 1));
  int64_t* db = (int64_t*)(dp + 6 * nn);
  int64_t* dl = db + nn;
  if (e == cudaSuccess) e = cudaMemcpyAsync(dm, mesh_idx, 4 * nn, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(ds, shape_idx, 4 * nn, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dtm, tf_mesh, 96 * nn, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dts, tf_shape, 96 * nn, cudaMemcpyHostToDevice, s);
  int rc = FCLGPU_OK;
  if (e != cudaSuccess) {
    rc = ms_cuda(e, "h2d");
  } else {
    fclgpu_mesh_shape_result dr = {dc, dd, dt, dp, db, dl};
    rc = fclgpu_mesh_shape_batch_device(meshes, num_meshes, shapes, n, dm, ds, dtm, dts, req, &dr, stream);
    if (rc == FCLGPU_OK) {
      if (req->mode == FCLGPU_MESH_SHAPE_COLLIDE) {
        e = cudaMemcpyAsync(res->counts, dc, 4 * nn, cudaMemcpyDeviceToHost, s);
      } else {
        e = cudaMemcpyAsync(res->min_distance, dd, 8 * nn, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess && res->tri) e = cudaMemcpyAsync(res->tri, dt, 4 * nn, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess && res->nearest_points)
          e = cudaMemcpyAsync(res->nearest_points, dp, 48 * nn, cudaMemcpyDeviceToHost, s);
      }
      if (e == cudaSuccess && res->num_bv_tests)
        e = cudaMemcpyAsync(res->num_bv_tests, db, 8 * nn, cudaMemcpyDeviceToHost, s);
      if (e == cudaSuccess && res->num_leaf_tests)
        e = cudaMemcpyAsync(res->num_leaf_tests, dl, 8 * nn, cudaMemcpyDeviceToHost, s);
      if (e == cudaSuccess) e = cudaStreamSynchronize(s);
      if (e != cudaSuccess) rc = ms_cuda(e, "d2h");
    }
  }
  cudaFree(d);
  return rc;
}

int fclgpu_mesh_shape_contacts_device(const fclgpu_mesh* meshes, int32_t num_meshes, fclgpu_shapeset shapes,
                                      int64_t n, const int32_t* mesh_idx, const int32_t* shape_idx,
                                      const double* tf_mesh, const double* tf_shape, int64_t num_max_contacts,
                                      fclgpu_mesh_shape_contacts_result* res, void* stream) {
  if (!res || n < 0 || !meshes || num_meshes <= 0 || !shapes)
    return ms_fail(FCLGPU_ERR_INVALID_ARGUMENT, "missing mesh-shape argument");
  if (num_max_contacts < 1) return ms_fail(FCLGPU_ERR_INVALID_ARGUMENT, "num_max_contacts must be >= 1");
  if (!res->offsets || (n > 0 && (!mesh_idx || !shape_idx || !tf_mesh || !tf_shape || !res->counts)) ||
      (res->capacity > 0 && !res->tris) || res->capacity < 0)
    return ms_fail(FCLGPU_ERR_INVALID_ARGUMENT, "missing mesh-shape input or output");
  const int ngeo = (res->pos ? 1 : 0) + (res->normal ? 1 : 0) + (res->penetration_depth ? 1 : 0);
  if (ngeo != 0 && ngeo != 3)
    return ms_fail(FCLGPU_ERR_INVALID_ARGUMENT, "pos, normal and penetration_depth go together");
  std::vector<DevMesh> table(num_meshes);
  int depth = 0;
  for (int32_t i = 0; i < num_meshes; ++i) {
    if (!meshes[i]) return ms_fail(FCLGPU_ERR_INVALID_ARGUMENT, "null mesh handle");
    table[i] = meshes[i]->dev;
    depth = std::max(depth, (int)meshes[i]->dev.max_depth);
  }
  if (depth + 2 > 256) return ms_fail(FCLGPU_ERR_STACK_DEPTH, "BVH deeper than the traversal stack");
  cudaStream_t s = (cudaStream_t)stream;
  res->total_contacts = 0;
  if (n == 0) {
    const int64_t zero = 0;
    cudaError_t e = cudaMemcpyAsync(res->offsets, &zero, 8, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    return e == cudaSuccess ? FCLGPU_OK : ms_cuda(e, "offsets");
  }
  std::lock_guard<std::mutex> lk(g_ms_mu);
  cudaError_t e = g_ms_meshes.ensure(sizeof(DevMesh) * num_meshes);
  if (e == cudaSuccess) e = g_ms_status.ensure(sizeof(unsigned));
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(g_ms_meshes.p, table.data(), sizeof(DevMesh) * num_meshes, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(g_ms_status.p, 0, sizeof(unsigned), s);
  if (e != cudaSuccess) return ms_cuda(e, "mesh-shape setup");
  MeshShapeLaunch L;
  L.meshes = static_cast<const DevMesh*>(g_ms_meshes.p);
  L.shapes = shapes->shapes;
  L.sverts = shapes->verts;
  L.n = n;
  L.mesh_idx = mesh_idx;
  L.shape_idx = shape_idx;
  L.tfm = tf_mesh;
  L.tfs = tf_shape;
  L.mode = 0;
  L.max_contacts = (int32_t)std::min<int64_t>(num_max_contacts, INT32_MAX);
  L.counts = res->counts;
  L.dist = nullptr;
  L.tri = nullptr;
  L.pts = nullptr;
  L.nbv = nullptr;
  L.nleaf = nullptr;
  L.status = static_cast<unsigned*>(g_ms_status.p);
  L.list_offsets = res->offsets;
  L.list_tris = res->tris;
  L.list_cap = res->capacity;
  if (ngeo == 3 && res->capacity > 0) {
    L.list_pos = res->pos;
    L.list_normal = res->normal;
    L.list_depth = res->penetration_depth;
  }
  int64_t total = 0;
  L.list_total = &total;
  e = run_mesh_shape_split(L, depth + 2, s);
  unsigned st = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&st, g_ms_status.p, sizeof(unsigned), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return ms_cuda(e, "mesh-shape kernel");
  if (st) return ms_fail(FCLGPU_ERR_STACK_DEPTH, "mesh-shape traversal stack overflow");
  res->total_contacts = total;
  if (total > res->capacity) return ms_fail(FCLGPU_ERR_CAPACITY, "tris buffer too small");
  return FCLGPU_OK;
}

int fclgpu_mesh_shape_contacts(const fclgpu_mesh* meshes, int32_t num_meshes, fclgpu_shapeset shapes, int64_t n,
                               const int32_t* mesh_idx, const int32_t* shape_idx, const double* tf_mesh,
                               const double* tf_shape, int64_t num_max_contacts,
                               fclgpu_mesh_shape_contacts_result* res, void* stream) {
  if (!res || n < 0 || res->capacity < 0 || !res->offsets || (n > 0 && !res->counts) ||
      (res->capacity > 0 && !res->tris))
    return ms_fail(FCLGPU_ERR_INVALID_ARGUMENT, "missing mesh-shape argument");
  const int ngeo = (res->pos ? 1 : 0) + (res->normal ? 1 : 0) + (res->penetration_depth ? 1 : 0);
  if (ngeo != 0 && ngeo != 3)
    return ms_fail(FCLGPU_ERR_INVALID_ARGUMENT, "pos, normal and penetration_depth go together");
  const bool geo = ngeo == 3;
  cudaStream_t s = (cudaStream_t)stream;
  const size_t nn = (size_t)n, cap = (size_t)res->capacity;
  // inputs, counts, offsets, the contact geometry and a device list as large as the caller's
  const size_t bytes = nn * (4 + 4 + 96 + 96 + 4) + 8 * (nn + 2) + (geo ? 56 * cap : 0) + 4 * cap + 64;
  char* d = nullptr;
  cudaError_t e = cudaMalloc(&d, bytes);
  if (e != cudaSuccess) return ms_cuda(e, "staging");
  double* dtm = (double*)d;
  double* dts = dtm + 12 * nn;
  int64_t* doff = (int64_t*)(dts + 12 * nn);
  double* dpos = (double*)(doff + nn + 2);
  double* dnrm = dpos + (geo ? 3 * cap : 0);
  double* ddep = dnrm + (geo ? 3 * cap : 0);
  int32_t* dm = (int32_t*)(ddep + (geo ? cap : 0));
  int32_t* ds = dm + nn;
  int32_t* dc = ds + nn;
  int32_t* dt = dc + nn;
  if (n > 0) {
    if (e == cudaSuccess) e = cudaMemcpyAsync(dm, mesh_idx, 4 * nn, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(ds, shape_idx, 4 * nn, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dtm, tf_mesh, 96 * nn, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dts, tf_shape, 96 * nn, cudaMemcpyHostToDevice, s);
  }
  int rc = FCLGPU_OK;
  if (e != cudaSuccess) {
    rc = ms_cuda(e, "h2d");
  } else {
    fclgpu_mesh_shape_contacts_result dr = {dc,  doff, dt, res->capacity, 0, geo ? dpos : nullptr,
                                             geo ? dnrm : nullptr, geo ? ddep : nullptr};
    rc = fclgpu_mesh_shape_contacts_device(meshes, num_meshes, shapes, n, dm, ds, dtm, dts, num_max_contacts, &dr,
                                           stream);
    res->total_contacts = dr.total_contacts;
    if (rc == FCLGPU_OK || rc == FCLGPU_ERR_CAPACITY) {
      if (n > 0) e = cudaMemcpyAsync(res->counts, dc, 4 * nn, cudaMemcpyDeviceToHost, s);
      if (e == cudaSuccess) e = cudaMemcpyAsync(res->offsets, doff, 8 * (nn + 1), cudaMemcpyDeviceToHost, s);
      if (e == cudaSuccess && rc == FCLGPU_OK && dr.total_contacts > 0)
        e = cudaMemcpyAsync(res->tris, dt, 4 * (size_t)dr.total_contacts, cudaMemcpyDeviceToHost, s);
      if (e == cudaSuccess && geo && rc == FCLGPU_OK && dr.total_contacts > 0) {
        const size_t tc = (size_t)dr.total_contacts;
        e = cudaMemcpyAsync(res->pos, dpos, 24 * tc, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaMemcpyAsync(res->normal, dnrm, 24 * tc, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaMemcpyAsync(res->penetration_depth, ddep, 8 * tc, cudaMemcpyDeviceToHost, s);
      }
      if (e == cudaSuccess) e = cudaStreamSynchronize(s);
      if (e != cudaSuccess) rc = ms_cuda(e, "d2h");
    }
  }
  cudaFree(d);
  return rc;
}

}  // extern "C"
