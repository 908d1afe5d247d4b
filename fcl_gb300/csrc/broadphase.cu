// Device broadphase kernels: world AABBs, LBVH build (Morton codes, radix sort,
// Karras hierarchy, bottom-up refit), candidate passes and narrowphase dispatch.
//
// Reference behaviour (FCL 0.7.0, paths relative to the FCL repository):
//   CollisionObject::computeAABB           narrowphase/collision_object-inl.h:116-131
//   AABB::overlap / AABB::distance         math/bv/AABB-inl.h:98-107, 292-315
//   collisionRecurse(root, query)          broadphase/broadphase_dynamic_AABB_tree-inl.h:526-547
//   distanceRecurse(root, query, min_dist) broadphase/broadphase_dynamic_AABB_tree-inl.h:658-701
//   DefaultCollisionFunction / DefaultDistanceFunction
//                                          broadphase/default_broadphase_callbacks.h:88-106, 195-215
// The hierarchy is built by the method of Karras, "Maximizing Parallelism in the
// Construction of BVHs, Octrees, and k-d Trees" (HPG 2012), over 30-bit Morton codes of
// the box centres, ties broken by object index.
#include <cfloat>

#include "broadphase.h"
#include "kernels.h"
#include "mesh_shape.cuh"
#include "shape_pair.cuh"

namespace fclgpu {

cudaError_t launch_exclusive_scan(const int32_t* counts, int64_t n, int64_t* offsets, int64_t* tmp, cudaStream_t s);

namespace {

constexpr int kBpStack = 64;  // Karras depth <= 30 key bits + 31 index bits
constexpr int kRadixBlock = 256;
constexpr int kScanTileElems = 4096;  // launch_exclusive_scan tile

int grid_for(int64_t n, int block) {
  const int64_t g = (n + block - 1) / block;
  return (int)(g < 1 ? 1 : (g > 152 * 64 ? 152 * 64 : g));
}

// ------------------------------------------------------------------ AABBs ----

// Eigen's isIdentity() with dummy_precision 1e-12 (diagonal isApprox(1), the rest
// isMuchSmallerThan(1)), on the rotation of a row-major 3x4 pose.
__device__ bool rot_is_identity(const double* t) {
  const double prec = 1e-12;
#pragma unroll
  for (int j = 0; j < 3; ++j)
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      const double a = t[4 * i + j];
      if (i == j) {
        if (!(fabs(a - 1.0) <= fmin(fabs(a), 1.0) * prec)) return false;
      } else {
        if (!(fabs(a) <= prec)) return false;
      }
    }
  return true;
}

__global__ void k_world_aabbs(const GeomRec* geoms, long long n, const int32_t* gid, const double* tf, double* a64,
                              float* a32) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const GeomRec& g = geoms[gid[i]];
    const double* p = tf + 12 * i;
    double lo[3], hi[3];
    if (rot_is_identity(p)) {
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        lo[k] = g.lo[k] + p[4 * k + 3];
        hi[k] = g.hi[k] + p[4 * k + 3];
      }
    } else {
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const double c = ((p[4 * k] * g.center[0] + p[4 * k + 1] * g.center[1]) + p[4 * k + 2] * g.center[2]) +
                         p[4 * k + 3];
        lo[k] = c - g.radius;
        hi[k] = c + g.radius;
      }
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      a64[6 * i + k] = lo[k];
      a64[6 * i + 3 + k] = hi[k];
      if (a32) {
        a32[6 * i + k] = __double2float_rd(lo[k]);
        a32[6 * i + 3 + k] = __double2float_ru(hi[k]);
      }
    }
  }
}

// ------------------------------------------------------------- LBVH build ----

struct BuildScratch {
  uint32_t* keys_a;
  uint32_t* keys_b;
  int32_t* vals_a;
  int32_t* vals_b;
  int32_t* hist;
  int64_t* hist_off;
  int64_t* scan_tmp;
  float* bounds;       // 6: centre min, centre max
  int32_t* node_parent;
  int32_t* leaf_parent;
  int32_t* flags;
};

size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

BuildScratch carve(void* base, int64_t n, size_t* total) {
  const int64_t ntiles = (n + kRadixBlock - 1) / kRadixBlock;
  const int64_t nh = 256 * ntiles;
  const int64_t nscan = (nh + kScanTileElems - 1) / kScanTileElems + 2;
  size_t off = 0;
  BuildScratch b;
  char* p = static_cast<char*>(base);
  auto take = [&](size_t bytes) {
    char* r = p ? p + off : nullptr;
    off += align256(bytes);
    return r;
  };
  b.keys_a = (uint32_t*)take(4 * n);
  b.keys_b = (uint32_t*)take(4 * n);
  b.vals_a = (int32_t*)take(4 * n);
  b.vals_b = (int32_t*)take(4 * n);
  b.hist = (int32_t*)take(4 * nh);
  b.hist_off = (int64_t*)take(8 * (nh + 1));
  b.scan_tmp = (int64_t*)take(8 * nscan);
  b.bounds = (float*)take(4 * 6);
  b.node_parent = (int32_t*)take(4 * n);
  b.leaf_parent = (int32_t*)take(4 * n);
  b.flags = (int32_t*)take(4 * n);
  if (total) *total = off;
  return b;
}

// centre bounds, one block
__global__ void __launch_bounds__(1024) k_center_bounds(const float* a32, int n, float* bounds) {
  __shared__ float sh[6][32];
  float mn[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, mx[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
  for (int i = threadIdx.x; i < n; i += blockDim.x)
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const float c = 0.5f * (a32[6 * i + k] + a32[6 * i + 3 + k]);
      mn[k] = fminf(mn[k], c);
      mx[k] = fmaxf(mx[k], c);
    }
#pragma unroll
  for (int k = 0; k < 3; ++k)
    for (int o = 16; o > 0; o >>= 1) {
      mn[k] = fminf(mn[k], __shfl_xor_sync(0xffffffffu, mn[k], o));
      mx[k] = fmaxf(mx[k], __shfl_xor_sync(0xffffffffu, mx[k], o));
    }
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0)
    for (int k = 0; k < 3; ++k) {
      sh[k][w] = mn[k];
      sh[3 + k][w] = mx[k];
    }
  __syncthreads();
  if (w == 0) {
    const int nw = blockDim.x >> 5;
    for (int k = 0; k < 3; ++k) {
      float a = lane < nw ? sh[k][lane] : FLT_MAX;
      float b = lane < nw ? sh[3 + k][lane] : -FLT_MAX;
      for (int o = 16; o > 0; o >>= 1) {
        a = fminf(a, __shfl_xor_sync(0xffffffffu, a, o));
        b = fmaxf(b, __shfl_xor_sync(0xffffffffu, b, o));
      }
      if (lane == 0) {
        bounds[k] = a;
        bounds[3 + k] = b;
      }
    }
  }
}

__device__ __forceinline__ uint32_t spread10(uint32_t v) {
  v = (v * 0x00010001u) & 0xFF0000FFu;
  v = (v * 0x00000101u) & 0x0F00F00Fu;
  v = (v * 0x00000011u) & 0xC30C30C3u;
  v = (v * 0x00000005u) & 0x49249249u;
  return v;
}

__global__ void k_morton(const float* a32, int n, const float* bounds, uint32_t* keys, int32_t* vals) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint32_t q[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const float c = 0.5f * (a32[6 * i + k] + a32[6 * i + 3 + k]);
    const float ext = bounds[3 + k] - bounds[k];
    float u = ext > 0.f ? (c - bounds[k]) / ext : 0.f;
    u = fminf(fmaxf(u * 1024.f, 0.f), 1023.f);
    q[k] = (uint32_t)u;
  }
  keys[i] = (spread10(q[0]) << 2) | (spread10(q[1]) << 1) | spread10(q[2]);
  vals[i] = i;
}

// stable LSD radix sort, 8-bit digits, one element per thread, 256-element tiles
__global__ void __launch_bounds__(kRadixBlock) k_radix_hist(const uint32_t* keys, int n, int shift, int ntiles,
                                                            int32_t* hist) {
  __shared__ int cnt[256];
  cnt[threadIdx.x] = 0;
  __syncthreads();
  const int i = blockIdx.x * kRadixBlock + threadIdx.x;
  if (i < n) atomicAdd(&cnt[(keys[i] >> shift) & 255u], 1);
  __syncthreads();
  hist[(long long)threadIdx.x * ntiles + blockIdx.x] = cnt[threadIdx.x];
}

__global__ void __launch_bounds__(kRadixBlock) k_radix_scatter(const uint32_t* kin, const int32_t* vin, int n,
                                                               int shift, int ntiles, const int64_t* off,
                                                               uint32_t* kout, int32_t* vout) {
  constexpr int kWarps = kRadixBlock / 32;
  __shared__ int wc[kWarps][256];
  const int i = blockIdx.x * kRadixBlock + threadIdx.x;
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const bool valid = i < n;
  const uint32_t key = valid ? kin[i] : 0u;
  const uint32_t d = valid ? ((key >> shift) & 255u) : 256u;
  for (int k = 0; k < kWarps; ++k) wc[k][threadIdx.x] = 0;
  __syncthreads();
  const unsigned peers = __match_any_sync(0xffffffffu, d);
  const unsigned lt = (1u << lane) - 1u;
  const int rank = __popc(peers & lt);
  if (valid && rank == 0) wc[w][d] = __popc(peers);
  __syncthreads();
  {
    int run = 0;
    for (int k = 0; k < kWarps; ++k) {
      const int t = wc[k][threadIdx.x];
      wc[k][threadIdx.x] = run;
      run += t;
    }
  }
  __syncthreads();
  if (valid) {
    const long long dst = off[(long long)d * ntiles + blockIdx.x] + wc[w][d] + rank;
    kout[dst] = key;
    vout[dst] = vin[i];
  }
}

__device__ __forceinline__ int kdelta(const uint32_t* k, int n, int i, int j) {
  if (j < 0 || j >= n) return -1;
  const uint32_t a = k[i], b = k[j];
  if (a != b) return __clz(a ^ b);
  return 32 + __clz((uint32_t)i ^ (uint32_t)j);
}

// Karras 2012, Figure 4: internal node i of n - 1
__global__ void k_karras(const uint32_t* keys, const int32_t* vals, int n, BpNode* nodes, int32_t* node_parent,
                         int32_t* leaf_parent) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n - 1) return;
  const int d = (kdelta(keys, n, i, i + 1) - kdelta(keys, n, i, i - 1)) >= 0 ? 1 : -1;
  const int dmin = kdelta(keys, n, i, i - d);
  int lmax = 2;
  while (kdelta(keys, n, i, i + lmax * d) > dmin) lmax *= 2;
  int l = 0;
  for (int t = lmax / 2; t >= 1; t /= 2)
    if (kdelta(keys, n, i, i + (l + t) * d) > dmin) l += t;
  const int j = i + l * d;
  const int dnode = kdelta(keys, n, i, j);
  int s = 0;
  for (int div = 2;; div *= 2) {
    const int t = (l + div - 1) / div;
    if (kdelta(keys, n, i, i + (s + t) * d) > dnode) s += t;
    if (t <= 1) break;
  }
  const int gamma = i + s * d + min(d, 0);
  const int lo = min(i, j), hi = max(i, j);
  int c0, c1;
  if (lo == gamma) {
    c0 = ~vals[gamma];
    leaf_parent[gamma] = i;
  } else {
    c0 = gamma;
    node_parent[gamma] = i;
  }
  if (hi == gamma + 1) {
    c1 = ~vals[gamma + 1];
    leaf_parent[gamma + 1] = i;
  } else {
    c1 = gamma + 1;
    node_parent[gamma + 1] = i;
  }
  nodes[i].c0 = c0;
  nodes[i].c1 = c1;
  nodes[i].pad0 = nodes[i].pad1 = 0;
  if (i == 0) node_parent[0] = -1;
}

__device__ __forceinline__ void write_slot(BpNode* nd, int slot, const float* lo, const float* hi) {
  volatile float* f = reinterpret_cast<volatile float*>(nd);
  const int b = slot ? 8 : 0;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    f[b + k] = lo[k];
    f[b + 4 + k] = hi[k];
  }
}

// bottom-up refit: the second thread to reach a node merges its two child boxes
__global__ void k_refit(const int32_t* vals, int n, const float* a32, BpNode* nodes, const int32_t* node_parent,
                        const int32_t* leaf_parent, int32_t* flags) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  const int obj = vals[p];
  float lo[3], hi[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    lo[k] = a32[6 * obj + k];
    hi[k] = a32[6 * obj + 3 + k];
  }
  int node = leaf_parent[p];
  int slot = (nodes[node].c0 == ~obj) ? 0 : 1;
  for (int guard = 0; guard < n; ++guard) {  // a path to the root has fewer than n nodes
    write_slot(nodes + node, slot, lo, hi);
    __threadfence();
    if (atomicAdd(&flags[node], 1) == 0) return;
    __threadfence();
    const volatile float* f = reinterpret_cast<const volatile float*>(nodes + node);
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      lo[k] = fminf(f[k], f[8 + k]);
      hi[k] = fmaxf(f[4 + k], f[12 + k]);
    }
    const int parent = node_parent[node];
    if (parent < 0) return;
    slot = (nodes[parent].c0 == node) ? 0 : 1;
    node = parent;
  }
}

// ------------------------------------------------------------------ queries ----

struct QBox {
  float lo[3], hi[3];
  double lo64[3], hi64[3];
};

__device__ __forceinline__ void load_qbox(const BpQueryView& Q, long long q, QBox& b) {
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    b.lo[k] = Q.aabb32[6 * q + k];
    b.hi[k] = Q.aabb32[6 * q + 3 + k];
    b.lo64[k] = Q.aabb64[6 * q + k];
    b.hi64[k] = Q.aabb64[6 * q + 3 + k];
  }
}

struct NodeRegs {
  float lo0[3], hi0[3], lo1[3], hi1[3];
  int c0, c1;
};

__device__ __forceinline__ void load_node(const BpNode* nodes, int i, NodeRegs& r) {
  const float4* p = reinterpret_cast<const float4*>(nodes + i);
  const float4 a = __ldg(p), b = __ldg(p + 1), c = __ldg(p + 2), d = __ldg(p + 3);
  r.lo0[0] = a.x; r.lo0[1] = a.y; r.lo0[2] = a.z; r.c0 = __float_as_int(a.w);
  r.hi0[0] = b.x; r.hi0[1] = b.y; r.hi0[2] = b.z; r.c1 = __float_as_int(b.w);
  r.lo1[0] = c.x; r.lo1[1] = c.y; r.lo1[2] = c.z;
  r.hi1[0] = d.x; r.hi1[1] = d.y; r.hi1[2] = d.z;
}

// AABB::overlap with the node box as *this and the query box as other
__device__ __forceinline__ bool ov32(const float* lo, const float* hi, const QBox& q) {
  return !(lo[0] > q.hi[0] || lo[1] > q.hi[1] || lo[2] > q.hi[2] || hi[0] < q.lo[0] || hi[1] < q.lo[1] ||
           hi[2] < q.lo[2]);
}
__device__ __forceinline__ bool ov64(const double* a, const QBox& q) {
  if (a[0] > q.hi64[0] || a[1] > q.hi64[1] || a[2] > q.hi64[2]) return false;
  if (a[3] < q.lo64[0] || a[4] < q.lo64[1] || a[5] < q.lo64[2]) return false;
  return true;
}
// lower bound (rounded down) of the distance between the query box and a node box
__device__ __forceinline__ float lb32(const float* lo, const float* hi, const QBox& q) {
  float s = 0.f;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    float g = 0.f;
    if (q.lo[k] > hi[k])
      g = __fsub_rd(q.lo[k], hi[k]);
    else if (lo[k] > q.hi[k])
      g = __fsub_rd(lo[k], q.hi[k]);
    s = __fadd_rd(s, __fmul_rd(g, g));
  }
  return __fsqrt_rd(s);
}
// AABB::distance with the query box as *this (distanceRecurse's order)
__device__ __forceinline__ double dist64(const QBox& q, const double* b) {
  double result = 0;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    if (q.lo64[k] > b[3 + k]) {
      const double delta = b[3 + k] - q.lo64[k];
      result += delta * delta;
    } else if (b[k] > q.hi64[k]) {
      const double delta = q.hi64[k] - b[k];
      result += delta * delta;
    }
  }
  return sqrt(result);
}

// Candidate traversal.  WITHIN = false: FP64 AABB overlap; WITHIN = true: FP64 AABB
// distance <= ub[q].
template <bool WITHIN>
__global__ void __launch_bounds__(128) k_bp_candidates(BpSceneView S, BpQueryView Q, const double* ub,
                                                       int32_t* counts, const int64_t* offsets, int2* pairs,
                                                       int64_t* node_visits, unsigned* status) {
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= Q.nq) return;
  QBox qb;
  load_qbox(Q, q, qb);
  const double bound = WITHIN ? ub[q] : 0.0;
  const float bound32 = WITHIN ? (float)bound : 0.f;  // compare lb32 <= bound via double below
  (void)bound32;
  const long long base = offsets ? offsets[q] : 0;
  int cnt = 0;
  long long visits = 0;
  auto leaf = [&](int obj) {
    if (Q.self && obj >= q) return;
    const double* a = S.aabb64 + 6 * (long long)obj;
    const bool take = WITHIN ? (dist64(qb, a) <= bound) : ov64(a, qb);
    if (take) {
      if (pairs) pairs[base + cnt] = make_int2((int)q, obj);
      ++cnt;
    }
  };
  auto keep = [&](const float* lo, const float* hi) {
    return WITHIN ? ((double)lb32(lo, hi, qb) <= bound) : ov32(lo, hi, qb);
  };
  if (S.n > 0) {
    if (S.root < 0) {
      leaf(~S.root);
    } else {
      int stack[kBpStack];
      int sp = 0;
      int node = S.root;
      for (;;) {
        if (++visits > S.n) {  // each of the n - 1 internal nodes is loaded at most once
          atomicOr(status, BP_ERR_STACK);
          break;
        }
        NodeRegs r;
        load_node(S.nodes, node, r);
        int next = -1;
        if (keep(r.lo0, r.hi0)) {
          if (r.c0 < 0)
            leaf(~r.c0);
          else
            next = r.c0;
        }
        if (keep(r.lo1, r.hi1)) {
          if (r.c1 < 0) {
            leaf(~r.c1);
          } else if (next < 0) {
            next = r.c1;
          } else if (sp < kBpStack) {
            stack[sp++] = r.c1;
          } else {
            atomicOr(status, BP_ERR_STACK);
            break;
          }
        }
        if (next >= 0) {
          node = next;
          continue;
        }
        if (sp == 0) break;
        node = stack[--sp];
      }
    }
  }
  if (counts) counts[q] = cnt;
  if (node_visits && visits) atomicAdd(reinterpret_cast<unsigned long long*>(node_visits), (unsigned long long)visits);
}

// world position of a point of the geometry, and for shapes the support point toward dir
__device__ D3v geom_point(const BpSceneView& S, const GeomRec& g, const double* tf) {
  const D3v r = v3(g.ref[0], g.ref[1], g.ref[2]);
  return v3(((tf[0] * r.x + tf[1] * r.y) + tf[2] * r.z) + tf[3], ((tf[4] * r.x + tf[5] * r.y) + tf[6] * r.z) + tf[7],
            ((tf[8] * r.x + tf[9] * r.y) + tf[10] * r.z) + tf[11]);
}
__device__ D3v geom_support(const BpSceneView& S, const GeomRec& g, const double* tf, const D3v& dir) {
  ShapeRef sh;
  sh.s = S.shapes[g.index];
  sh.verts = S.sverts;
  // local direction R^T dir
  const D3v ld = v3((tf[0] * dir.x + tf[4] * dir.y) + tf[8] * dir.z, (tf[1] * dir.x + tf[5] * dir.y) + tf[9] * dir.z,
                    (tf[2] * dir.x + tf[6] * dir.y) + tf[10] * dir.z);
  const D3v p = shape_support(sh, ld);
  return v3(((tf[0] * p.x + tf[1] * p.y) + tf[2] * p.z) + tf[3], ((tf[4] * p.x + tf[5] * p.y) + tf[6] * p.z) + tf[7],
            ((tf[8] * p.x + tf[9] * p.y) + tf[10] * p.z) + tf[11]);
}
__device__ __forceinline__ double d3len(const D3v& a) { return sqrt((a.x * a.x + a.y * a.y) + a.z * a.z); }

// Upper bound of the distance between scene object obj and query q: the distance
// between one point of each (support points toward each other for shapes).
__device__ double pair_upper_bound(const BpSceneView& S, const BpQueryView& Q, int obj, long long q) {
  const GeomRec& go = S.geoms[S.gid[obj]];
  const GeomRec& gq = S.geoms[Q.gid[q]];
  const double* to = S.tf + 12 * (long long)obj;
  const double* tq = Q.tf + 12 * q;
  D3v pa = geom_point(S, go, to);
  D3v pb = geom_point(S, gq, tq);
  const double best = d3len(pa - pb);
  if (!(best > 0)) return best;
  // the support functions (minkowski_diff-inl.h:65-265) take unit directions
  const D3v dir = d3scale(pb - pa, 1.0 / best);
  if (go.kind == GEOM_SHAPE) pa = geom_support(S, go, to, dir);
  if (gq.kind == GEOM_SHAPE) pb = geom_support(S, gq, tq, d3neg(dir));
  return fmin(best, d3len(pa - pb));
}

__global__ void __launch_bounds__(128) k_bp_dist_bound(BpSceneView S, BpQueryView Q, double* ub, unsigned* status) {
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= Q.nq) return;
  QBox qb;
  load_qbox(Q, q, qb);
  double best = DBL_MAX;
  auto leaf = [&](int obj) {
    if (Q.self && obj >= q) return;
    if (dist64(qb, S.aabb64 + 6 * (long long)obj) > best) return;
    best = fmin(best, pair_upper_bound(S, Q, obj, q));
  };
  if (S.n > 0) {
    if (S.root < 0) {
      leaf(~S.root);
    } else {
      int stack[kBpStack];
      float slb[kBpStack];
      int sp = 0;
      int node = S.root;
      for (int guard = 0;; ++guard) {
        if (guard >= S.n) {  // each internal node is loaded at most once
          atomicOr(status, BP_ERR_STACK);
          break;
        }
        NodeRegs r;
        load_node(S.nodes, node, r);
        const float l0 = lb32(r.lo0, r.hi0, qb), l1 = lb32(r.lo1, r.hi1, qb);
        // visit the nearer child first, as distanceRecurse does
        const bool first1 = l1 < l0;
        int next = -1;
        float next_lb = 0.f;
        for (int t = 0; t < 2; ++t) {
          const int side = first1 ? 1 - t : t;
          const int c = side ? r.c1 : r.c0;
          const float l = side ? l1 : l0;
          if ((double)l > best) continue;
          if (c < 0) {
            leaf(~c);
          } else if (next < 0) {
            next = c;
            next_lb = l;
          } else if (sp < kBpStack) {
            stack[sp] = c;
            slb[sp] = l;
            ++sp;
          } else {
            atomicOr(status, BP_ERR_STACK);
          }
        }
        (void)next_lb;
        if (next >= 0) {
          node = next;
          continue;
        }
        bool found = false;
        while (sp > 0) {
          --sp;
          if ((double)slb[sp] <= best) {
            node = stack[sp];
            found = true;
            break;
          }
        }
        if (!found) break;
      }
    }
  }
  ub[q] = best;
}

__global__ void k_bp_query_gids(const int2* refs, long long nq, int ns, int nm, int32_t* gid, unsigned* status) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < nq; q += stride) {
    const int2 r = refs[q];
    int g = 0;
    if (r.x == GEOM_SHAPE && r.y >= 0 && r.y < ns) {
      g = r.y;
    } else if (r.x == GEOM_MESH && r.y >= 0 && r.y < nm) {
      g = ns + r.y;
    } else {
      atomicOr(status, BP_ERR_REF);
    }
    gid[q] = g;
  }
}

__global__ void k_bp_classify(BpSceneView S, BpQueryView Q, const int2* pairs, long long n, int32_t* kind) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const int2 p = pairs[i];
    const int ko = S.geoms[S.gid[p.y]].kind, kq = S.geoms[Q.gid[p.x]].kind;
    kind[i] = (ko == GEOM_SHAPE && kq == GEOM_SHAPE) ? 0 : ((ko == GEOM_MESH && kq == GEOM_MESH) ? 1 : 2);
  }
}

// fcl::collide / fcl::distance of one (scene object, query) shape pair, in the
// callback's argument order (scene object first)
__global__ void __launch_bounds__(128) k_bp_shape_narrow(BpSceneView S, BpQueryView Q, const int2* pairs, long long n,
                                                         const int32_t* kind, int mode, int32_t* hit, double* dist,
                                                         double* pts) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    if (kind[i] != 0) continue;
    const int2 p = pairs[i];
    const DevShape sa = S.shapes[S.geoms[S.gid[p.y]].index];
    const DevShape sb = S.shapes[S.geoms[Q.gid[p.x]].index];
    PairOut o;
    shape_pair_query(sa, sb, S.sverts, S.tf + 12 * (long long)p.y, Q.tf + 12 * (long long)p.x, o,
                     mode == PAIR_INTERSECT ? (PAIR_INTERSECT | PAIR_NO_CONTACT) : mode);
    if (mode == PAIR_INTERSECT) {
      hit[i] = o.hit;
    } else {
      dist[i] = o.dist;
      if (pts) {
        pts[6 * i + 0] = o.p1.x;
        pts[6 * i + 1] = o.p1.y;
        pts[6 * i + 2] = o.p1.z;
        pts[6 * i + 3] = o.p2.x;
        pts[6 * i + 4] = o.p2.y;
        pts[6 * i + 5] = o.p2.z;
      }
    }
  }
}

__global__ void k_bp_list(const int32_t* kind, long long n, int32_t want, const int2* pairs, const int32_t* qdone,
                          int64_t* list, unsigned long long* count) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
    if (kind[i] == want && !(qdone && qdone[pairs[i].x])) list[atomicAdd(count, 1ull)] = i;
}

__global__ void k_bp_query_done(long long nq, const int64_t* off, const int32_t* hit, long long maxc,
                                int32_t* qdone) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < nq; q += stride) {
    long long total = 0;
    for (long long i = off[q]; i < off[q + 1]; ++i) total += hit[i];
    qdone[q] = total >= maxc ? 1 : 0;
  }
}

__global__ void k_bp_gather_mesh(BpSceneView S, BpQueryView Q, const int2* pairs, const int64_t* list, long long nl,
                                 int32_t nm, int32_t* pair_index, double* tf1, double* tf2) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x; j < nl; j += stride) {
    const int2 p = pairs[list[j]];
    pair_index[j] = S.geoms[S.gid[p.y]].index * nm + S.geoms[Q.gid[p.x]].index;
#pragma unroll
    for (int k = 0; k < 12; ++k) {
      tf1[12 * j + k] = S.tf[12 * (long long)p.y + k];
      tf2[12 * j + k] = Q.tf[12 * (long long)p.x + k];
    }
  }
}

__global__ void k_bp_gather_mixed(BpSceneView S, BpQueryView Q, const int2* pairs, const int64_t* list, long long nl,
                                  int32_t* mesh_idx, int32_t* shape_idx, double* tfm, double* tfs, int32_t* bv_src,
                                  int32_t* need, int32_t* query_of) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x; j < nl; j += stride) {
    const int2 p = pairs[list[j]];
    const GeomRec& go = S.geoms[S.gid[p.y]];
    const GeomRec& gq = S.geoms[Q.gid[p.x]];
    const bool obj_is_mesh = go.kind == GEOM_MESH;
    mesh_idx[j] = obj_is_mesh ? go.index : gq.index;
    shape_idx[j] = obj_is_mesh ? gq.index : go.index;
    if (query_of) query_of[j] = p.x;
    if (bv_src) {
      const long long src = obj_is_mesh ? (long long)p.x : Q.nq + p.y;
      bv_src[j] = (int32_t)src;
      need[src] = 1;
    }
    const double* a = obj_is_mesh ? S.tf + 12 * (long long)p.y : Q.tf + 12 * (long long)p.x;
    const double* b = obj_is_mesh ? Q.tf + 12 * (long long)p.x : S.tf + 12 * (long long)p.y;
#pragma unroll
    for (int k = 0; k < 12; ++k) {
      tfm[12 * j + k] = a[k];
      tfs[12 * j + k] = b[k];
    }
  }
}

// world-frame shape BV per needed source: queries first, then scene objects
__global__ void __launch_bounds__(128) k_bp_shape_bvs(BpSceneView S, BpQueryView Q, const int32_t* need,
                                                      ShapeBV* table) {
  const long long n = Q.nq + S.n;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long src = (long long)blockIdx.x * blockDim.x + threadIdx.x; src < n; src += stride) {
    if (!need[src]) continue;
    const bool is_q = src < Q.nq;
    const long long o = src - Q.nq;
    ShapeBV* cache = static_cast<ShapeBV*>(S.bv_cache);
    if (!is_q && S.bv_ok && S.bv_ok[o]) {  // a scene object keeps its pose between updates
      table[src] = cache[o];
      continue;
    }
    const GeomRec& g = S.geoms[is_q ? Q.gid[src] : S.gid[o]];
    M3<double> R;
    D3v t;
    load_tf(is_q ? Q.tf + 12 * src : S.tf + 12 * o, R, t);
    shape_obbrss(S.shapes[g.index], S.sverts, R, t, table[src]);
    if (!is_q && S.bv_ok) {
      cache[o] = table[src];
      S.bv_ok[o] = 1;
    }
  }
}

__global__ void k_bp_scatter_mixed_dist(const int64_t* list, long long nl, const double* d, const int32_t* tri,
                                        const double* pts, double* dist, int32_t* b12, double* outpts) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x; j < nl; j += stride) {
    const long long i = list[j];
    dist[i] = d[j];
    b12[2 * i] = tri[j];
    b12[2 * i + 1] = -1;
    for (int k = 0; k < 6; ++k) outpts[6 * i + k] = pts[6 * j + k];
  }
}

__global__ void k_bp_scatter_hits(const int64_t* list, long long nl, const int32_t* counts, int32_t* hit) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x; j < nl; j += stride) hit[list[j]] = counts[j];
}

__global__ void k_bp_scatter_dist(const int64_t* list, long long nl, const double* d, const int32_t* ids,
                                  const double* pts, double* dist, int32_t* b12, double* outpts) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x; j < nl; j += stride) {
    const long long i = list[j];
    dist[i] = d[j];
    if (ids) {
      b12[2 * i] = ids[2 * j];
      b12[2 * i + 1] = ids[2 * j + 1];
    }
    if (pts)
      for (int k = 0; k < 6; ++k) outpts[6 * i + k] = pts[6 * j + k];
  }
}

__global__ void k_bp_reduce_collide(long long nq, const int64_t* off, const int2* pairs, const int32_t* hit,
                                    long long maxc, int64_t* num_contacts, int32_t* num_objects,
                                    int32_t* first_object) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < nq; q += stride) {
    long long total = 0;
    int nobj = 0, first = -1;
    for (long long i = off[q]; i < off[q + 1]; ++i) {
      const int h = hit[i];
      if (h > 0) {
        total += h;
        ++nobj;
        const int o = pairs[i].y;
        if (first < 0 || o < first) first = o;
      }
    }
    if (num_contacts) num_contacts[q] = total < maxc ? total : maxc;
    if (num_objects) num_objects[q] = nobj;
    if (first_object) first_object[q] = first;
  }
}

__global__ void k_bp_reduce_distance(long long nq, const int64_t* off, const int2* pairs, const double* dist,
                                     const int32_t* b12, const double* pts, double* min_distance, int32_t* object,
                                     int32_t* ids, double* nearest) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < nq; q += stride) {
    double best = DBL_MAX;
    int bo = -1;
    long long bi = -1;
    for (long long i = off[q]; i < off[q + 1]; ++i) {
      const double d = dist[i];
      const int o = pairs[i].y;
      if (d < best || (d == best && bo >= 0 && o < bo)) {
        best = d;
        bo = o;
        bi = i;
      }
    }
    min_distance[q] = best;
    if (object) object[q] = bo;
    if (ids) {
      ids[2 * q] = bi >= 0 ? b12[2 * bi] : -1;
      ids[2 * q + 1] = bi >= 0 ? b12[2 * bi + 1] : -1;
    }
    if (nearest)
      for (int k = 0; k < 6; ++k) nearest[6 * q + k] = bi >= 0 ? pts[6 * bi + k] : 0.0;
  }
}

// ------------------------------------------------------------- contact lists ----

// One thread per query: its candidate slots sorted by object index (insertion sort;
// a query overlaps few objects).
__global__ void k_bp_sort_segments(long long nq, const int64_t* off, const int2* pairs, int64_t* perm) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < nq; q += stride) {
    const long long lo = off[q], hi = off[q + 1];
    for (long long i = lo; i < hi; ++i) {
      const int oi = pairs[i].y;
      long long j = i;
      while (j > lo && pairs[perm[j - 1]].y > oi) {
        perm[j] = perm[j - 1];
        --j;
      }
      perm[j] = i;
    }
  }
}

__global__ void k_bp_inverse_index(const int64_t* list, long long nl, int32_t* index) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < nl; k += stride)
    index[list[k]] = (int32_t)k;
}

__global__ void k_bp_gather_counts(const int64_t* perm, long long n, const int32_t* hit, int32_t* ccount) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x; j < n; j += stride) ccount[j] = hit[perm[j]];
}

__global__ void k_bp_query_contacts(long long nq, const int64_t* off, const int64_t* coff, int64_t* counts,
                                    int64_t* out_off) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q <= nq; q += stride) {
    const int64_t a = coff[off[q]];
    if (out_off) out_off[q] = a;
    if (q < nq && counts) counts[q] = coff[off[q + 1]] - a;
  }
}

__global__ void k_bp_fill_contacts(const int64_t* perm, long long n, const int2* pairs, const int32_t* kind,
                                   const int32_t* hit, const int64_t* coff, const int32_t* mm_index,
                                   const int64_t* mm_off, const int32_t* mm_contacts, const int32_t* ms_index,
                                   const int64_t* ms_off, const int32_t* ms_tris, int32_t* out) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x; j < n; j += stride) {
    const long long slot = perm[j];
    const int c = hit[slot];
    if (c <= 0) continue;
    const int obj = pairs[slot].y;
    int32_t* o = out + 3 * coff[j];
    const int k = kind[slot];
    if (k == 0) {
      o[0] = obj;
      o[1] = -1;
      o[2] = -1;
    } else if (k == 1) {
      const int32_t* src = mm_contacts + 2 * mm_off[mm_index[slot]];
      for (int t = 0; t < c; ++t) {
        o[3 * t] = obj;
        o[3 * t + 1] = src[2 * t];
        o[3 * t + 2] = src[2 * t + 1];
      }
    } else {
      const int32_t* src = ms_tris + ms_off[ms_index[slot]];
      for (int t = 0; t < c; ++t) {
        o[3 * t] = obj;
        o[3 * t + 1] = src[t];
        o[3 * t + 2] = -1;
      }
    }
  }
}

}  // namespace

// ------------------------------------------------------------------ launches ----

cudaError_t launch_world_aabbs(const GeomRec* geoms, int64_t n, const int32_t* gid, const double* tf, double* aabb64,
                               float* aabb32, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_world_aabbs<<<grid_for(n, 256), 256, 0, s>>>(geoms, n, gid, tf, aabb64, aabb32);
  ++g_kernel_launches;
  return cudaGetLastError();
}

size_t bp_build_scratch_bytes(int64_t n) {
  size_t total = 0;
  carve(nullptr, n, &total);
  return total;
}

cudaError_t launch_lbvh_build(int32_t n, const float* aabb32, BpNode* nodes, void* scratch, cudaStream_t s) {
  if (n < 2) return cudaSuccess;
  BuildScratch b = carve(scratch, n, nullptr);
  const int ntiles = (n + kRadixBlock - 1) / kRadixBlock;
  const int g = (n + 255) / 256;
  k_center_bounds<<<1, 1024, 0, s>>>(aabb32, n, b.bounds);
  k_morton<<<g, 256, 0, s>>>(aabb32, n, b.bounds, b.keys_a, b.vals_a);
  g_kernel_launches += 2;
  uint32_t *kin = b.keys_a, *kout = b.keys_b;
  int32_t *vin = b.vals_a, *vout = b.vals_b;
  for (int shift = 0; shift < 32; shift += 8) {
    k_radix_hist<<<ntiles, kRadixBlock, 0, s>>>(kin, n, shift, ntiles, b.hist);
    ++g_kernel_launches;
    cudaError_t e = launch_exclusive_scan(b.hist, 256ll * ntiles, b.hist_off, b.scan_tmp, s);
    if (e != cudaSuccess) return e;
    k_radix_scatter<<<ntiles, kRadixBlock, 0, s>>>(kin, vin, n, shift, ntiles, b.hist_off, kout, vout);
    ++g_kernel_launches;
    uint32_t* tk = kin;
    kin = kout;
    kout = tk;
    int32_t* tv = vin;
    vin = vout;
    vout = tv;
  }
  // after four passes the sorted keys are back in keys_a / vals_a
  k_karras<<<(n - 1 + 255) / 256, 256, 0, s>>>(kin, vin, n, nodes, b.node_parent, b.leaf_parent);
  cudaMemsetAsync(b.flags, 0, sizeof(int32_t) * n, s);
  k_refit<<<g, 256, 0, s>>>(vin, n, aabb32, nodes, b.node_parent, b.leaf_parent, b.flags);
  g_kernel_launches += 2;
  return cudaGetLastError();
}

cudaError_t launch_bp_overlap(const BpSceneView& S, const BpQueryView& Q, int32_t* counts, const int64_t* offsets,
                              int2* pairs, int64_t* node_visits, unsigned* status, cudaStream_t s) {
  if (Q.nq <= 0) return cudaSuccess;
  k_bp_candidates<false><<<(unsigned)((Q.nq + 127) / 128), 128, 0, s>>>(S, Q, nullptr, counts, offsets, pairs,
                                                                        node_visits, status);
  ++g_kernel_launches;
  return cudaGetLastError();
}

cudaError_t launch_bp_dist_bound(const BpSceneView& S, const BpQueryView& Q, double* ub, unsigned* status,
                                 cudaStream_t s) {
  if (Q.nq <= 0) return cudaSuccess;
  k_bp_dist_bound<<<(unsigned)((Q.nq + 127) / 128), 128, 0, s>>>(S, Q, ub, status);
  ++g_kernel_launches;
  return cudaGetLastError();
}

cudaError_t launch_bp_dist_candidates(const BpSceneView& S, const BpQueryView& Q, const double* ub, int32_t* counts,
                                      const int64_t* offsets, int2* pairs, int64_t* node_visits, unsigned* status,
                                      cudaStream_t s) {
  if (Q.nq <= 0) return cudaSuccess;
  k_bp_candidates<true><<<(unsigned)((Q.nq + 127) / 128), 128, 0, s>>>(S, Q, ub, counts, offsets, pairs, node_visits,
                                                                       status);
  ++g_kernel_launches;
  return cudaGetLastError();
}

cudaError_t launch_bp_query_gids(const int2* refs, int64_t nq, int32_t ns, int32_t nm, int32_t* gid,
                                 unsigned* status, cudaStream_t s) {
  if (nq <= 0) return cudaSuccess;
  k_bp_query_gids<<<grid_for(nq, 256), 256, 0, s>>>(refs, nq, ns, nm, gid, status);
  ++g_kernel_launches;
  return cudaGetLastError();
}

cudaError_t launch_bp_classify(const BpSceneView& S, const BpQueryView& Q, const int2* pairs, int64_t n,
                               int32_t* kind, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_bp_classify<<<grid_for(n, 256), 256, 0, s>>>(S, Q, pairs, n, kind);
  ++g_kernel_launches;
  return cudaGetLastError();
}

cudaError_t launch_bp_shape_narrow(const BpSceneView& S, const BpQueryView& Q, const int2* pairs, int64_t n,
                                   const int32_t* kind, int mode, int32_t* hit, double* dist, double* pts,
                                   cudaStream_t s) {
  const cudaError_t ep = upload_solver_params(s);
  if (ep != cudaSuccess) return ep;
  if (n <= 0) return cudaSuccess;
  k_bp_shape_narrow<<<grid_for(n, 128), 128, 0, s>>>(S, Q, pairs, n, kind, mode, hit, dist, pts);
  ++g_kernel_launches;
  return cudaGetLastError();
}

cudaError_t launch_bp_gather_mesh(const BpSceneView& S, const BpQueryView& Q, const int2* pairs,
                                  const int64_t* list, int64_t nlist, int32_t nm, int32_t* pair_index, double* tf1,
                                  double* tf2, cudaStream_t s) {
  if (nlist <= 0) return cudaSuccess;
  k_bp_gather_mesh<<<grid_for(nlist, 256), 256, 0, s>>>(S, Q, pairs, list, nlist, nm, pair_index, tf1, tf2);
  ++g_kernel_launches;
  return cudaGetLastError();
}

cudaError_t launch_bp_list(const int32_t* kind, int64_t n, int32_t want, const int2* pairs, const int32_t* qdone,
                           int64_t* list, unsigned long long* count, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_bp_list<<<grid_for(n, 256), 256, 0, s>>>(kind, n, want, pairs, qdone, list, count);
  ++g_kernel_launches;
  return cudaGetLastError();
}

cudaError_t launch_bp_query_done(int64_t nq, const int64_t* offsets, const int32_t* hit, int64_t max_contacts,
                                 int32_t* qdone, cudaStream_t s) {
  if (nq <= 0) return cudaSuccess;
  k_bp_query_done<<<grid_for(nq, 256), 256, 0, s>>>(nq, offsets, hit, max_contacts, qdone);
  ++g_kernel_launches;
  return cudaGetLastError();
}

cudaError_t launch_bp_gather_mixed(const BpSceneView& S, const BpQueryView& Q, const int2* pairs,
                                   const int64_t* list, int64_t nlist, int32_t* mesh_idx, int32_t* shape_idx,
                                   double* tfm, double* tfs, int32_t* bv_src, int32_t* need, int32_t* query_of,
                                   cudaStream_t s) {
  if (nlist <= 0) return cudaSuccess;
  k_bp_gather_mixed<<<grid_for(nlist, 256), 256, 0, s>>>(S, Q, pairs, list, nlist, mesh_idx, shape_idx, tfm, tfs,
                                                          bv_src, need, query_of);
  ++g_kernel_launches;
  return cudaGetLastError();
}

cudaError_t launch_bp_shape_bvs(const BpSceneView& S, const BpQueryView& Q, const int32_t* need, void* table,
                                cudaStream_t s) {
  const long long n = Q.nq + S.n;
  k_bp_shape_bvs<<<grid_for(n, 128), 128, 0, s>>>(S, Q, need, static_cast<ShapeBV*>(table));
  ++g_kernel_launches;
  return cudaGetLastError();
}

cudaError_t launch_bp_scatter_mixed_dist(const int64_t* list, int64_t nlist, const double* d, const int32_t* tri,
                                         const double* pts, double* dist, int32_t* b12, double* outpts,
                                         cudaStream_t s) {
  if (nlist <= 0) return cudaSuccess;
  k_bp_scatter_mixed_dist<<<grid_for(nlist, 256), 256, 0, s>>>(list, nlist, d, tri, pts, dist, b12, outpts);
  ++g_kernel_launches;
  return cudaGetLastError();
}

cudaError_t launch_bp_scatter_hits(const int64_t* list, int64_t nlist, const int32_t* counts, int32_t* hit,
                                   cudaStream_t s) {
  if (nlist <= 0) return cudaSuccess;
  k_bp_scatter_hits<<<grid_for(nlist, 256), 256, 0, s>>>(list, nlist, counts, hit);
  ++g_kernel_launches;
  return cudaGetLastError();
}

cudaError_t launch_bp_scatter_dist(const int64_t* list, int64_t nlist, const double* d, const int32_t* ids,
                                   const double* pts, double* dist, int32_t* b12, double* outpts, cudaStream_t s) {
  if (nlist <= 0) return cudaSuccess;
  k_bp_scatter_dist<<<grid_for(nlist, 256), 256, 0, s>>>(list, nlist, d, ids, pts, dist, b12, outpts);
  ++g_kernel_launches;
  return cudaGetLastError();
}

cudaError_t launch_bp_reduce_collide(int64_t nq, const int64_t* offsets, const int2* pairs, const int32_t* hit,
                                     int64_t max_contacts, int64_t* num_contacts, int32_t* num_objects,
                                     int32_t* first_object, cudaStream_t s) {
  if (nq <= 0) return cudaSuccess;
  k_bp_reduce_collide<<<grid_for(nq, 256), 256, 0, s>>>(nq, offsets, pairs, hit, max_contacts, num_contacts,
                                                        num_objects, first_object);
  ++g_kernel_launches;
  return cudaGetLastError();
}

cudaError_t launch_bp_reduce_distance(int64_t nq, const int64_t* offsets, const int2* pairs, const double* dist,
                                      const int32_t* b12, const double* pts, double* min_distance, int32_t* object,
                                      int32_t* ids, double* nearest, cudaStream_t s) {
  if (nq <= 0) return cudaSuccess;
  k_bp_reduce_distance<<<grid_for(nq, 256), 256, 0, s>>>(nq, offsets, pairs, dist, b12, pts, min_distance, object,
                                                         ids, nearest);
  ++g_kernel_launches;
  return cudaGetLastError();
}

cudaError_t launch_bp_sort_segments(int64_t nq, const int64_t* offsets, const int2* pairs, int64_t* perm,
                                    cudaStream_t s) {
  k_bp_sort_segments<<<grid_for(nq, 128), 128, 0, s>>>(nq, offsets, pairs, perm);
  ++g_kernel_launches;
  return cudaGetLastError();
}

cudaError_t launch_bp_inverse_index(const int64_t* list, int64_t nlist, int32_t* index, cudaStream_t s) {
  if (nlist <= 0) return cudaSuccess;
  k_bp_inverse_index<<<grid_for(nlist, 256), 256, 0, s>>>(list, nlist, index);
  ++g_kernel_launches;
  return cudaGetLastError();
}

cudaError_t launch_bp_gather_counts(const int64_t* perm, int64_t total, const int32_t* hit, int32_t* ccount,
                                    cudaStream_t s) {
  if (total <= 0) return cudaSuccess;
  k_bp_gather_counts<<<grid_for(total, 256), 256, 0, s>>>(perm, total, hit, ccount);
  ++g_kernel_launches;
  return cudaGetLastError();
}

cudaError_t launch_bp_query_contacts(int64_t nq, const int64_t* offsets, const int64_t* coff, int64_t* counts,
                                     int64_t* out_offsets, cudaStream_t s) {
  k_bp_query_contacts<<<grid_for(nq + 1, 256), 256, 0, s>>>(nq, offsets, coff, counts, out_offsets);
  ++g_kernel_launches;
  return cudaGetLastError();
}

cudaError_t launch_bp_fill_contacts(const int64_t* perm, int64_t total, const int2* pairs, const int32_t* kind,
                                    const int32_t* hit, const int64_t* coff, const int32_t* mm_index,
                                    const int64_t* mm_off, const int32_t* mm_contacts, const int32_t* ms_index,
                                    const int64_t* ms_off, const int32_t* ms_tris, int32_t* out, cudaStream_t s) {
  if (total <= 0) return cudaSuccess;
  k_bp_fill_contacts<<<grid_for(total, 128), 128, 0, s>>>(perm, total, pairs, kind, hit, coff, mm_index, mm_off,
                                                          mm_contacts, ms_index, ms_off, ms_tris, out);
  ++g_kernel_launches;
  return cudaGetLastError();
}

}  // namespace fclgpu
