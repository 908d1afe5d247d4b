// Batched BVHModel<OBBRSS> x BVHModel<OBBRSS> distance on the GPU.
//
// One thread runs one query.  The plain FP64 form (PREC 0) is FCL's distance
// traversal: preprocess with triangle 0 x triangle 0
// (mesh_distance_traversal_node-inl.h:545-586), then distanceRecurse
// (traversal_recurse-inl.h:257-316): RSS distance to both children of the larger
// node, nearer child first, a child skipped when canStop(d) = d >= min_distance
// (rel_err = abs_err = 0, :147-153), leaf = triDistance with DistanceResult's strict
// "<" update (distance_result-inl.h:84-105); nearest points mapped to world by tf1
// (postprocess, :589-603).
//
// The FP32 form (PREC 1) is the certified traversal of distance_traverse.cuh: BV
// pairs are pruned with FP32 support-function gaps whose forward error is bounded,
// triangle pairs are skipped only when a certified FP32 lower bound exceeds the best
// FP64 distance so far, and every other triangle pair is evaluated with FCL's FP64
// triDistance and the strict "<" update.  The reported distance, triangle ids and
// witness points are FP64 values of the winning pair.
#include <math_constants.h>

#include <algorithm>

#include "distance_traverse.cuh"
#include "filter32.cuh"
#include "geom.cuh"
#include "kernels.h"

namespace fclgpu {

namespace {

struct DStack {
  int b1, b2;
  double d;
};

__device__ __forceinline__ void load_tfs(const DistanceLaunch& L, long long qi, double* a, double* b) {
  if (L.tf1) {
#pragma unroll
    for (int i = 0; i < 12; ++i) a[i] = __ldg(L.tf1 + 12 * qi + i);
  } else {
#pragma unroll
    for (int i = 0; i < 12; ++i) a[i] = (i == 0 || i == 5 || i == 10) ? 1.0 : 0.0;
  }
#pragma unroll
  for (int i = 0; i < 12; ++i) b[i] = __ldg(L.tf2 + 12 * qi + i);
}

// Exact FP64 triangle distance of triangle p1 (mesh A) and p2 (mesh B moved by R,T);
// points in A's frame.
__device__ __noinline__ double leaf_distance64(const DevMesh& A, const DevMesh& B, int p1, int p2,
                                               const M3<double>& R, const V3<double>& T, V3<double>& P,
                                               V3<double>& Q) {
  const int* ta = A.tris + 3 * (long long)p1;
  const int* tb = B.tris + 3 * (long long)p2;
  V3<double> T1[3], T2[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const double* pa = A.verts64 + 3 * (long long)__ldg(ta + k);
    const double* pb = B.verts64 + 3 * (long long)__ldg(tb + k);
    T1[k] = v3(__ldg(pa), __ldg(pa + 1), __ldg(pa + 2));
    T2[k] = mulv(R, v3(__ldg(pb), __ldg(pb + 1), __ldg(pb + 2))) + T;
  }
  return tri_distance<double>(T1, T2, P, Q);
}

__device__ __forceinline__ double rss_distance64(const DevMesh& A, const DevMesh& B, int b1, int b2,
                                                 const M3<double>& R, const V3<double>& T) {
  M3<double> A1, A2;
  const double* x1 = A.rss64[b1].axis;
  const double* x2 = B.rss64[b2].axis;
#pragma unroll
  for (int i = 0; i < 9; ++i) {
    A1.m[i] = __ldg(x1 + i);
    A2.m[i] = __ldg(x2 + i);
  }
  const double* r1 = reinterpret_cast<const double*>(A.rss64 + b1);
  const double* r2 = reinterpret_cast<const double*>(B.rss64 + b2);
  const double l1[2] = {__ldg(r1 + 3), __ldg(r1 + 4)};
  const double l2[2] = {__ldg(r2 + 3), __ldg(r2 + 4)};
  return rss_distance<double>(R, T, A1, v3(__ldg(r1), __ldg(r1 + 1), __ldg(r1 + 2)), l1, __ldg(r1 + 5), A2,
                              v3(__ldg(r2), __ldg(r2 + 1), __ldg(r2 + 2)), l2, __ldg(r2 + 5));
}

__device__ __forceinline__ bool first_over_second(const DevMesh& A, const DevMesh& B, int b1, int b2, bool l1,
                                                  bool l2) {
  if (l2) return true;
  if (l1) return false;
  return size_key(A, b1) > size_key(B, b2);
}

// FCL's distance traversal in FP64 (the reference's operation order).
template <int STACK>
__device__ __noinline__ void distance_query_fp64(const DevMesh& A, const DevMesh& B, const M3<double>& R,
                                                 const V3<double>& T, DistOut& o) {
  o.nbv = o.nleaf = o.nrc = 0;
  o.status = 0;
  {
    V3<double> P, Q;
    const double d = leaf_distance64(A, B, 0, 0, R, T, P, Q);
    o.d = 1.7976931348623157e308;
    o.id1 = o.id2 = 0;
    o.P = o.Q = v3(0.0, 0.0, 0.0);
    if (o.d > d) {
      o.d = d;
      o.P = P;
      o.Q = Q;
    }
  }
  DStack stk[STACK];
  int sp = 0;
  int b1 = 0, b2 = 0;
  for (;;) {
    const int c1 = __ldg(&A.nodes64[b1].child), c2 = __ldg(&B.nodes64[b2].child);
    const bool l1 = c1 < 0, l2 = c2 < 0;
    bool descend = false;
    if (l1 && l2) {
      ++o.nleaf;
      const int p1 = -(c1 + 1), p2 = -(c2 + 1);
      V3<double> P, Q;
      const double d = leaf_distance64(A, B, p1, p2, R, T, P, Q);
      if (o.d > d) {
        o.d = d;
        o.id1 = p1;
        o.id2 = p2;
        o.P = P;
        o.Q = Q;
      }
    } else {
      int a1, a2, e1, e2;
      if (first_over_second(A, B, b1, b2, l1, l2)) {
        a1 = c1; a2 = b2; e1 = c1 + 1; e2 = b2;
      } else {
        a1 = b1; a2 = c2; e1 = b1; e2 = c2 + 1;
      }
      const double d1 = rss_distance64(A, B, a1, a2, R, T);
      const double d2 = rss_distance64(A, B, e1, e2, R, T);
      o.nbv += 2;
      if (sp >= STACK) {
        o.status |= DEV_ERR_STACK;
        break;
      }
      int f1, f2;
      double fd;
      if (d2 < d1) {
        stk[sp++] = DStack{a1, a2, d1};
        f1 = e1; f2 = e2; fd = d2;
      } else {
        stk[sp++] = DStack{e1, e2, d2};
        f1 = a1; f2 = a2; fd = d1;
      }
      if (!(fd >= o.d)) {  // !canStop(fd)
        b1 = f1;
        b2 = f2;
        descend = true;
      }
    }
    if (descend) continue;
    bool found = false;
    while (sp > 0) {
      const DStack e = stk[--sp];
      if (!(e.d >= o.d)) {
        b1 = e.b1;
        b2 = e.b2;
        found = true;
        break;
      }
    }
    if (!found) break;
  }
}

// Writes one query's result (witness points to world by tf1, the postprocess of
// mesh_distance_traversal_node-inl.h:589-603).
__device__ __forceinline__ void write_result(const DistanceLaunch& L, long long qi, const DistOut& o) {
  L.dist[qi] = o.d;
  if (L.ids) {
    L.ids[2 * qi] = o.id1;
    L.ids[2 * qi + 1] = o.id2;
  }
  if (L.nearest && L.points) {
    M3<double> R1;
    V3<double> t1;
    if (L.tf1) {
      const double* ta = L.tf1 + 12 * qi;
      for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) R1(r, c) = __ldg(ta + 4 * r + c);
      t1 = v3(__ldg(ta + 3), __ldg(ta + 7), __ldg(ta + 11));
    } else {
      for (int i = 0; i < 9; ++i) R1.m[i] = (i == 0 || i == 4 || i == 8) ? 1.0 : 0.0;
      t1 = v3(0.0, 0.0, 0.0);
    }
    const V3<double> w1 = mulv(R1, o.P) + t1;
    const V3<double> w2 = mulv(R1, o.Q) + t1;
    double* out = L.points + 6 * qi;
    out[0] = w1.x; out[1] = w1.y; out[2] = w1.z;
    out[3] = w2.x; out[4] = w2.y; out[5] = w2.z;
  }
  if (L.margins && L.within) L.within[qi] = (o.d <= __ldg(L.margins + qi)) ? 1 : 0;
  if (L.want_stats) {
    if (L.nbv) L.nbv[qi] = o.nbv;
    if (L.nleaf) L.nleaf[qi] = o.nleaf;
    if (L.nrecheck) L.nrecheck[qi] = o.nrc;
  }
}

// Pair index of query qi, or -1 (status set, result NaN) when it is out of range.
__device__ __forceinline__ int query_pair(const DistanceLaunch& L, long long qi) {
  const int pi = L.pair_of_query ? __ldg(L.pair_of_query + qi) : 0;
  if (pi < 0 || pi >= L.num_pairs) {
    atomicOr(&L.ctr->status, DEV_ERR_PAIR);
    L.dist[qi] = __longlong_as_double(0x7ff8000000000000ll);
    return -1;
  }
  return pi;
}

// The plain FP64 form: one query per thread, FCL's traversal.
template <int STACK>
__global__ void __launch_bounds__(128) k_mesh_distance(const DistanceLaunch L) {
  for (;;) {
    const long long qi = (long long)atomicAdd(&L.ctr->work, 1ull);
    if (qi >= L.n) break;
    const int pi = query_pair(L, qi);
    if (pi < 0) continue;
    const int2 mp = L.pairs[pi];
    const DevMesh A = L.meshes[mp.x];
    const DevMesh B = L.meshes[mp.y];
    double ta[12], tb[12];
    load_tfs(L, qi, ta, tb);
    M3<double> R;
    V3<double> T;
    rel_distance(ta, tb, R, T);
    DistOut o;
    distance_query_fp64<STACK>(A, B, R, T, o);
    if (o.status) atomicOr(&L.ctr->status, o.status);
    write_result(L, qi, o);
  }
}

// The certified FP32 form (distance_traverse.cuh).  Each lane owns one query at a
// time.  In every iteration of the warp loop the warp picks one phase and the lanes
// whose query is in that phase advance it by one step; __syncwarp() then brings the
// lanes back together.  Traversal steps run whenever lanes are traversing, except
// that once at least kBatch lanes wait for an FP64 triangle distance (or for the
// FP32 witness stage) those run first, so these long, FP64-heavy steps execute with
// many lanes at once.  A lane whose query ends fetches the next one.  Queries that
// the certified form does not take (DistCert::init) run the FP64 form in place.
// Capped at 128 registers: the FP64 leaf and fallback functions spill a little.
template <int STACK>
__global__ void __launch_bounds__(128, 4) k_mesh_distance_cert(const DistanceLaunch L) {
  constexpr int kBatch = 8;
  DistCert<STACK> c;
  long long qi = 0;
  auto start = [&]() -> bool {
    for (;;) {
      qi = (long long)atomicAdd(&L.ctr->work, 1ull);
      if (qi >= L.n) return false;
      const int pi = query_pair(L, qi);
      if (pi < 0) continue;
      const int2 mp = L.pairs[pi];
      double ta[12], tb[12];
      load_tfs(L, qi, ta, tb);
      M3<double> R;
      V3<double> T;
      rel_distance(ta, tb, R, T);
      if (c.init(L.meshes + mp.x, L.meshes + mp.y, R, T)) return true;
      DistOut o;
      distance_query_fp64<STACK>(L.meshes[mp.x], L.meshes[mp.y], R, T, o);
      if (o.status) atomicOr(&L.ctr->status, o.status);
      o.nrc = -1;  // marks an FP64 run
      write_result(L, qi, o);
    }
  };
  bool have = start();
  for (;;) {
    const int ph = have ? c.phase : DC_DONE;
    const unsigned mT = __ballot_sync(0xffffffffu, ph == DC_TRAVERSE);
    const unsigned mW = __ballot_sync(0xffffffffu, ph == DC_WITNESS);
    const unsigned mE = __ballot_sync(0xffffffffu, ph == DC_EXACT);
    if (!(mT | mW | mE)) break;
    int run;
    if (__popc(mE) >= kBatch || (mE && !mT && !mW))
      run = DC_EXACT;
    else if (__popc(mW) >= kBatch || (mW && !mT))
      run = DC_WITNESS;
    else
      run = DC_TRAVERSE;
    if (ph == run) {
      c.run_phase(run);
      if (c.phase == DC_DONE) {
        if (c.o.status) atomicOr(&L.ctr->status, c.o.status);
        write_result(L, qi, c.o);
        have = start();
      }
    }
    __syncwarp();
  }
}

// Distance values alone (no ids, witness points, margins or statistics), one warp per
// query, for batches too small to fill the GPU with one query per lane: the slowest
// query's serial traversal would set the batch's time.  FCL's distance is the
// smallest FP64 triDistance over the triangle pairs it visits, and a BV pair it prunes
// is at least its running minimum apart; with bounds that contain their triangles
// (DistCert::init refuses refitted meshes and rotations that are not orthonormal) it
// is the smallest over all triangle pairs, whatever the visit order.  The warp keeps a
// stack of BV pairs in shared memory and expands up to 32 a step with the certified
// bounds of distance_traverse.cuh (rss_pair_bound along the query direction and the
// pair's own centre line; tri_gap_bound, tri_witness_bound and tri_gap64 for triangle
// pairs, each with its derived error), pushes the children sorted by bound (nearest
// on top), and runs FCL's FP64 triDistance only for triangle pairs whose bound does
// not exceed the best distance so far by more than m64 (or lies within 2^-6 of their
// size, where triDistance may take its overlap branch).  Pairs with a zero distance end
// the query.  Queries that DistCert refuses get NaN here and run the FP64 form after
// (k_mesh_distance_redo), as do queries whose stack would outgrow shared memory.
constexpr int kDwWarps = 2;
constexpr long long kDistanceWarpMaxQueries = 65536;
constexpr int kDwFront = 1536;

__device__ __forceinline__ bool dw_less(float ka, int na, int pa, float kb, int nb, int pb) {
  return ka < kb || (ka == kb && (na < nb || (na == nb && pa < pb)));
}
// 64 entries held two per lane (entry e = lane + 32 * slot), sorted ascending by
// (bound, b1, b2) with a bitonic network
__device__ __forceinline__ void dw_sort64(float& k0, int& a0, int& c0, float& k1, int& a1, int& c1, int lane) {
  const unsigned full = 0xffffffffu;
#pragma unroll
  for (int k = 2; k <= 64; k <<= 1) {
#pragma unroll
    for (int j = k >> 1; j > 0; j >>= 1) {
      if (j == 32) {
        if (dw_less(k1, a1, c1, k0, a0, c0)) {
          const float tk = k0;
          const int ta = a0, tc = c0;
          k0 = k1;
          a0 = a1;
          c0 = c1;
          k1 = tk;
          a1 = ta;
          c1 = tc;
        }
        continue;
      }
#pragma unroll
      for (int slot = 0; slot < 2; ++slot) {
        float& kk = slot ? k1 : k0;
        int& aa = slot ? a1 : a0;
        int& cc = slot ? c1 : c0;
        const int e = lane + 32 * slot;
        const float pk = __shfl_xor_sync(full, kk, j);
        const int pa = __shfl_xor_sync(full, aa, j);
        const int pc = __shfl_xor_sync(full, cc, j);
        const bool up = (e & k) == 0, lower = (e & j) == 0;
        const bool p_first = dw_less(pk, pa, pc, kk, aa, cc);
        const bool take = lower ? (up ? p_first : !p_first) : (up ? !p_first : p_first);
        if (take) {
          kk = pk;
          aa = pa;
          cc = pc;
        }
      }
    }
  }
}

__global__ void __launch_bounds__(32 * kDwWarps) k_mesh_distance_warp(const DistanceLaunch L) {
  __shared__ int32_t fa[kDwWarps][kDwFront], fb[kDwWarps][kDwFront];
  __shared__ float fl[kDwWarps][kDwFront];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const long long qi = (long long)blockIdx.x * kDwWarps + w;
  if (qi >= L.n) return;
  const unsigned full = 0xffffffffu;
  const int pi = query_pair(L, qi);
  if (pi < 0) return;
  const int2 mp = L.pairs[pi];
  DistCert<1> c;  // set-up, direction and error terms only; the stack lives in shared memory
  {
    double ta[12], tb[12];
    load_tfs(L, qi, ta, tb);
    M3<double> R;
    V3<double> T;
    rel_distance(ta, tb, R, T);
    if (!c.init(L.meshes + mp.x, L.meshes + mp.y, R, T)) {
      if (lane == 0) L.dist[qi] = __longlong_as_double(0x7ff8000000000000ll);
      return;
    }
  }
  const DevMesh& A = *c.A;
  const DevMesh& B = *c.B;
  double best = 1.7976931348623157e308;
  V3<double> bP = v3(0.0, 0.0, 0.0), bQ = bP;
  if (lane == 0) {
    fa[w][0] = 0;
    fb[w][0] = 0;
    fl[w][0] = -1.f;
  }
  int size = 1;
  bool overflow = false;
  __syncwarp();
  while (size > 0) {
    const int take = size < 32 ? size : 32;
    int b1 = -1, b2 = -1;
    float lb = 0.f;
    if (lane < take) {
      b1 = fa[w][size - 1 - lane];
      b2 = fb[w][size - 1 - lane];
      lb = fl[w][size - 1 - lane];
    }
    size -= take;
    __syncwarp();
    if (b1 >= 0 && lb > c.best_up) b1 = -1;
    float k0 = CUDART_INF_F, k1 = CUDART_INF_F;
    int x0 = -1, y0 = -1, x1 = -1, y1 = -1;
    double d = 1.7976931348623157e308;
    V3<double> P, Q;
    if (b1 >= 0) {
      const int c1 = f2i_hd(ld4(A.nodes32, 4 * (long long)b1 + 3).w);
      const int c2 = f2i_hd(ld4(B.nodes32, 4 * (long long)b2 + 3).w);
      const bool l1 = c1 < 0, l2 = c2 < 0;
      if (l1 && l2) {
        const int p1 = -(c1 + 1), p2 = -(c2 + 1);
        float tsize;
        const float Lg = tri_gap_bound(A, B, p1, p2, c.dir, tsize);
        const float near = 0.015625f * tsize;
        if (!(Lg > fmaxf(c.best_up, near))) {
          float wv[3], l;
          const float Lw = tri_witness_bound(c.qf, A, B, p1, p2, wv, l);
          bool eval = !((double)Lw > c.not_better) || !(Lw > near);
          if (eval && Lw > near && best < 1.7976931348623157e308) {
            V3<double> pu, pv;
            bool vv;
            const double L64 = tri_gap64(A, B, p1, p2, c.R, c.T, wv, c.tau, pu, pv, vv);
            if (L64 > c.not_better)
              eval = false;
            else if (vv && same_point(pu, bP, c.vtol) && same_point(pv, bQ, c.vtol))
              eval = false;  // the best's own vertex pair: the same distance, not smaller
          }
          if (eval) d = leaf_distance64_hd(A, B, p1, p2, c.R, c.T, P, Q);
        }
      } else {
        const bool fos = l2 ? true : (l1 ? false : size_key(A, b1) > size_key(B, b2));
        int a1, a2, e1, e2;
        float L1, L2;
        if (fos) {
          a1 = c1; a2 = b2; e1 = c1 + 1; e2 = b2;
          const RssF rb = load_rss(B, b2);
          L1 = rss_pair_bound(load_rss(A, a1), rb, c.dir, c.qf, c.Ec0);
          L2 = rss_pair_bound(load_rss(A, e1), rb, c.dir, c.qf, c.Ec0);
        } else {
          a1 = b1; a2 = c2; e1 = b1; e2 = c2 + 1;
          const RssF ra = load_rss(A, b1);
          L1 = rss_pair_bound(ra, load_rss(B, a2), c.dir, c.qf, c.Ec0);
          L2 = rss_pair_bound(ra, load_rss(B, e2), c.dir, c.qf, c.Ec0);
        }
        if (!(L1 > c.best_up)) {
          k0 = L1;
          x0 = a1;
          y0 = a2;
        }
        if (!(L2 > c.best_up)) {
          k1 = L2;
          x1 = e1;
          y1 = e2;
        }
      }
    }
    // the step's smallest FP64 distance becomes the best, with its witness points
    double dm = d;
    for (int off = 16; off > 0; off >>= 1) dm = fmin(dm, __shfl_xor_sync(full, dm, off));
    if (dm < best) {
      const int win = __ffs(__ballot_sync(full, d == dm)) - 1;
      best = dm;
      bP = v3(__shfl_sync(full, P.x, win), __shfl_sync(full, P.y, win), __shfl_sync(full, P.z, win));
      bQ = v3(__shfl_sync(full, Q.x, win), __shfl_sync(full, Q.y, win), __shfl_sync(full, Q.z, win));
      if (best == 0.0) break;  // nothing is smaller
      c.best_up = (float)best * (1.f + 2.f * FCLG_U32) + c.m64;
      c.not_better = best + (double)c.m64;
      set_dist_dir(A, B, c.R, c.T, bQ.x - bP.x, bQ.y - bP.y, bQ.z - bP.z, c.dir);
    }
    if (k0 > c.best_up) x0 = -1, k0 = CUDART_INF_F;
    if (k1 > c.best_up) x1 = -1, k1 = CUDART_INF_F;
    const int np = __popc(__ballot_sync(full, x0 >= 0)) + __popc(__ballot_sync(full, x1 >= 0));
    if (np == 0) continue;
    if (size + np > kDwFront) {
      overflow = true;
      break;
    }
    dw_sort64(k0, x0, y0, k1, x1, y1, lane);
    if (lane < np) {
      fa[w][size + np - 1 - lane] = x0;
      fb[w][size + np - 1 - lane] = y0;
      fl[w][size + np - 1 - lane] = k0;
    }
    if (lane + 32 < np) {
      fa[w][size + np - 33 - lane] = x1;
      fb[w][size + np - 33 - lane] = y1;
      fl[w][size + np - 33 - lane] = k1;
    }
    size += np;
    __syncwarp();
  }
  // a stack that would overflow hands the query to the FP64 form as well
  if (lane == 0) L.dist[qi] = overflow ? __longlong_as_double(0x7ff8000000000000ll) : best;
}

// The FP64 form for the queries k_mesh_distance_warp left NaN.
template <int STACK>
__global__ void __launch_bounds__(128) k_mesh_distance_redo(const DistanceLaunch L) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long qi = (long long)blockIdx.x * blockDim.x + threadIdx.x; qi < L.n; qi += stride) {
    if (!isnan(L.dist[qi])) continue;
    const int pi = L.pair_of_query ? __ldg(L.pair_of_query + qi) : 0;
    if (pi < 0 || pi >= L.num_pairs) continue;  // status already set
    const int2 mp = L.pairs[pi];
    double ta[12], tb[12];
    load_tfs(L, qi, ta, tb);
    M3<double> R;
    V3<double> T;
    rel_distance(ta, tb, R, T);
    DistOut o;
    distance_query_fp64<STACK>(L.meshes[mp.x], L.meshes[mp.y], R, T, o);
    if (o.status) atomicOr(&L.ctr->status, o.status);
    L.dist[qi] = o.d;
  }
}

}  // namespace

cudaError_t launch_mesh_distance(const DistanceLaunch& L, int precision, int stack_entries, int grid, int block,
                                 cudaStream_t s) {
  ++g_kernel_launches;
  const bool values_only = !L.ids && !(L.nearest && L.points) && !(L.margins && L.within) && !L.want_stats;
  if (precision != 0 && values_only && L.n <= kDistanceWarpMaxQueries && stack_entries <= 64) {
    k_mesh_distance_warp<<<(unsigned)((L.n + kDwWarps - 1) / kDwWarps), 32 * kDwWarps, 0, s>>>(L);
    k_mesh_distance_redo<64><<<(unsigned)std::min<long long>((L.n + 127) / 128, 152 * 8), 128, 0, s>>>(L);
    ++g_kernel_launches;
    return cudaGetLastError();
  }
  if (precision == 0) {
    if (stack_entries <= 64)
      k_mesh_distance<64><<<grid, block, 0, s>>>(L);
    else
      k_mesh_distance<256><<<grid, block, 0, s>>>(L);
  } else {
    if (stack_entries <= 64)
      k_mesh_distance_cert<64><<<grid, block, 0, s>>>(L);
    else
      k_mesh_distance_cert<256><<<grid, block, 0, s>>>(L);
  }
  return cudaGetLastError();
}

int distance_grid(int precision, int stack_entries, int block) {
  int dev = 0, sms = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const void* k = precision == 0
                      ? (stack_entries <= 64 ? (const void*)k_mesh_distance<64> : (const void*)k_mesh_distance<256>)
                      : (stack_entries <= 64 ? (const void*)k_mesh_distance_cert<64>
                                             : (const void*)k_mesh_distance_cert<256>);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, block, 0);
  if (per_sm < 1) per_sm = 1;
  return sms * per_sm;
}

}  // namespace fclgpu
