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
// The FP32 form (PREC 1) traverses with FP32 RSS distances widened by a slack
// (2^-12 relative + 64u times the coordinate scale) as pruning lower bounds, and FP32
// triangle distances (points taken relative to the first vertex, offset in
// float-float) with a slack E = 2^-18 d + 128u times the pair's coordinate scale.  A
// leaf whose FP32 interval can still reach the best distance so far -- and every
// leaf near contact, where triDistance switches branches -- is re-evaluated at once
// with the exact FP64 triangle distance and the strict "<" update, in visit order,
// so the reported distance, triangle ids and witness points are FP64 values of the
// winning pair, and the pruning bound is the exact best.
#include "filter32.cuh"
#include "geom.cuh"
#include "kernels.h"

namespace fclgpu {

namespace {

struct DStack {
  int b1, b2;
  double d;
};
struct FStack {
  int b1, b2;
  float d;
};

struct DistOut {
  double d;
  int id1, id2;
  V3<double> P, Q;  // first mesh's frame
  long long nbv, nleaf, nrc;
  unsigned status;
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

// ---------------------------------------------------------------------------------
// FP32 form helpers
// ---------------------------------------------------------------------------------

// Triangle pair in FP32, both relative to triangle 1's first vertex (Q moved by R,T).
__device__ __forceinline__ float tri_distance_f32(const QueryF32& q, const float4* ta, const float4* tb,
                                                  float& scale) {
  const float4 x0 = __ldg(ta), x1 = __ldg(ta + 1), x2 = __ldg(ta + 2);
  const float4 y0 = __ldg(tb), y1 = __ldg(tb + 1), y2 = __ldg(tb + 2);
  const float Ph[3] = {x0.x, x0.y, x0.z}, Pl[3] = {x0.w, x1.x, x1.y};
  const float Qh[3] = {y0.x, y0.y, y0.z}, Ql[3] = {y0.w, y1.x, y1.y};
  float D[3];
#pragma unroll
  for (int r = 0; r < 3; ++r) {
    float hi, lo;
    two_sum(q.T[r], -Ph[r], hi, lo);
    lo += q.Tl[r] - Pl[r];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const float Rh = q.R[3 * r + k], Rlo = q.Rl[3 * r + k];
      const float p = Rh * Qh[k];
      const float pe = fmaf(Rh, Qh[k], -p) + fmaf(Rh, Ql[k], Rlo * Qh[k]);
      float s, e;
      two_sum(hi, p, s, e);
      hi = s;
      lo += e + pe;
    }
    D[r] = hi + lo;
  }
  const F3 dq2 = rot3(q.R, f3(y1.z, y1.w, y2.x));
  const F3 dq3 = rot3(q.R, f3(y2.y, y2.z, y2.w));
  V3<float> T1[3], T2[3];
  T1[0] = v3(0.f, 0.f, 0.f);
  T1[1] = v3(x1.z, x1.w, x2.x);
  T1[2] = v3(x2.y, x2.z, x2.w);
  T2[0] = v3(D[0], D[1], D[2]);
  T2[1] = v3(D[0] + dq2.x, D[1] + dq2.y, D[2] + dq2.z);
  T2[2] = v3(D[0] + dq3.x, D[1] + dq3.y, D[2] + dq3.z);
  float l = 0.f;
#pragma unroll
  for (int k = 0; k < 3; ++k)
    l = fmaxf(l, fmaxf(fmaxf(fabsf(T1[k].x), fabsf(T1[k].y)), fmaxf(fmaxf(fabsf(T1[k].z), fabsf(T2[k].x)),
                                                                      fmaxf(fabsf(T2[k].y), fabsf(T2[k].z)))));
  scale = l;
  V3<float> P, Q;
  return tri_distance<float>(T1, T2, P, Q);
}

__device__ __forceinline__ float rss_distance_f32(const QueryF32& q, const DevMesh& A, const DevMesh& B, int b1,
                                                  int b2) {
  const float4* ra = reinterpret_cast<const float4*>(A.rss32) + 5 * (long long)b1;
  const float4* rb = reinterpret_cast<const float4*>(B.rss32) + 5 * (long long)b2;
  M3<float> A1, A2, R0;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const float4 ca = __ldg(ra + 2 + k), cb = __ldg(rb + 2 + k);
    A1(0, k) = ca.x; A1(1, k) = ca.y; A1(2, k) = ca.z;
    A2(0, k) = cb.x; A2(1, k) = cb.y; A2(2, k) = cb.z;
  }
#pragma unroll
  for (int i = 0; i < 9; ++i) R0.m[i] = q.R[i];
  const float4 r1a = __ldg(ra), r1b = __ldg(ra + 1), r2a = __ldg(rb), r2b = __ldg(rb + 1);
  const float l1[2] = {r1b.x, r1b.y}, l2[2] = {r2b.x, r2b.y};
  return rss_distance<float>(R0, v3(q.T[0], q.T[1], q.T[2]), A1, v3(r1a.x, r1a.y, r1a.z), l1, r1a.w, A2,
                             v3(r2a.x, r2a.y, r2a.z), l2, r2a.w);
}

template <int STACK>
__global__ void __launch_bounds__(128) k_mesh_distance(const DistanceLaunch L, int prec) {
  for (;;) {
    const long long qi = (long long)atomicAdd(&L.ctr->work, 1ull);
    if (qi >= L.n) break;
    const int pi = L.pair_of_query ? __ldg(L.pair_of_query + qi) : 0;
    if (pi < 0 || pi >= L.num_pairs) {  // reported through the status word, query left NaN
      atomicOr(&L.ctr->status, DEV_ERR_PAIR);
      L.dist[qi] = __longlong_as_double(0x7ff8000000000000ll);
      continue;
    }
    const int2 mp = L.pairs[pi];
    const DevMesh A = L.meshes[mp.x];
    const DevMesh B = L.meshes[mp.y];
    double ta[12], tb[12];
    load_tfs(L, qi, ta, tb);
    M3<double> R;
    V3<double> T;
    rel_distance(ta, tb, R, T);
    DistOut o;
    bool exact = (prec == 0);
    if (!exact) {
      QueryF32 qf;
      make_query_f32(R, T, A.rmax, B.rmax, A.vmax, B.vmax, qf);
      const float u = FCLG_U32;
      const float tau = fmaxf(fabsf(qf.T[0]), fmaxf(fabsf(qf.T[1]), fabsf(qf.T[2])));
      const float rss_abs = 64.f * u * (float)(A.rmax + B.rmax) + 64.f * u * 1.7321f * tau;
      const float rel = 3.814697265625e-6f;  // 2^-18 of the distance
      long long nbv = 0, nleaf = 0, nrc64 = 0;
      // exact FP64 best so far (strict "<" in visit order, as DistanceResult::update);
      // best_up is a float upper bound of it used for pruning
      o.d = 1.7976931348623157e308;
      o.id1 = o.id2 = 0;
      o.P = o.Q = v3(0.0, 0.0, 0.0);
      float best_up = 3.0e38f;
      auto exact_leaf = [&](int p1, int p2) {
        V3<double> P, Q;
        const double d64 = leaf_distance64(A, B, p1, p2, R, T, P, Q);
        ++nrc64;
        if (o.d > d64) {
          o.d = d64;
          o.id1 = p1;
          o.id2 = p2;
          o.P = P;
          o.Q = Q;
          best_up = (float)d64 * (1.f + 2.f * u) + 1e-37f;
        }
      };
      // preprocess pair (triangle 0, triangle 0)
      exact_leaf(0, 0);
      FStack stk[STACK];
      int sp = 0;
      int b1 = 0, b2 = 0;
      for (;;) {
        const int c1 = __float_as_int(__ldg(reinterpret_cast<const float4*>(A.nodes32) + 4 * (long long)b1 + 3).w);
        const int c2 = __float_as_int(__ldg(reinterpret_cast<const float4*>(B.nodes32) + 4 * (long long)b2 + 3).w);
        const bool l1 = c1 < 0, l2 = c2 < 0;
        bool descend = false;
        if (l1 && l2) {
          ++nleaf;
          const int p1 = -(c1 + 1), p2 = -(c2 + 1);
          float sc;
          const float d = tri_distance_f32(qf, reinterpret_cast<const float4*>(A.tri32) + 3 * (long long)p1,
                                           reinterpret_cast<const float4*>(B.tri32) + 3 * (long long)p2, sc);
          const float E = rel * d + 128.f * u * sc + qf.dabs * 2.f;
          // near contact triDistance switches between its edge/face and overlap
          // branches, so such pairs always take the exact value; otherwise only a
          // pair whose FP32 interval can still reach the best is re-evaluated
          if (d <= 3.90625e-3f * sc || d - E <= best_up) exact_leaf(p1, p2);
        } else {
          int a1, a2, e1, e2;
          if (first_over_second(A, B, b1, b2, l1, l2)) {
            a1 = c1; a2 = b2; e1 = c1 + 1; e2 = b2;
          } else {
            a1 = b1; a2 = c2; e1 = b1; e2 = c2 + 1;
          }
          float d1 = rss_distance_f32(qf, A, B, a1, a2);
          float d2 = rss_distance_f32(qf, A, B, e1, e2);
          d1 = d1 - (2.44140625e-4f * d1 + rss_abs);
          d2 = d2 - (2.44140625e-4f * d2 + rss_abs);
          nbv += 2;
          if (sp >= STACK) {
            atomicOr(&L.ctr->status, DEV_ERR_STACK);
            break;
          }
          int f1, f2;
          float fd;
          if (d2 < d1) {
            stk[sp++] = FStack{a1, a2, d1};
            f1 = e1; f2 = e2; fd = d2;
          } else {
            stk[sp++] = FStack{e1, e2, d2};
            f1 = a1; f2 = a2; fd = d1;
          }
          if (!(fd > best_up)) {
            b1 = f1;
            b2 = f2;
            descend = true;
          }
        }
        if (descend) continue;
        bool found = false;
        while (sp > 0) {
          const FStack e = stk[--sp];
          if (!(e.d > best_up)) {
            b1 = e.b1;
            b2 = e.b2;
            found = true;
            break;
          }
        }
        if (!found) break;
      }
      o.nbv = nbv;
      o.nleaf = nleaf;
      o.nrc = nrc64;
      o.status = 0;
    }
    if (exact) {
      distance_query_fp64<STACK>(A, B, R, T, o);
      if (o.status) atomicOr(&L.ctr->status, o.status);
      if (prec != 0) o.nrc = -1;  // marks an FP64 re-run
    }
    L.dist[qi] = o.d;
    if (L.ids) {
      L.ids[2 * qi] = o.id1;
      L.ids[2 * qi + 1] = o.id2;
    }
    if (L.nearest && L.points) {
      M3<double> R1;
      for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) R1(r, c) = ta[4 * r + c];
      const V3<double> t1 = v3(ta[3], ta[7], ta[11]);
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
}

}  // namespace

cudaError_t launch_mesh_distance(const DistanceLaunch& L, int precision, int stack_entries, int grid, int block,
                                 cudaStream_t s) {
  ++g_kernel_launches;
  if (stack_entries <= 64)
    k_mesh_distance<64><<<grid, block, 0, s>>>(L, precision);
  else
    k_mesh_distance<256><<<grid, block, 0, s>>>(L, precision);
  return cudaGetLastError();
}

int distance_grid(int precision, int stack_entries, int block) {
  (void)precision;
  int dev = 0, sms = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(
      &per_sm, stack_entries <= 64 ? (const void*)k_mesh_distance<64> : (const void*)k_mesh_distance<256>, block, 0);
  if (per_sm < 1) per_sm = 1;
  return sms * per_sm;
}

}  // namespace fclgpu
