// Batched BVHModel<OBBRSS> x BVHModel<OBBRSS> distance on the GPU.
//
// One thread runs one query.  The plain FP64 form (PREC 0) is FCL's distance
// traversal: preprocess with triangle 0 x triangle 0
// (mesh_distance_traversal_node-inl.h:545-586), then distanceRecurse
// (traversal_recurse-inl.h:257-316): RSS distance to both children of the larger
// node, nearer child first, a child skipped when canStop(d) = d >= min_distance
// (rel_err = abs_err = 0, :147-153), leaf = triDistance with DistanceResult's strict
// "<" update (distance_result-inl.h:84-105); nearest points mapped to world by tf1.
//
// The FP32 form (PREC 1) traverses with FP32 RSS bounds widened by a slack, keeps
// every leaf whose FP32 distance interval can still hold the minimum as a
// candidate, and finishes the candidates with the exact FP64 triangle distance in
// visit order (strict "<"), so the reported distance and witness points are the
// FP64 values of the winning triangle pair.
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
  const double* x1 = A.nodes64[b1].axis;
  const double* x2 = B.nodes64[b2].axis;
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

template <int STACK>
__global__ void __launch_bounds__(128) k_mesh_distance_fp64(const DistanceLaunch L) {
  for (;;) {
    const long long qi = (long long)atomicAdd(&L.ctr->work, 1ull);
    if (qi >= L.n) break;
    const int pi = L.pair_of_query ? __ldg(L.pair_of_query + qi) : 0;
    const int2 mp = L.pairs[pi];
    const DevMesh A = L.meshes[mp.x];
    const DevMesh B = L.meshes[mp.y];
    double ta[12], tb[12];
    load_tfs(L, qi, ta, tb);
    M3<double> R;
    V3<double> T;
    rel_distance(ta, tb, R, T);

    long long nbv = 0, nleaf = 0;
    // preprocess: triangle 0 x triangle 0
    V3<double> bestP, bestQ;
    double best;
    int id1 = 0, id2 = 0;
    {
      V3<double> P, Q;
      const double d = leaf_distance64(A, B, 0, 0, R, T, P, Q);
      best = 1.7976931348623157e308;
      if (best > d) {
        best = d;
        bestP = P;
        bestQ = Q;
      } else {
        bestP = bestQ = v3(0.0, 0.0, 0.0);
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
        ++nleaf;
        const int p1 = -(c1 + 1), p2 = -(c2 + 1);
        V3<double> P, Q;
        const double d = leaf_distance64(A, B, p1, p2, R, T, P, Q);
        if (best > d) {
          best = d;
          id1 = p1;
          id2 = p2;
          bestP = P;
          bestQ = Q;
        }
      } else {
        int a1, a2, e1, e2;
        bool fos;
        if (l2)
          fos = true;
        else if (l1)
          fos = false;
        else
          fos = __ldg(A.size64 + b1) > __ldg(B.size64 + b2);
        if (fos) {
          a1 = c1; a2 = b2; e1 = c1 + 1; e2 = b2;
        } else {
          a1 = b1; a2 = c2; e1 = b1; e2 = c2 + 1;
        }
        const double d1 = rss_distance64(A, B, a1, a2, R, T);
        const double d2 = rss_distance64(A, B, e1, e2, R, T);
        nbv += 2;
        if (sp >= STACK) {
          atomicOr(&L.ctr->status, DEV_ERR_STACK);
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
        if (!(fd >= best)) {  // !canStop(fd)
          b1 = f1;
          b2 = f2;
          descend = true;
        }
      }
      if (descend) continue;
      bool found = false;
      while (sp > 0) {
        const DStack e = stk[--sp];
        if (!(e.d >= best)) {
          b1 = e.b1;
          b2 = e.b2;
          found = true;
          break;
        }
      }
      if (!found) break;
    }
    L.dist[qi] = best;
    if (L.ids) {
      L.ids[2 * qi] = id1;
      L.ids[2 * qi + 1] = id2;
    }
    if (L.nearest && L.points) {
      // postprocess: world = tf1 * p
      M3<double> R1;
      for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) R1(r, c) = ta[4 * r + c];
      const V3<double> t1 = v3(ta[3], ta[7], ta[11]);
      const V3<double> w1 = mulv(R1, bestP) + t1;
      const V3<double> w2 = mulv(R1, bestQ) + t1;
      double* o = L.points + 6 * qi;
      o[0] = w1.x; o[1] = w1.y; o[2] = w1.z;
      o[3] = w2.x; o[4] = w2.y; o[5] = w2.z;
    }
    if (L.margins && L.within) L.within[qi] = (best <= __ldg(L.margins + qi)) ? 1 : 0;
    if (L.want_stats) {
      if (L.nbv) L.nbv[qi] = nbv;
      if (L.nleaf) L.nleaf[qi] = nleaf;
      if (L.nrecheck) L.nrecheck[qi] = 0;
    }
  }
}

}  // namespace

cudaError_t launch_mesh_distance(const DistanceLaunch& L, int precision, int stack_entries, int grid, int block,
                                 cudaStream_t s) {
  ++g_kernel_launches;
  (void)precision;
  if (stack_entries <= 64)
    k_mesh_distance_fp64<64><<<grid, block, 0, s>>>(L);
  else
    k_mesh_distance_fp64<256><<<grid, block, 0, s>>>(L);
  return cudaGetLastError();
}

int distance_grid(int precision, int stack_entries, int block) {
  (void)precision;
  int dev = 0, sms = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(
      &per_sm, stack_entries <= 64 ? (const void*)k_mesh_distance_fp64<64> : (const void*)k_mesh_distance_fp64<256>,
      block, 0);
  if (per_sm < 1) per_sm = 1;
  return sms * per_sm;
}

}  // namespace fclgpu
