// Batched convex shape-pair collide + distance (GJKSolver_indep semantics).
//
// Per pair: fcl::collide with contact (closed form where GJKSolver_indep has one,
// gjk_solver_indep-inl.h:242-262, else GJK + EPA, :111-166); if the pair does not
// collide, fcl::distance (closed form where registered, :710-860, else GJK,
// :593-645).  Box-box intersection is the closed form boxBoxIntersect with the
// deepest contact point (num_max_contacts = 1).  FP64, reference operation order.
//
// The batch runs in stages so that the lanes of a warp execute the same code: the
// pairs are bucketed by their (type, type) combination (a counting sort), then
//   1. intersect, in bucket order: closed forms, or the FP32-certified GJK; a GJK that
//      ends Inside is marked for EPA and appended to a list;
//   2. EPA (recomputing that GJK, deterministic) over the list only;
//   3. distance, in bucket order, for the pairs that do not collide.
// The EPA state (the largest per-thread state) lives only in stage 2.
#include <algorithm>

#include "shape_pair.cuh"
#include "shapes.h"

namespace fclgpu {

double g_last_shape_ms = -1.0;

namespace {

constexpr int kKeys = 64;  // (type_a, type_b), 8 x 8

__device__ __forceinline__ int pair_key(const ShapeLaunch& L, long long q) {
  return (L.shapes[__ldg(L.ia + q)].type & 7) * 8 + (L.shapes[__ldg(L.ib + q)].type & 7);
}

__global__ void k_shape_hist(ShapeLaunch L, unsigned* bins) {
  __shared__ unsigned h[kKeys];
  for (int k = threadIdx.x; k < kKeys; k += blockDim.x) h[k] = 0;
  __syncthreads();
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < L.n; q += stride)
    atomicAdd(&h[pair_key(L, q)], 1u);
  __syncthreads();
  for (int k = threadIdx.x; k < kKeys; k += blockDim.x)
    if (h[k]) atomicAdd(&bins[k], h[k]);
}

// one block of kKeys threads: bins -> exclusive starts (the scatter cursors)
__global__ void k_shape_starts(unsigned* bins) {
  __shared__ unsigned v[kKeys];
  const int k = threadIdx.x;
  v[k] = bins[k];
  __syncthreads();
  if (k == 0) {
    unsigned run = 0;
    for (int i = 0; i < kKeys; ++i) {
      const unsigned c = v[i];
      v[i] = run;
      run += c;
    }
  }
  __syncthreads();
  bins[k] = v[k];
}

__global__ void k_shape_scatter(ShapeLaunch L, unsigned* cursor) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < L.n; q += stride)
    L.order[atomicAdd(&cursor[pair_key(L, q)], 1u)] = (int32_t)q;
}

__device__ __forceinline__ void store3(double* p, const D3v& v) {
  p[0] = v.x;
  p[1] = v.y;
  p[2] = v.z;
}

__global__ void __launch_bounds__(128) k_shape_intersect(ShapeLaunch L) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < L.n; t += stride) {
    const long long q = L.order[t];
    PairOut o;
    shape_pair_query(L.shapes[__ldg(L.ia + q)], L.shapes[__ldg(L.ib + q)], L.verts, L.tf1 + 12 * q, L.tf2 + 12 * q, o,
                     PAIR_INTERSECT | PAIR_DEFER_EPA);
    L.hit[q] = o.hit;
    store3(L.normal + 3 * q, o.normal);
    store3(L.point + 3 * q, o.point);
    L.depth[q] = o.depth;
    L.dist[q] = -1;
    store3(L.p1 + 3 * q, v3(0.0, 0.0, 0.0));
    store3(L.p2 + 3 * q, v3(0.0, 0.0, 0.0));
    if (L.status) {
      L.status[2 * q] = o.gstat;
      L.status[2 * q + 1] = o.estat;
    }
    if (o.estat == kEpaPending) L.epa_list[atomicAdd(L.epa_count, 1ull)] = (int32_t)q;
  }
}

__global__ void __launch_bounds__(128) k_shape_epa(ShapeLaunch L) {
  const long long n = (long long)*L.epa_count;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += stride) {
    const long long q = L.epa_list[t];
    PairOut o;
    shape_pair_query(L.shapes[__ldg(L.ia + q)], L.shapes[__ldg(L.ib + q)], L.verts, L.tf1 + 12 * q, L.tf2 + 12 * q, o,
                     PAIR_INTERSECT);
    L.hit[q] = o.hit;
    store3(L.normal + 3 * q, o.normal);
    store3(L.point + 3 * q, o.point);
    L.depth[q] = o.depth;
    if (L.status) {
      L.status[2 * q] = o.gstat;
      L.status[2 * q + 1] = o.estat;
    }
  }
}

// Distance for the separated pairs, in bucket order, with lane refill: a lane whose GJK
// ends writes its result and takes the next pair at once (a closed-form pair is done
// in the same pass), so the lanes of a warp stay in the GJK iteration together instead
// of idling until the warp's slowest pair ends.  The distance GJK's status replaces the
// intersect's, as fcl::collide then fcl::distance on one solver; closed-form distances
// leave it.
__global__ void __launch_bounds__(128) k_shape_distance(ShapeLaunch L, unsigned long long* next) {
  SimplexVert V[4];
  GjkState g;
  M3<double> R1;
  D3v t1;
  long long q = -1;
  bool has = false, exhausted = false;
  for (;;) {
    if (!has && !exhausted) {
      const long long t = (long long)atomicAdd(next, 1ull);
      if (t >= L.n) {
        exhausted = true;
      } else {
        q = L.order[t];
        if (!L.hit[q]) {
          const DevShape sa = L.shapes[__ldg(L.ia + q)], sb = L.shapes[__ldg(L.ib + q)];
          if (distance_uses_gjk(sa.type, sb.type)) {
            ShapeRef A, B;
            A.s = sa;
            B.s = sb;
            A.verts = B.verts = L.verts;
            M3<double> R2;
            D3v t2;
            load_tf(L.tf1 + 12 * q, R1, t1);
            load_tf(L.tf2 + 12 * q, R2, t2);
            gjk_distance_begin(A, R1, t1, B, R2, t2, V, g);
            has = true;
          } else {
            PairOut o;
            shape_pair_query(sa, sb, L.verts, L.tf1 + 12 * q, L.tf2 + 12 * q, o, PAIR_DISTANCE);
            L.dist[q] = o.dist;
            store3(L.p1 + 3 * q, o.p1);
            store3(L.p2 + 3 * q, o.p2);
          }
        }
      }
    }
    if (__all_sync(0xffffffffu, exhausted && !has)) break;
    if (has && g.step()) {
      PairOut o;
      o.p1 = o.p2 = v3(0.0, 0.0, 0.0);
      gjk_distance_end(g, R1, t1, o);
      L.dist[q] = o.dist;
      store3(L.p1 + 3 * q, o.p1);
      store3(L.p2 + 3 * q, o.p2);
      if (L.status) L.status[2 * q] = o.gstat;
      has = false;
    }
  }
}

int grid_of(const void* kernel, int block, long long n) {
  int dev = 0, sms = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, block, 0);
  if (per_sm < 1) per_sm = 1;
  const long long want = (n + block - 1) / block;
  return (int)std::max<long long>(1, std::min<long long>(want, (long long)sms * per_sm));
}

__global__ void __launch_bounds__(128) k_shape_collide_only(ShapeLaunch L) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < L.n; q += stride) {
    PairOut o;
    shape_pair_query(L.shapes[__ldg(L.ia + q)], L.shapes[__ldg(L.ib + q)], L.verts, L.tf1 + 12 * q, L.tf2 + 12 * q, o,
                     PAIR_INTERSECT | PAIR_NO_CONTACT);
    L.hit[q] = o.hit;
  }
}

}  // namespace

cudaError_t launch_shape_collide_only(const ShapeLaunch& L, cudaStream_t s) {
  const cudaError_t ep = upload_solver_params(s);
  if (ep != cudaSuccess) return ep;
  k_shape_collide_only<<<grid_of((const void*)k_shape_collide_only, 128, L.n), 128, 0, s>>>(L);
  ++g_kernel_launches;
  return cudaGetLastError();
}

cudaError_t launch_shape_batch(const ShapeLaunch& L, unsigned* bins, cudaStream_t s) {
  const int block = 128;
  cudaError_t e;
  if ((e = upload_solver_params(s))) return e;
  if ((e = cudaMemsetAsync(bins, 0, sizeof(unsigned) * kKeys, s))) return e;
  if ((e = cudaMemsetAsync(L.epa_count, 0, sizeof(unsigned long long), s))) return e;
  k_shape_hist<<<grid_of((const void*)k_shape_hist, 256, L.n), 256, 0, s>>>(L, bins);
  k_shape_starts<<<1, kKeys, 0, s>>>(bins);
  k_shape_scatter<<<grid_of((const void*)k_shape_scatter, 256, L.n), 256, 0, s>>>(L, bins);
  k_shape_intersect<<<grid_of((const void*)k_shape_intersect, block, L.n), block, 0, s>>>(L);
  k_shape_epa<<<grid_of((const void*)k_shape_epa, block, L.n), block, 0, s>>>(L);
  unsigned long long* next = L.epa_count + 1;
  if ((e = cudaMemsetAsync(next, 0, sizeof(unsigned long long), s))) return e;
  k_shape_distance<<<grid_of((const void*)k_shape_distance, block, L.n), block, 0, s>>>(L, next);
  g_kernel_launches += 6;
  return cudaGetLastError();
}

}  // namespace fclgpu
