// Batched convex shape-pair collide + distance (GJKSolver_indep semantics).
//
// Per pair: fcl::collide with contact (closed form where GJKSolver_indep has one,
// gjk_solver_indep-inl.h:242-262, else GJK + EPA, :111-166); if the pair does not
// collide, fcl::distance (closed form where registered, :710-860, else GJK,
// :593-645).  Box-box intersection is the closed form boxBoxIntersect with the
// deepest contact point (num_max_contacts = 1).  One thread per pair, FP64, reference
// operation order; EPA state lives in thread-local memory and is only touched by
// colliding pairs.
#include "shape_pair.cuh"
#include "shapes.h"

namespace fclgpu {

double g_last_shape_ms = -1.0;

namespace {

__global__ void __launch_bounds__(128) k_shape_batch(ShapeLaunch L) {
  for (;;) {
    const long long q = (long long)atomicAdd(&L.ctr->work, 1ull);
    if (q >= L.n) break;
    PairOut o;
    shape_pair_query(L.shapes[__ldg(L.ia + q)], L.shapes[__ldg(L.ib + q)], L.verts, L.tf1 + 12 * q, L.tf2 + 12 * q, o);
    L.hit[q] = o.hit;
    double* nr = L.normal + 3 * q;
    double* pt = L.point + 3 * q;
    double* w1 = L.p1 + 3 * q;
    double* w2 = L.p2 + 3 * q;
    nr[0] = o.normal.x; nr[1] = o.normal.y; nr[2] = o.normal.z;
    pt[0] = o.point.x; pt[1] = o.point.y; pt[2] = o.point.z;
    w1[0] = o.p1.x; w1[1] = o.p1.y; w1[2] = o.p1.z;
    w2[0] = o.p2.x; w2[1] = o.p2.y; w2[2] = o.p2.z;
    L.depth[q] = o.depth;
    L.dist[q] = o.dist;
    if (L.status) {
      L.status[2 * q] = o.gstat;
      L.status[2 * q + 1] = o.estat;
    }
  }
}

}  // namespace

cudaError_t launch_shape_batch(const ShapeLaunch& L, int grid, int block, cudaStream_t s) {
  ++g_kernel_launches;
  k_shape_batch<<<grid, block, 0, s>>>(L);
  return cudaGetLastError();
}

int shape_grid(int block) {
  int dev = 0, sms = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, (const void*)k_shape_batch, block, 0);
  if (per_sm < 1) per_sm = 1;
  return sms * per_sm;
}

}  // namespace fclgpu
