// Continuous collision of mesh pairs, FCL's default solver: continuousCollideNaive
// (narrowphase/continuous_collision-inl.h:134-171) with the translation (default), linear
// or screw motion (math/motion/, motion.cuh).  FCL samples the motion at
// n_iter = min(num_max_iterations, ceil(1 / toc_err)) times t_i = i / (n_iter - 1) and
// returns the first t_i at which the discrete collide() (default request: one contact)
// reports a collision.
//
// On the device every (query, sample) pair becomes one query of the collide batch:
// k_ccd_poses writes the sampled transforms, the batch runs with num_max_contacts = 1,
// and k_ccd_reduce takes the first colliding sample of each query.  Samples after the
// first colliding one are evaluated although FCL would skip them; they change nothing.
#include <cuda_runtime.h>

#include "kernels.h"
#include "motion.cuh"

namespace fclgpu {

namespace {

__global__ void k_ccd_poses(CcdLaunch L) {
  const int64_t total = L.n * L.n_iter;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < total; k += stride) {
    const int64_t q = k / L.n_iter;
    const int64_t i = k - q * L.n_iter;
    const double t = (double)i / (double)(L.n_iter - 1);
    double a0[12], a1[12], b0[12], b1[12];
    for (int j = 0; j < 12; ++j) {
      if (L.tf1_beg) {
        a0[j] = __ldg(L.tf1_beg + 12 * q + j);
        a1[j] = __ldg(L.tf1_end + 12 * q + j);
      } else {
        a0[j] = a1[j] = (j == 0 || j == 5 || j == 10) ? 1.0 : 0.0;
      }
      b0[j] = __ldg(L.tf2_beg + 12 * q + j);
      b1[j] = __ldg(L.tf2_end + 12 * q + j);
    }
    motion_at(L.motion, a0, a1, t, L.tfa + 12 * k);
    motion_at(L.motion, b0, b1, t, L.tfb + 12 * k);
    L.pq_expanded[k] = L.pair_of_query ? __ldg(L.pair_of_query + q) : 0;
  }
}

__global__ void k_ccd_reduce(CcdLaunch L, const int32_t* counts) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < L.n; q += stride) {
    int64_t hit = -1;
    for (int64_t i = 0; i < L.n_iter; ++i)
      if (counts[q * L.n_iter + i] > 0) {
        hit = i;
        break;
      }
    L.is_collide[q] = hit >= 0 ? 1 : 0;
    L.toc[q] = hit >= 0 ? (double)hit / (double)(L.n_iter - 1) : 1.0;
    if (hit >= 0) {
      const int64_t k = q * L.n_iter + hit;
      if (L.contact_tf1)
        for (int j = 0; j < 12; ++j) L.contact_tf1[12 * q + j] = L.tfa[12 * k + j];
      if (L.contact_tf2)
        for (int j = 0; j < 12; ++j) L.contact_tf2[12 * q + j] = L.tfb[12 * k + j];
    }
  }
}

unsigned ccd_grid(int64_t items, int block) {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  int64_t g = (items + block - 1) / block;
  const int64_t cap = (int64_t)sms * 16;
  if (g > cap) g = cap;
  if (g < 1) g = 1;
  return (unsigned)g;
}

}  // namespace

cudaError_t launch_ccd_poses(const CcdLaunch& L, cudaStream_t s) {
  if (L.n <= 0 || L.n_iter <= 0) return cudaSuccess;
  k_ccd_poses<<<ccd_grid(L.n * L.n_iter, 128), 128, 0, s>>>(L);
  ++g_kernel_launches;
  return cudaGetLastError();
}

cudaError_t launch_ccd_reduce(const CcdLaunch& L, const int32_t* counts, cudaStream_t s) {
  if (L.n <= 0) return cudaSuccess;
  k_ccd_reduce<<<ccd_grid(L.n, 256), 256, 0, s>>>(L, counts);
  ++g_kernel_launches;
  return cudaGetLastError();
}

}  // namespace fclgpu
