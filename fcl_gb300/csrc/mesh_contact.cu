// Contact information of a mesh-mesh collide batch with CollisionRequest::enable_contact
// = true (mesh_collision_traversal_node-inl.h:579-600).  FCL's traversal with contacts
// visits the same BV and triangle pairs in the same order as without; only the leaf
// differs: an intersecting triangle pair adds 0, 1 or 2 contacts (each with a world
// position, the world normal and the penetration depth), no more than num_max_contacts
// minus the contacts already held, and the traversal stops once num_max_contacts
// contacts exist.  So the batch runs in three passes over the intersecting triangle
// pairs that the pair traversal lists in FCL's DFS order:
//
//   k_contact_info    one thread per listed pair: its contacts (tri_contact.cuh, FP64);
//   k_contact_counts  one thread per query: contacts = min(sum over its pairs, max), and
//                     a flag when the pair list was cut at its cap before the query held
//                     num_max_contacts contacts (a pair with no contact point: the list
//                     is then re-run with a larger cap);
//   k_contact_emit    one thread per listed pair: its contacts, truncated where the
//                     query's running total reaches num_max_contacts, written at the
//                     query's output offset.
#include <cuda_runtime.h>

#include "kernels.h"
#include "tri_contact.cuh"

namespace fclgpu {

namespace {

__device__ __forceinline__ V3<double> vtx64(const double* V, int i) {
  return v3<double>(__ldg(V + 3 * i), __ldg(V + 3 * i + 1), __ldg(V + 3 * i + 2));
}

// largest q in [0, n) with off[q] <= j (off has n + 1 entries, off[n] > j)
__device__ __forceinline__ int64_t query_of_pair(const int64_t* off, int64_t n, int64_t j) {
  int64_t lo = 0, hi = n - 1;
  while (lo < hi) {
    const int64_t mid = (lo + hi + 1) >> 1;
    if (__ldg(reinterpret_cast<const long long*>(off) + mid) <= (long long)j)
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}

__global__ void k_contact_info(ContactLaunch L) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < L.npairs; j += stride) {
    const int64_t qi = query_of_pair(L.poff, L.n, j);
    L.qid[j] = (int32_t)qi;
    const int pi = L.pair_of_query ? __ldg(L.pair_of_query + qi) : 0;
    const int2 mp = L.pairs[pi];
    const DevMesh A = L.meshes[mp.x];
    const DevMesh B = L.meshes[mp.y];
    double ta[12], tb[12];
    if (L.tf1) {
      for (int k = 0; k < 12; ++k) ta[k] = __ldg(L.tf1 + 12 * qi + k);
    } else {
      for (int k = 0; k < 12; ++k) ta[k] = (k == 0 || k == 5 || k == 10) ? 1.0 : 0.0;
    }
    for (int k = 0; k < 12; ++k) tb[k] = __ldg(L.tf2 + 12 * qi + k);
    M3<double> R;
    V3<double> T;
    rel_collide(ta, tb, R, T);
    const int2 pr = L.plist[j];
    V3<double> P[3], Q[3];
    for (int k = 0; k < 3; ++k) {
      P[k] = vtx64(A.verts64, __ldg(A.tris + 3 * (int64_t)pr.x + k));
      Q[k] = vtx64(B.verts64, __ldg(B.tris + 3 * (int64_t)pr.y + k));
    }
    TriContact c;
    tri_contact_world(P, Q, R, T, ta, c);
    L.nc[j] = c.n;
    double* o = L.info + 10 * j;
    for (int i = 0; i < 2; ++i)
      for (int k = 0; k < 3; ++k) o[3 * i + k] = c.pos[i][k];
    for (int k = 0; k < 3; ++k) o[6 + k] = c.normal[k];
    o[9] = c.depth;
  }
}

__global__ void k_contact_counts(ContactLaunch L, const int32_t* pair_counts, int32_t* counts,
                                 unsigned int* incomplete) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < L.n; q += stride) {
    const int64_t a = L.poff[q], b = L.poff[q + 1];
    const int64_t tot = L.G[b] - L.G[a];
    counts[q] = (int32_t)(tot < L.max_contacts ? tot : L.max_contacts);
    if (pair_counts[q] >= L.pair_cap && tot < L.max_contacts) atomicAdd(incomplete, 1u);
  }
}

__global__ void k_contact_emit(ContactLaunch L, const int64_t* out_off, int32_t* ids, double* pos, double* normal,
                               double* depth) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < L.npairs; j += stride) {
    const int nc = L.nc[j];
    if (nc == 0) continue;
    const int64_t qi = L.qid[j];
    const int64_t before = L.G[j] - L.G[L.poff[qi]];
    const int64_t room = (int64_t)L.max_contacts - before;
    if (room <= 0) continue;
    const int m = (int64_t)nc < room ? nc : (int)room;
    const int64_t base = out_off[qi] + before;
    const int2 pr = L.plist[j];
    const double* in = L.info + 10 * j;
    for (int t = 0; t < m; ++t) {
      const int64_t o = base + t;
      if (ids) {
        ids[2 * o] = pr.x;
        ids[2 * o + 1] = pr.y;
      }
      if (pos)
        for (int k = 0; k < 3; ++k) pos[3 * o + k] = in[3 * t + k];
      if (normal)
        for (int k = 0; k < 3; ++k) normal[3 * o + k] = in[6 + k];
      if (depth) depth[o] = in[9];
    }
  }
}

unsigned grid_for(int64_t items, int block) {
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

cudaError_t launch_contact_info(const ContactLaunch& L, cudaStream_t s) {
  if (L.npairs <= 0) return cudaSuccess;
  k_contact_info<<<grid_for(L.npairs, 128), 128, 0, s>>>(L);
  ++g_kernel_launches;
  return cudaGetLastError();
}

cudaError_t launch_contact_counts(const ContactLaunch& L, const int32_t* pair_counts, int32_t* counts,
                                  unsigned int* incomplete, cudaStream_t s) {
  if (L.n <= 0) return cudaSuccess;
  k_contact_counts<<<grid_for(L.n, 256), 256, 0, s>>>(L, pair_counts, counts, incomplete);
  ++g_kernel_launches;
  return cudaGetLastError();
}

cudaError_t launch_contact_emit(const ContactLaunch& L, const int64_t* out_off, int32_t* ids, double* pos,
                                double* normal, double* depth, cudaStream_t s) {
  if (L.npairs <= 0) return cudaSuccess;
  k_contact_emit<<<grid_for(L.npairs, 256), 256, 0, s>>>(L, out_off, ids, pos, normal, depth);
  ++g_kernel_launches;
  return cudaGetLastError();
}

}  // namespace fclgpu
