// Batched BVHModel<OBBRSS> x BVHModel<OBBRSS> collide on the GPU.
//
// One thread runs one query (mesh pair + pose) as an explicit-stack depth-first
// traversal that visits BV pairs in exactly the order of FCL's collisionRecurse
// (narrowphase/detail/traversal/traversal_recurse-inl.h:82-129): test the pair,
// descend into the larger node first (firstOverSecond,
// bvh_collision_traversal_node-inl.h:77-89), stop as soon as
// num_max_contacts contacts are found (canStop, collision_request-inl.h:76-82).
// Threads fetch queries from a device work counter until the batch is drained
// (persistent launch), so very uneven query costs balance across the GPU.
//
// Precision forms:
//   PREC 0 (plain FP64) reads the FP64 node mirror and evaluates every test exactly
//          as the reference does;
//   PREC 1 (FP32 + recheck) reads the packed FP32 store and evaluates the filtered
//          predicates of filter32.cuh; an uncertain decision re-runs the exact FP64
//          test on the FP64 mirror.  Decisions -- hence contact sets, contact order
//          and traversal statistics -- equal PREC 0's bit for bit.
// Contacts go to per-thread chunks of a record scratch (query, rank, b1, b2); a scan
// of the per-query counts and a scatter kernel then lay them out query by query.
#include "collide_traverse.cuh"

namespace fclgpu {

int64_t g_kernel_launches = 0;

namespace {

constexpr int kChunk = 16;

struct ContactSink {
  int4* rec;
  long long cap;
  unsigned long long* ctr;
  unsigned int* status;
  long long base;
  int used;

  __device__ __forceinline__ void push(int q, int rank, int b1, int b2) {
    if (base < 0 || used == kChunk) {
      base = (long long)atomicAdd(ctr, (unsigned long long)kChunk);
      used = 0;
    }
    const long long pos = base + used++;
    if (pos < cap)
      rec[pos] = make_int4(q, rank, b1, b2);
    else
      atomicOr(status, DEV_ERR_RECORDS);
  }
  __device__ __forceinline__ void flush() {
    if (base < 0) return;
    for (; used < kChunk; ++used) {
      const long long pos = base + used;
      if (pos < cap) rec[pos] = make_int4(-1, 0, 0, 0);
    }
  }
};

template <int PREC, int STACK>
__global__ void __launch_bounds__(128) k_mesh_collide(const CollideLaunch L) {
  ContactSink sink{L.records, L.record_cap, &L.ctr->records, &L.ctr->status, -1, 0};
  for (;;) {
    const long long qi = (long long)atomicAdd(&L.ctr->work, 1ull);
    if (qi >= L.n) break;
    QueryStats st;
    const int ncont = collide_query<PREC, STACK>(L, qi, sink, st);
    if (st.status) atomicOr(&L.ctr->status, st.status);
    L.counts[qi] = ncont;
    if (L.want_stats) {
      if (L.nbv) L.nbv[qi] = st.nbv;
      if (L.nleaf) L.nleaf[qi] = st.nleaf;
      if (L.nrecheck) L.nrecheck[qi] = st.nrecheck;
    }
  }
  sink.flush();
}

// ---------------------------------------------------------------------------------
// Exclusive scan of int32 counts into int64 offsets (three passes over 4096-tiles).
// ---------------------------------------------------------------------------------
constexpr int kScanBlock = 1024;
constexpr int kScanTile = 4096;

__device__ __forceinline__ long long block_exclusive_scan(long long v, long long* sh, long long& total) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  long long x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const long long y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) sh[wid] = x;
  __syncthreads();
  if (wid == 0) {
    long long w = (lane < (int)(blockDim.x >> 5)) ? sh[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const long long y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    sh[lane] = w;
  }
  __syncthreads();
  const long long warp_prefix = (wid > 0) ? sh[wid - 1] : 0;
  total = sh[(blockDim.x >> 5) - 1];
  __syncthreads();
  return warp_prefix + x - v;
}

__global__ void __launch_bounds__(kScanBlock) k_scan_tiles(const int32_t* counts, long long n, long long* tile_sums) {
  __shared__ long long sh[32];
  const long long base = (long long)blockIdx.x * kScanTile + 4ll * threadIdx.x;
  long long s = 0;
#pragma unroll
  for (int k = 0; k < 4; ++k)
    if (base + k < n) s += counts[base + k];
  long long total;
  block_exclusive_scan(s, sh, total);
  if (threadIdx.x == 0) tile_sums[blockIdx.x] = total;
}

__global__ void __launch_bounds__(kScanBlock) k_scan_sums(long long* tile_sums, long long ntiles, long long* grand) {
  __shared__ long long sh[32];
  long long carry = 0;
  for (long long base = 0; base < ntiles; base += kScanBlock) {
    const long long i = base + threadIdx.x;
    const long long v = (i < ntiles) ? tile_sums[i] : 0;
    long long total;
    const long long ex = block_exclusive_scan(v, sh, total);
    if (i < ntiles) tile_sums[i] = carry + ex;
    carry += total;
  }
  if (threadIdx.x == 0) *grand = carry;
}

__global__ void __launch_bounds__(kScanBlock) k_scan_apply(const int32_t* counts, long long n,
                                                           const long long* tile_sums, long long* offsets) {
  __shared__ long long sh[32];
  const long long base = (long long)blockIdx.x * kScanTile + 4ll * threadIdx.x;
  long long v[4];
  long long s = 0;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    v[k] = (base + k < n) ? counts[base + k] : 0;
    s += v[k];
  }
  long long total;
  long long ex = block_exclusive_scan(s, sh, total) + tile_sums[blockIdx.x];
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    if (base + k < n) offsets[base + k] = ex;
    ex += v[k];
  }
}

__global__ void k_set_last(long long* offsets, long long n, const long long* grand) { offsets[n] = *grand; }

__global__ void __launch_bounds__(256) k_scatter_contacts(const int4* rec, long long nrec, const long long* offsets,
                                                          int32_t* contacts) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < nrec; i += stride) {
    const int4 r = rec[i];
    if (r.x < 0) continue;
    const long long o = offsets[r.x] + r.y;
    reinterpret_cast<int2*>(contacts)[o] = make_int2(r.z, r.w);
  }
}

}  // namespace

cudaError_t launch_mesh_collide(const CollideLaunch& L, int precision, int stack_entries, int grid, int block,
                                cudaStream_t s) {
  ++g_kernel_launches;
  if (precision == 0) {
    if (stack_entries <= 64)
      k_mesh_collide<0, 64><<<grid, block, 0, s>>>(L);
    else
      k_mesh_collide<0, 256><<<grid, block, 0, s>>>(L);
  } else {
    if (stack_entries <= 64)
      k_mesh_collide<1, 64><<<grid, block, 0, s>>>(L);
    else
      k_mesh_collide<1, 256><<<grid, block, 0, s>>>(L);
  }
  return cudaGetLastError();
}

cudaError_t launch_exclusive_scan(const int32_t* counts, int64_t n, int64_t* offsets, int64_t* tmp, cudaStream_t s) {
  const long long ntiles = (n + kScanTile - 1) / kScanTile;
  long long* tiles = reinterpret_cast<long long*>(tmp);
  long long* grand = tiles + ntiles + 1;
  long long* off = reinterpret_cast<long long*>(offsets);
  if (ntiles > 0) {
    k_scan_tiles<<<(unsigned)ntiles, kScanBlock, 0, s>>>(counts, n, tiles);
    k_scan_sums<<<1, kScanBlock, 0, s>>>(tiles, ntiles, grand);
    k_scan_apply<<<(unsigned)ntiles, kScanBlock, 0, s>>>(counts, n, tiles, off);
    g_kernel_launches += 3;
  } else {
    cudaMemsetAsync(grand, 0, sizeof(long long), s);
  }
  k_set_last<<<1, 1, 0, s>>>(off, n, grand);
  ++g_kernel_launches;
  return cudaGetLastError();
}

cudaError_t launch_scatter_contacts(const int4* records, int64_t nrec, const int64_t* offsets, int32_t* contacts,
                                    cudaStream_t s) {
  if (nrec <= 0) return cudaSuccess;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  long long blocks = (nrec + 255) / 256;
  const long long cap = (long long)sms * 8;
  if (blocks > cap) blocks = cap;
  k_scatter_contacts<<<(unsigned)blocks, 256, 0, s>>>(records, nrec, reinterpret_cast<const long long*>(offsets),
                                                      contacts);
  ++g_kernel_launches;
  return cudaGetLastError();
}

int collide_grid(int precision, int stack_entries, int block) {
  int dev = 0, sms = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const void* k;
  if (precision == 0)
    k = stack_entries <= 64 ? (const void*)k_mesh_collide<0, 64> : (const void*)k_mesh_collide<0, 256>;
  else
    k = stack_entries <= 64 ? (const void*)k_mesh_collide<1, 64> : (const void*)k_mesh_collide<1, 256>;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, block, 0);
  if (per_sm < 1) per_sm = 1;
  return sms * per_sm;
}

}  // namespace fclgpu
