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
// Work-splitting rounds.  Items [item_lo, item_hi) run with a BV-test budget; an
// item that exhausts it writes its frontier as child items (contiguous ids, DFS
// order) for the next round.
// ---------------------------------------------------------------------------------
struct SplitSink : ContactSink {
  int4* items;
  long long item_cap;
  unsigned long long* item_ctr;
  int32_t* child_start;
  int32_t* child_count;
  bool dumped;

  __device__ __forceinline__ void dump(long long item, long long qi, int2 cur, const int2* stk, int sp) {
    const int k = 1 + sp;
    const long long b = (long long)atomicAdd(item_ctr, (unsigned long long)k);
    if (b + k > item_cap || b + k > 0x7fffffffll) {
      atomicOr(status, DEV_ERR_ITEMS);
      return;
    }
    items[b] = make_int4((int)qi, cur.x, cur.y, 0);
    for (int j = 0; j < sp; ++j) {
      const int2 e = stk[sp - 1 - j];
      items[b + 1 + j] = make_int4((int)qi, e.x, e.y, 0);
    }
    child_start[item] = (int32_t)b;
    child_count[item] = k;
    dumped = true;
  }
};

template <int PREC, int STACK>
__global__ void __launch_bounds__(128) k_collide_round(const CollideLaunch L) {
  SplitSink sink;
  sink.rec = L.records;
  sink.cap = L.record_cap;
  sink.ctr = &L.ctr->records;
  sink.status = &L.ctr->status;
  sink.base = -1;
  sink.used = 0;
  sink.items = L.items;
  sink.item_cap = L.item_cap;
  sink.item_ctr = &L.ctr->items;
  sink.child_start = L.child_start;
  sink.child_count = L.child_count;
  const long long span = L.item_hi - L.item_lo;
  for (;;) {
    const long long k = (long long)atomicAdd(&L.ctr->work, 1ull);
    if (k >= span) break;
    const long long item = L.item_lo + k;
    long long qi;
    int b1, b2;
    if (item < L.n) {
      qi = item;
      b1 = b2 = 0;
    } else {
      const int4 it = L.items[item];
      qi = it.x;
      b1 = it.y;
      b2 = it.z;
    }
    sink.dumped = false;
    QueryStats st;
    const int ncont = collide_item<PREC, STACK>(L, qi, b1, b2, item, L.budget, L.num_max_contacts, sink, st);
    if (st.status) atomicOr(&L.ctr->status, st.status);
    L.own[item] = ncont;
    if (!sink.dumped) L.child_count[item] = 0;
    if (L.want_stats) {
      if (L.nbv) atomicAdd((unsigned long long*)(L.nbv + qi), (unsigned long long)st.nbv);
      if (L.nleaf) atomicAdd((unsigned long long*)(L.nleaf + qi), (unsigned long long)st.nleaf);
      if (L.nrecheck) atomicAdd((unsigned long long*)(L.nrecheck + qi), (unsigned long long)st.nrecheck);
    }
  }
  sink.flush();
}

// total[i] = own[i] + sum of the totals of its children (children are in a later
// round, whose totals are already known when rounds are processed last to first).
__global__ void k_item_totals(const CollideLaunch L, long long lo, long long hi, long long* total) {
  const long long i = lo + (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= hi) return;
  long long t = L.own[i];
  const int c = L.child_count[i];
  if (c > 0) {
    const long long s = L.child_start[i];
    for (int j = 0; j < c; ++j) t += total[s + j];
  }
  total[i] = t;
}

__global__ void k_item_counts(const CollideLaunch L, const long long* total, int32_t* capped,
                              unsigned long long* ncapped) {
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= L.n) return;
  const long long t = total[q];
  const long long m = L.num_max_contacts;
  L.counts[q] = (int32_t)(t < m ? t : m);
  if (t >= m && L.child_count[q] > 0 && capped) {
    const unsigned long long k = atomicAdd(ncapped, 1ull);
    capped[k] = (int32_t)q;
  }
}

// rel_start of the children of round items [lo, hi): the position of the child's
// first contact inside its query's DFS-order contact list.
__global__ void k_item_starts(const CollideLaunch L, long long lo, long long hi, const long long* total,
                              long long* rel_start) {
  const long long i = lo + (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= hi) return;
  if (i < L.n) rel_start[i] = 0;
  const int c = L.child_count[i];
  if (c <= 0) return;
  long long run = rel_start[i] + L.own[i];
  const long long s = L.child_start[i];
  for (int j = 0; j < c; ++j) {
    rel_start[s + j] = run;
    run += total[s + j];
  }
}

__global__ void __launch_bounds__(256) k_scatter_items(const CollideLaunch L, long long nrec,
                                                       const long long* rel_start, const long long* offsets,
                                                       int32_t* contacts) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < nrec; i += stride) {
    const int4 r = L.records[i];
    if (r.x < 0) continue;
    const long long item = r.x;
    const long long q = item < L.n ? item : (long long)L.items[item].x;
    const long long pos = rel_start[item] + r.y;
    if (pos >= L.num_max_contacts) continue;
    reinterpret_cast<int2*>(contacts)[offsets[q] + pos] = make_int2(r.z, r.w);
  }
}

struct NullSink {
  FCLG_HD void push(int, int, int, int) {}
};

template <int PREC, int STACK>
__global__ void __launch_bounds__(128) k_collide_stats(const CollideLaunch L, const int32_t* list, long long nlist) {
  NullSink sink;
  for (;;) {
    const long long k = (long long)atomicAdd(&L.ctr->work, 1ull);
    if (k >= nlist) break;
    const long long qi = list[k];
    QueryStats st;
    collide_query<PREC, STACK>(L, qi, sink, st);
    if (L.nbv) L.nbv[qi] = st.nbv;
    if (L.nleaf) L.nleaf[qi] = st.nleaf;
    if (L.nrecheck) L.nrecheck[qi] = st.nrecheck;
  }
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

cudaError_t launch_collide_round(const CollideLaunch& L, int precision, int stack_entries, int grid, int block,
                                 cudaStream_t s) {
  ++g_kernel_launches;
  if (precision == 0) {
    if (stack_entries <= 64)
      k_collide_round<0, 64><<<grid, block, 0, s>>>(L);
    else
      k_collide_round<0, 256><<<grid, block, 0, s>>>(L);
  } else {
    if (stack_entries <= 64)
      k_collide_round<1, 64><<<grid, block, 0, s>>>(L);
    else
      k_collide_round<1, 256><<<grid, block, 0, s>>>(L);
  }
  return cudaGetLastError();
}

cudaError_t launch_item_totals(const CollideLaunch& L, int64_t lo, int64_t hi, int64_t* total, cudaStream_t s) {
  if (hi <= lo) return cudaSuccess;
  const long long nb = (hi - lo + 255) / 256;
  k_item_totals<<<(unsigned)nb, 256, 0, s>>>(L, lo, hi, reinterpret_cast<long long*>(total));
  ++g_kernel_launches;
  return cudaGetLastError();
}

cudaError_t launch_item_counts(const CollideLaunch& L, const int64_t* total, int32_t* capped, cudaStream_t s) {
  if (L.n <= 0) return cudaSuccess;
  const long long nb = (L.n + 255) / 256;
  k_item_counts<<<(unsigned)nb, 256, 0, s>>>(L, reinterpret_cast<const long long*>(total), capped,
                                             &L.ctr->capped_split);
  ++g_kernel_launches;
  return cudaGetLastError();
}

cudaError_t launch_item_starts(const CollideLaunch& L, int64_t lo, int64_t hi, const int64_t* total,
                               int64_t* rel_start, cudaStream_t s) {
  if (hi <= lo) return cudaSuccess;
  const long long nb = (hi - lo + 255) / 256;
  k_item_starts<<<(unsigned)nb, 256, 0, s>>>(L, lo, hi, reinterpret_cast<const long long*>(total),
                                             reinterpret_cast<long long*>(rel_start));
  ++g_kernel_launches;
  return cudaGetLastError();
}

cudaError_t launch_scatter_items(const CollideLaunch& L, int64_t nrec, const int64_t* rel_start,
                                 const int64_t* offsets, int32_t* contacts, cudaStream_t s) {
  if (nrec <= 0) return cudaSuccess;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  long long blocks = (nrec + 255) / 256;
  if (blocks > (long long)sms * 8) blocks = (long long)sms * 8;
  k_scatter_items<<<(unsigned)blocks, 256, 0, s>>>(L, nrec, reinterpret_cast<const long long*>(rel_start),
                                                   reinterpret_cast<const long long*>(offsets), contacts);
  ++g_kernel_launches;
  return cudaGetLastError();
}

cudaError_t launch_collide_stats(const CollideLaunch& L, const int32_t* list, int64_t nlist, int precision,
                                 int stack_entries, cudaStream_t s) {
  if (nlist <= 0) return cudaSuccess;
  const int grid = collide_grid(precision, stack_entries, 128);
  ++g_kernel_launches;
  if (precision == 0) {
    if (stack_entries <= 64)
      k_collide_stats<0, 64><<<grid, 128, 0, s>>>(L, list, nlist);
    else
      k_collide_stats<0, 256><<<grid, 128, 0, s>>>(L, list, nlist);
  } else {
    if (stack_entries <= 64)
      k_collide_stats<1, 64><<<grid, 128, 0, s>>>(L, list, nlist);
    else
      k_collide_stats<1, 256><<<grid, 128, 0, s>>>(L, list, nlist);
  }
  return cudaGetLastError();
}

int collide_round_grid(int precision, int stack_entries, int block) {
  int dev = 0, sms = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const void* k;
  if (precision == 0)
    k = stack_entries <= 64 ? (const void*)k_collide_round<0, 64> : (const void*)k_collide_round<0, 256>;
  else
    k = stack_entries <= 64 ? (const void*)k_collide_round<1, 64> : (const void*)k_collide_round<1, 256>;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, block, 0);
  if (per_sm < 1) per_sm = 1;
  return sms * per_sm;
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
