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

// One round over items [lo, hi): threads fetch items from the work counter until it
// passes hi.  Items of this round were written by other blocks in the previous round of
// a persistent launch, so they are read past L1 (__ldcg).
template <int PREC, int STACK>
__device__ __forceinline__ void collide_round_body(const CollideLaunch& L, long long lo, long long hi) {
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
  const long long span = hi - lo;
  for (;;) {
    const long long k = (long long)atomicAdd(&L.ctr->work, 1ull);
    if (k >= span) break;
    const long long item = lo + k;
    long long qi;
    int b1, b2;
    if (item < L.n) {
      qi = item;
      b1 = b2 = 0;
    } else {
      const int4 it = __ldcg(L.items + item);
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

template <int PREC, int STACK>
__global__ void __launch_bounds__(128) k_collide_round(const CollideLaunch L) {
  collide_round_body<PREC, STACK>(L, L.item_lo, L.item_hi);
}

// ---------------------------------------------------------------------------------
// FP32 form with warp-batched leaf tests.  Each lane runs its item's DFS (BV tests,
// the common case), but a leaf pair whose boxes overlap is not tested at once: it
// goes to the warp's queue in shared memory, and whenever 32 are queued all lanes test
// one each.  Without the queue nearly every warp step carried some lane's leaf test
// (about one step in eleven is a leaf for each lane) and the other 31 lanes waited.
// A lane's queued leaves keep its DFS order, so the contact ranks it receives are its
// DFS-order ranks.  A lane learns of its contacts only when its leaves are tested, so
// an item capped at num_max_contacts can run past FCL's stop point: the extra contacts
// land past the cap and are dropped by the assembly, and such queries take their
// statistics from the exact serial pass.
// ---------------------------------------------------------------------------------
constexpr int kWbWarps = 4;
constexpr int kWbQueue = 64;  // >= 31 left over + 32 appended in one step

struct WbCtx {
  QueryF32 qf;
  const float4* tri_a;
  const float4* tri_b;
  long long qi;
  long long item;
  int pair;
  int ncont;    // contacts recorded for the lane's item
  int pending;  // queued leaf pairs of the lane's item
  int nrecheck;
};

struct WbShared {
  WbCtx ctx[kWbWarps][32];
  int3 queue[kWbWarps][kWbQueue];
};

template <int STACK>
__device__ __forceinline__ void collide_round_wb_body(const CollideLaunch& L, long long lo, long long hi,
                                                      WbShared& sh) {
  WbCtx (&ctx)[kWbWarps][32] = sh.ctx;
  int3 (&queue)[kWbWarps][kWbQueue] = sh.queue;
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const unsigned full = 0xffffffffu;
  const unsigned lt = (1u << lane) - 1u;
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
  const long long span = hi - lo;
  WbCtx& me = ctx[w][lane];

  bool have = false, draining = false, exhausted = false, dumped = false;
  long long item = 0, qi = 0;
  int b1 = 0, b2 = 0, sp = 0;
  int2 stk[STACK];
  long long nbv = 0, nleaf = 0;
  DevMesh A, B;
  QueryF32 qf;
  M3<double> R;
  V3<double> T;
  int qn = 0;  // queue length (the same in every lane)

  for (;;) {
    // (a) a free lane takes the next item
    if (!have && !draining && !exhausted) {
      const long long k = (long long)atomicAdd(&L.ctr->work, 1ull);
      if (k >= span) {
        exhausted = true;
      } else {
        item = lo + k;
        if (item < L.n) {
          qi = item;
          b1 = b2 = 0;
        } else {
          const int4 it = __ldcg(L.items + item);
          qi = it.x;
          b1 = it.y;
          b2 = it.z;
        }
        const int pi = L.pair_of_query ? L.pair_of_query[qi] : 0;
        const int2 mp = L.pairs[pi];
        A = L.meshes[mp.x];
        B = L.meshes[mp.y];
        double ta[12];
        query_transform_collide(L.tf1, L.tf2, qi, R, T, ta);
        make_query_f32(R, T, A.cmax, B.cmax, A.vmax, B.vmax, qf);
        me.qf = qf;
        me.tri_a = reinterpret_cast<const float4*>(A.tri32);
        me.tri_b = reinterpret_cast<const float4*>(B.tri32);
        me.qi = qi;
        me.item = item;
        me.pair = pi;
        me.ncont = 0;
        me.pending = 0;
        me.nrecheck = 0;
        sp = 0;
        nbv = nleaf = 0;
        dumped = false;
        have = L.num_max_contacts > 0;
        draining = !have;
      }
    }
    // (b) up to kWbSteps DFS steps; stop at the first leaf pair to queue
    bool produced = false;
    int3 entry = make_int3(lane, 0, 0);
    for (int step = 0; step < L.wb_steps && have && !produced; ++step) {
      if (me.ncont >= L.num_max_contacts) {  // canStop (known contacts)
        have = false;
        draining = true;
        break;
      }
      if (nbv >= L.budget) {
        sink.dumped = false;
        sink.dump(item, qi, make_int2(b1, b2), stk, sp);
        dumped = sink.dumped;
        have = false;
        draining = true;
        break;
      }
      const float4* pa = reinterpret_cast<const float4*>(A.nodes32) + 4 * (long long)b1;
      const float4* pb = reinterpret_cast<const float4*>(B.nodes32) + 4 * (long long)b2;
      const float4 a0 = __ldg(pa), a1 = __ldg(pa + 1), a2 = __ldg(pa + 2), ea = __ldg(pa + 3);
      const float4 x0 = __ldg(pb), x1 = __ldg(pb + 1), x2 = __ldg(pb + 2), eb = __ldg(pb + 3);
      const int c1 = __float_as_int(ea.w), c2 = __float_as_int(eb.w);
      int r = obb_overlap_f32(qf, a0, a1, a2, ea, x0, x1, x2, eb);
      if (r == F_UNSURE) {
        ++me.nrecheck;
        r = bv_overlap64(A, B, b1, b2, R, T) ? F_TRUE : F_FALSE;
      }
      ++nbv;
      bool next_from_stack = true;
      if (r == F_TRUE) {
        const bool l1 = c1 < 0, l2 = c2 < 0;
        if (l1 && l2) {
          ++nleaf;
          produced = true;
          entry = make_int3(lane, -(c1 + 1), -(c2 + 1));
        } else {
          const bool first_over_second = l2 ? true : (l1 ? false : size_key(A, b1) > size_key(B, b2));
          if (sp >= STACK || (L.stack_limit > 0 && sp >= L.stack_limit)) {
            atomicOr(&L.ctr->status, DEV_ERR_STACK);
            have = false;
            draining = true;
            break;
          }
          if (first_over_second) {
            stk[sp++] = make_int2(c1 + 1, b2);
            b1 = c1;
          } else {
            stk[sp++] = make_int2(b1, c2 + 1);
            b2 = c2;
          }
          next_from_stack = false;
        }
      }
      if (next_from_stack) {
        if (sp == 0) {
          have = false;
          draining = true;
        } else {
          const int2 e = stk[--sp];
          b1 = e.x;
          b2 = e.y;
        }
      }
    }
    // (c) queue the leaf pairs found in this step, in lane order
    const unsigned pm = __ballot_sync(full, produced);
    if (produced) {
      queue[w][qn + __popc(pm & lt)] = entry;
      ++me.pending;
    }
    qn += __popc(pm);
    __syncwarp();
    // (d) test queued leaves: in batches of 32, and whatever is left once no lane can
    // produce more before its queued leaves are known
    const unsigned running = __ballot_sync(full, have);
    while (qn >= 32 || (qn > 0 && running == 0)) {
      const int cnt = qn < 32 ? qn : 32;
      const bool mine = lane < cnt;
      const int3 e = mine ? queue[w][lane] : make_int3(-1 - lane, 0, 0);
      bool hit = false;
      if (mine) {
        const WbCtx& o = ctx[w][e.x];
        const float4* ta4 = o.tri_a + 3 * (long long)e.y;
        const float4* tb4 = o.tri_b + 3 * (long long)e.z;
        int r = tri_intersect_f32(o.qf, __ldg(ta4), __ldg(ta4 + 1), __ldg(ta4 + 2), __ldg(tb4), __ldg(tb4 + 1),
                                  __ldg(tb4 + 2));
        if (r == F_UNSURE) {
          atomicAdd(&ctx[w][e.x].nrecheck, 1);
          const int2 mp = L.pairs[o.pair];
          M3<double> Ro;
          V3<double> To;
          double ta[12];
          query_transform_collide(L.tf1, L.tf2, o.qi, Ro, To, ta);
          r = leaf_collide64(L.meshes[mp.x], L.meshes[mp.y], e.y, e.z, Ro, To) ? F_TRUE : F_FALSE;
        }
        hit = (r == F_TRUE);
      }
      const unsigned hm = __ballot_sync(full, hit);
      const unsigned peers = __match_any_sync(full, e.x);
      if (hit) {
        const int rank = ctx[w][e.x].ncont + __popc(peers & hm & lt);
        sink.push((int)ctx[w][e.x].item, rank, e.y, e.z);
      }
      __syncwarp();
      if (mine && (peers & lt) == 0) {  // the first lane of each owner's group
        ctx[w][e.x].ncont += __popc(peers & hm);
        ctx[w][e.x].pending -= __popc(peers);
      }
      // drop the tested entries
      int3 rest = make_int3(0, 0, 0);
      const bool keep = lane < qn - cnt;
      if (keep) rest = queue[w][cnt + lane];
      __syncwarp();
      if (keep) queue[w][lane] = rest;
      qn -= cnt;
      __syncwarp();
    }
    // (e) a lane whose item ended and whose leaves are all tested records the item
    if (draining && me.pending == 0) {
      L.own[item] = me.ncont;
      if (!dumped) L.child_count[item] = 0;
      if (L.want_stats) {
        if (L.nbv) atomicAdd((unsigned long long*)(L.nbv + qi), (unsigned long long)nbv);
        if (L.nleaf) atomicAdd((unsigned long long*)(L.nleaf + qi), (unsigned long long)nleaf);
        if (L.nrecheck) atomicAdd((unsigned long long*)(L.nrecheck + qi), (unsigned long long)me.nrecheck);
      }
      draining = false;
    }
    __syncwarp();
    if (__all_sync(full, exhausted && !have && !draining) && qn == 0) break;
  }
  sink.flush();
}

// MINB: blocks per SM the register allocation targets (1 = no limit, 158 registers;
// 4 = 128 registers with a few spills); the autotuner picks the faster.
template <int STACK, int MINB>
__global__ void __launch_bounds__(128, MINB) k_collide_round_wb(const CollideLaunch L) {
  __shared__ WbShared sh;
  collide_round_wb_body<STACK>(L, L.item_lo, L.item_hi, sh);
}

// ---------------------------------------------------------------------------------
// Persistent form: all rounds in one cooperative launch.  Between rounds the grid meets
// at a barrier; block 0 then records the round's item range, moves the range on to the
// items the round appended and clears the work counter, and the grid meets again.  The
// barrier's wait is bounded (PersistCtl::timeout_ns): a block that gives up sets
// DEV_ERR_BARRIER and returns, the others give up at their next barrier, and the host
// runs the batch again one launch per round.
// ---------------------------------------------------------------------------------
__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ bool grid_barrier(PersistCtl* c) {
  __shared__ int ok_s;
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile unsigned* vgen = &c->gen;
    const unsigned g = *vgen;
    __threadfence();
    const unsigned a = atomicAdd(&c->arrive, 1u);
    int ok = 1;
    if (a + 1 == c->nblocks) {
      atomicExch(&c->arrive, 0u);
      __threadfence();
      atomicAdd(&c->gen, 1u);
    } else {
      ok = 0;
      const unsigned long long t0 = global_ns();
      for (unsigned long long it = 0; it < kBarrierMaxSpins; ++it) {
        if (*vgen != g) {
          ok = 1;
          break;
        }
        __nanosleep(256);
        if ((it & 63) == 63 && global_ns() - t0 > c->timeout_ns) break;
      }
      if (!ok) atomicOr(&c->err, DEV_ERR_BARRIER);
    }
    __threadfence();
    ok_s = ok;
  }
  __syncthreads();
  return ok_s != 0;
}

template <int PREC, int STACK, bool WB>
__device__ __forceinline__ void run_round(const CollideLaunch& L, long long lo, long long hi) {
  if constexpr (WB) {
    __shared__ WbShared sh;
    collide_round_wb_body<STACK>(L, lo, hi, sh);
  } else {
    collide_round_body<PREC, STACK>(L, lo, hi);
  }
}

template <int PREC, int STACK, int MINB, bool WB>
__global__ void __launch_bounds__(128, MINB) k_collide_persist(const CollideLaunch L, PersistCtl* ctl,
                                                                long long* table) {
  volatile PersistCtl* vc = ctl;
  for (unsigned r = 0;; ++r) {
    const long long lo = (long long)vc->lo, hi = (long long)vc->hi;
    if (vc->stop || lo >= hi) break;
    run_round<PREC, STACK, WB>(L, lo, hi);
    if (!grid_barrier(ctl)) return;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      table[2 * r] = lo;
      table[2 * r + 1] = hi;
      const unsigned st = atomicOr(&L.ctr->status, 0u);
      const unsigned long long items = atomicAdd(&L.ctr->items, 0ull);
      atomicExch(&L.ctr->work, 0ull);
      vc->nrounds = r + 1;
      vc->lo = (unsigned long long)hi;
      vc->hi = items;
      if ((st & (DEV_ERR_STACK | DEV_ERR_RECORDS | DEV_ERR_ITEMS)) || r + 1 >= vc->max_rounds) vc->stop = 1;
      __threadfence();
    }
    if (!grid_barrier(ctl)) return;
  }
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
  // a capped query may have run past FCL's stop point (split across items, or its
  // leaf tests batched after further BV tests): its statistics need the serial pass
  if (t >= m && capped) {
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
  } else if (L.wb_variant == 1) {
    if (stack_entries <= 64)
      k_collide_round_wb<64, 4><<<grid, 32 * kWbWarps, 0, s>>>(L);
    else
      k_collide_round_wb<256, 4><<<grid, 32 * kWbWarps, 0, s>>>(L);
  } else {
    if (stack_entries <= 64)
      k_collide_round_wb<64, 1><<<grid, 32 * kWbWarps, 0, s>>>(L);
    else
      k_collide_round_wb<256, 1><<<grid, 32 * kWbWarps, 0, s>>>(L);
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

namespace {
// the persistent kernel of a configuration: FP64 form, or the FP32 warp-batched form
// in its register variant
const void* persist_kernel(int precision, int stack_entries, int variant) {
  const bool small = stack_entries <= 64;
  if (precision == 0)
    return small ? (const void*)k_collide_persist<0, 64, 1, false> : (const void*)k_collide_persist<0, 256, 1, false>;
  if (variant == 1)
    return small ? (const void*)k_collide_persist<1, 64, 4, true> : (const void*)k_collide_persist<1, 256, 4, true>;
  return small ? (const void*)k_collide_persist<1, 64, 1, true> : (const void*)k_collide_persist<1, 256, 1, true>;
}
}  // namespace

int collide_persistent_grid(int precision, int stack_entries, int variant) {
  int dev = 0, sms = 0, coop = 0, per_sm = 0;
  cudaGetDevice(&dev);
  if (cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev) != cudaSuccess || !coop) return 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, persist_kernel(precision, stack_entries, variant),
                                                    32 * kWbWarps, 0) != cudaSuccess)
    return 0;
  return per_sm < 1 ? 0 : sms * per_sm;
}

cudaError_t launch_collide_persistent(const CollideLaunch& L, int precision, int stack_entries, int grid,
                                      PersistCtl* ctl, int64_t* table, cudaStream_t s) {
  CollideLaunch Lc = L;
  long long* tab = reinterpret_cast<long long*>(table);
  void* args[] = {&Lc, &ctl, &tab};
  ++g_kernel_launches;
  return cudaLaunchCooperativeKernel(persist_kernel(precision, stack_entries, L.wb_variant), dim3(grid),
                                     dim3(32 * kWbWarps), args, 0, s);
}

int collide_round_grid(int precision, int stack_entries, int block, int variant) {
  int dev = 0, sms = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const void* k;
  if (precision == 0)
    k = stack_entries <= 64 ? (const void*)k_collide_round<0, 64> : (const void*)k_collide_round<0, 256>;
  else if (variant == 1)
    k = stack_entries <= 64 ? (const void*)k_collide_round_wb<64, 4> : (const void*)k_collide_round_wb<256, 4>;
  else
    k = stack_entries <= 64 ? (const void*)k_collide_round_wb<64, 1> : (const void*)k_collide_round_wb<256, 1>;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, precision == 0 ? block : 32 * kWbWarps, 0);
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
