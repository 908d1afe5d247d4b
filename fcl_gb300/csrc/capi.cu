// C ABI of the library (include/fclgpu.h): mesh registry, batched collide and
// distance entry points, device scratch management and status reporting.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/fclgpu.h"
#include "bvh_build.h"
#include "kernels.h"

using namespace fclgpu;

#include "mesh_handle.h"

namespace fclgpu {
void set_error_detail(const std::string& what);
}
int repack_mesh(fclgpu_mesh m, cudaStream_t s);  // mesh_refit.cu

namespace {

std::recursive_mutex g_mu;
int g_device = -1;
thread_local std::string g_detail;

int fail(int code, const std::string& why) {
  g_detail = why;
  return code;
}
int cuda_fail(cudaError_t e, const char* where) {
  g_detail = std::string(where) + ": " + cudaGetErrorString(e);
  return (e == cudaErrorMemoryAllocation) ? FCLGPU_ERR_OUT_OF_MEMORY : FCLGPU_ERR_CUDA;
}

#define CK(expr, where)                              \
  do {                                               \
    cudaError_t e_ = (expr);                         \
    if (e_ != cudaSuccess) return cuda_fail(e_, where); \
  } while (0)

// Grow-only device buffer.
struct DevBuf {
  void* p = nullptr;
  size_t cap = 0;
  cudaError_t ensure(size_t bytes) {
    if (bytes <= cap) return cudaSuccess;
    if (p) {
      cudaError_t e = cudaFree(p);
      if (e != cudaSuccess) return e;
      p = nullptr;
      cap = 0;
    }
    size_t want = std::max<size_t>(bytes, 256);
    cudaError_t e = cudaMalloc(&p, want);
    if (e == cudaSuccess) cap = want;
    return e;
  }
};

struct Scratch {
  DevBuf meshes, pairs, ctr, records, counts, offsets, scan_tmp;
  DevBuf in_pair, in_tf1, in_tf2, in_margin;
  DevBuf out_contacts, out_nbv, out_nleaf, out_nrc, out_dist, out_ids, out_pts, out_within;
  int64_t record_hint = 0;
  int64_t last_nrec = 0;  // records written by the last collide launch
};
Scratch g_scratch;

// Device time of the main traversal kernel of the most recent batch (CUDA events
// recorded on the batch's stream around that launch).
cudaEvent_t g_ev[2] = {nullptr, nullptr};
double g_last_kernel_ms = -1.0;
int ensure_events() {
  if (!g_ev[0]) {
    CK(cudaEventCreate(&g_ev[0]), "event");
    CK(cudaEventCreate(&g_ev[1]), "event");
  }
  return FCLGPU_OK;
}

int ensure_init() {
  if (g_device >= 0) return FCLGPU_OK;
  int dev = 0;
  CK(cudaGetDevice(&dev), "cudaGetDevice");
  g_device = dev;
  return FCLGPU_OK;
}

template <class T>
int upload(DevBuf& b, const T* host, size_t count, cudaStream_t s, const char* what) {
  CK(b.ensure(sizeof(T) * std::max<size_t>(count, 1)), what);
  if (count) CK(cudaMemcpyAsync(b.p, host, sizeof(T) * count, cudaMemcpyHostToDevice, s), what);
  return FCLGPU_OK;
}

// Common validation + mesh/pair tables.  Returns the traversal stack size needed.
int prepare_tables(const fclgpu_mesh* meshes, int32_t num_meshes, const int32_t* pairs_host, int32_t num_pairs,
                   cudaStream_t s, int* stack_entries) {
  if (!meshes || num_meshes <= 0 || !pairs_host || num_pairs <= 0)
    return fail(FCLGPU_ERR_INVALID_ARGUMENT, "meshes and pairs must be non-empty");
  std::vector<DevMesh> tab(num_meshes);
  for (int i = 0; i < num_meshes; ++i) {
    if (!meshes[i]) return fail(FCLGPU_ERR_INVALID_ARGUMENT, "null mesh handle");
    tab[i] = meshes[i]->dev;
  }
  int need = 0;
  for (int p = 0; p < num_pairs; ++p) {
    const int a = pairs_host[2 * p], b = pairs_host[2 * p + 1];
    if (a < 0 || a >= num_meshes || b < 0 || b >= num_meshes)
      return fail(FCLGPU_ERR_INVALID_ARGUMENT, "pair index out of range");
    need = std::max(need, tab[a].max_depth + tab[b].max_depth + 2);
  }
  if (need > 256) return fail(FCLGPU_ERR_STACK_DEPTH, "BVH pair deeper than 256 levels");
  *stack_entries = need <= 64 ? 64 : 256;
  int rc = upload(g_scratch.meshes, tab.data(), tab.size(), s, "upload mesh table");
  if (rc) return rc;
  std::vector<int2> pr(num_pairs);
  for (int p = 0; p < num_pairs; ++p) pr[p] = make_int2(pairs_host[2 * p], pairs_host[2 * p + 1]);
  rc = upload(g_scratch.pairs, pr.data(), pr.size(), s, "upload pair table");
  if (rc) return rc;
  return FCLGPU_OK;
}


// ---------------------------------------------------------------------------------
// Collide batch core: budgeted rounds of work items, then the item-tree assembly.
// ---------------------------------------------------------------------------------
struct SplitScratch {
  DevBuf items, own, cstart, ccount, total, rel_start, capped;
  DevBuf persist;  // PersistCtl, then the round table (persistent launch)
  int64_t item_hint = 0;
  CollideLaunch last;       // launch description of the last batch (for the scatter)
  int64_t last_nrec = 0;
  std::vector<std::pair<int64_t, int64_t>> rounds;
  std::vector<cudaEvent_t> ev;
};
SplitScratch g_split;

// Tuning knobs of the FP32 collide rounds (set by fclgpu_set_collide_tuning, picked by
// the autotuner in fcl_gb300/api.py): BV tests per item per round, DFS steps per lane
// between two warp leaf batches.
// defaults: the autotuner's pick on the 64-pair exhaustive-contact workload
int64_t g_default_budget = 1024;
int32_t g_wb_steps = 4;
int32_t g_wb_variant = 1;
// testing aids (fclgpu_set_collide_test_limits): initial scratch capacities, stack limit
int64_t g_test_records = 0, g_test_items = 0;
int32_t g_test_stack = 0;
// all rounds in one cooperative launch (fclgpu_set_collide_persistent): on/off, the
// grid barrier's wait limit, and (testing) blocks the barrier waits for beyond the grid
int32_t g_persist = 1;
int64_t g_persist_fallbacks = 0;
int64_t g_barrier_timeout_ns = 60000000000ll;
int32_t g_test_missing_blocks = 0;
constexpr int kPersistRounds = 1024;
constexpr size_t kPersistCtlBytes = 64;
static_assert(sizeof(PersistCtl) <= kPersistCtlBytes, "control block");

int collide_core(int64_t n, const int32_t* pair_of_query, const double* tf1, const double* tf2,
                 const fclgpu_collide_request* req, int32_t* counts, int64_t* offsets, int64_t* nbv, int64_t* nleaf,
                 int64_t* nrc, int stack, cudaStream_t s, int64_t* total_out) {
  Scratch& S = g_scratch;
  SplitScratch& P = g_split;
  CK(S.ctr.ensure(sizeof(BatchCounters)), "counters");
  const int64_t maxc = std::max<int64_t>(req->num_max_contacts, 0);
  const int64_t budget = req->budget > 0 ? req->budget : g_default_budget;
  int64_t rec_cap = std::max<int64_t>(S.record_hint, std::min<int64_t>(n * std::max<int64_t>(maxc, 1), 4 * n) + 65536);
  int64_t item_cap = std::max<int64_t>(P.item_hint, 4 * n + (1 << 20));
  if (g_test_records > 0) rec_cap = g_test_records;
  if (g_test_items > 0) item_cap = std::max<int64_t>(g_test_items, n);
  bool persist_ok = true;
  for (int attempt = 0; attempt < 9; ++attempt) {
    CK(S.records.ensure(sizeof(int4) * (size_t)rec_cap), "record scratch");
    // the buffers only grow; a test limit still caps the part a batch may use
    rec_cap = std::min<int64_t>((int64_t)(S.records.cap / sizeof(int4)),
                                g_test_records > 0 ? rec_cap : INT64_MAX);
    CK(P.items.ensure(sizeof(int4) * (size_t)item_cap), "item scratch");
    item_cap = std::min<int64_t>((int64_t)(P.items.cap / sizeof(int4)), g_test_items > 0 ? item_cap : INT64_MAX);
    CK(P.own.ensure(4 * (size_t)item_cap), "item scratch");
    CK(P.cstart.ensure(4 * (size_t)item_cap), "item scratch");
    CK(P.ccount.ensure(4 * (size_t)item_cap), "item scratch");
    if (req->enable_statistics) {
      if (nbv) CK(cudaMemsetAsync(nbv, 0, 8 * n, s), "stats");
      if (nleaf) CK(cudaMemsetAsync(nleaf, 0, 8 * n, s), "stats");
      if (nrc) CK(cudaMemsetAsync(nrc, 0, 8 * n, s), "stats");
    }
    BatchCounters h0;
    std::memset(&h0, 0, sizeof(h0));
    h0.items = (unsigned long long)n;
    CK(cudaMemcpyAsync(S.ctr.p, &h0, sizeof(h0), cudaMemcpyHostToDevice, s), "counters");
    CollideLaunch L{};
    L.meshes = (const DevMesh*)S.meshes.p;
    L.pairs = (const int2*)S.pairs.p;
    L.pair_of_query = pair_of_query;
    L.tf1 = tf1;
    L.tf2 = tf2;
    L.n = n;
    L.num_max_contacts = (int32_t)std::min<int64_t>(maxc, INT32_MAX);
    L.want_stats = req->enable_statistics;
    L.ctr = (BatchCounters*)S.ctr.p;
    L.records = (int4*)S.records.p;
    L.record_cap = rec_cap;
    L.counts = counts;
    L.nbv = nbv;
    L.nleaf = nleaf;
    L.nrecheck = nrc;
    L.items = (int4*)P.items.p;
    L.item_cap = item_cap;
    L.budget = budget;
    L.wb_steps = g_wb_steps;
    L.wb_variant = g_wb_variant;
    L.stack_limit = g_test_stack;
    L.own = (int32_t*)P.own.p;
    L.child_start = (int32_t*)P.cstart.p;
    L.child_count = (int32_t*)P.ccount.p;
    const int block = 128;
    const int grid = collide_round_grid(req->precision, stack, block, g_wb_variant);
    P.rounds.clear();
    int64_t lo = 0, hi = n;
    bool retry = false;
    double kernel_ms = 0.0;
    BatchCounters hc{};
    // a capacity overflow: grow the scratch and run the batch again
    auto overflow = [&]() {
      if (hc.status & DEV_ERR_RECORDS) rec_cap = std::max<int64_t>(rec_cap * 2, (int64_t)hc.records + 65536);
      if (hc.status & DEV_ERR_ITEMS) item_cap = std::max<int64_t>(item_cap * 2, (int64_t)hc.items + 65536);
      S.record_hint = rec_cap;
      P.item_hint = item_cap;
    };
    if (P.ev.size() < 2) {
      for (int k = 0; k < 2; ++k) {
        cudaEvent_t e;
        CK(cudaEventCreate(&e), "event");
        P.ev.push_back(e);
      }
    }
    // all rounds in one cooperative launch; the rounds' ranges come back in one read
    const int pgrid = (g_persist && persist_ok) ? collide_persistent_grid(req->precision, stack, g_wb_variant) : 0;
    if (pgrid > 0 && hi > lo) {
      CK(P.persist.ensure(kPersistCtlBytes + 16 * (size_t)kPersistRounds), "persistent control");
      std::vector<unsigned char> hb(kPersistCtlBytes + 16 * (size_t)kPersistRounds);
      PersistCtl c;
      std::memset(&c, 0, sizeof(c));
      c.lo = 0;
      c.hi = (unsigned long long)n;
      c.nblocks = (unsigned)(pgrid + g_test_missing_blocks);
      c.max_rounds = kPersistRounds;
      c.timeout_ns = (unsigned long long)g_barrier_timeout_ns;
      PersistCtl* dctl = (PersistCtl*)P.persist.p;
      int64_t* dtab = (int64_t*)((char*)P.persist.p + kPersistCtlBytes);
      CK(cudaMemcpyAsync(dctl, &c, sizeof(c), cudaMemcpyHostToDevice, s), "persistent control");
      CK(cudaEventRecord(P.ev[0], s), "event");
      CK(launch_collide_persistent(L, req->precision, stack, pgrid, dctl, dtab, s), "persistent collide");
      CK(cudaEventRecord(P.ev[1], s), "event");
      CK(cudaMemcpyAsync(hb.data(), P.persist.p, hb.size(), cudaMemcpyDeviceToHost, s), "persistent control");
      CK(cudaMemcpyAsync(&hc, S.ctr.p, sizeof(hc), cudaMemcpyDeviceToHost, s), "read counters");
      CK(cudaStreamSynchronize(s), "persistent collide");
      float ms = 0.f;
      CK(cudaEventElapsedTime(&ms, P.ev[0], P.ev[1]), "event");
      kernel_ms += ms;
      std::memcpy(&c, hb.data(), sizeof(c));
      if (c.err & DEV_ERR_BARRIER) {  // run the batch again, one launch per round
        persist_ok = false;
        g_persist_fallbacks++;
        continue;
      }
      if (hc.status & DEV_ERR_STACK) return fail(FCLGPU_ERR_DEVICE_STATUS, "traversal stack overflow");
      if (hc.status & (DEV_ERR_RECORDS | DEV_ERR_ITEMS)) {
        overflow();
        if (item_cap > 0x7fffffffll) return fail(FCLGPU_ERR_OUT_OF_MEMORY, "work items exceed 2^31");
        continue;
      }
      const int64_t* tab = (const int64_t*)(hb.data() + kPersistCtlBytes);
      for (unsigned r = 0; r < c.nrounds; ++r) P.rounds.emplace_back(tab[2 * r], tab[2 * r + 1]);
      lo = (int64_t)c.lo;
      hi = (int64_t)c.hi;
      CK(cudaMemsetAsync(&L.ctr->work, 0, sizeof(unsigned long long), s), "counters");
    }
    for (int round = 0; round < 100000 && hi > lo; ++round) {
      L.item_lo = lo;
      L.item_hi = hi;
      P.rounds.emplace_back(lo, hi);
      CK(cudaMemsetAsync(&L.ctr->work, 0, sizeof(unsigned long long), s), "counters");
      CK(cudaEventRecord(P.ev[0], s), "event");
      CK(launch_collide_round(L, req->precision, stack, grid, block, s), "collide round");
      CK(cudaEventRecord(P.ev[1], s), "event");
      CK(cudaMemcpyAsync(&hc, S.ctr.p, sizeof(hc), cudaMemcpyDeviceToHost, s), "read counters");
      CK(cudaStreamSynchronize(s), "collide round");
      float ms = 0.f;
      CK(cudaEventElapsedTime(&ms, P.ev[0], P.ev[1]), "event");
      kernel_ms += ms;
      if (hc.status & DEV_ERR_STACK) return fail(FCLGPU_ERR_DEVICE_STATUS, "traversal stack overflow");
      if (hc.status & (DEV_ERR_RECORDS | DEV_ERR_ITEMS)) {
        overflow();
        if (item_cap > 0x7fffffffll) return fail(FCLGPU_ERR_OUT_OF_MEMORY, "work items exceed 2^31");
        retry = true;
        break;
      }
      lo = hi;
      hi = (int64_t)hc.items;
    }
    if (retry) continue;
    g_last_kernel_ms = kernel_ms;
    const int64_t nitems = hi;
    S.record_hint = std::max<int64_t>(S.record_hint, (int64_t)hc.records);
    P.item_hint = std::max<int64_t>(P.item_hint, nitems);
    P.last_nrec = (int64_t)hc.records;
    // assembly: totals bottom-up, counts and offsets, starts top-down
    CK(P.total.ensure(8 * (size_t)std::max<int64_t>(nitems, 1)), "item scratch");
    CK(P.rel_start.ensure(8 * (size_t)std::max<int64_t>(nitems, 1)), "item scratch");
    CK(P.capped.ensure(4 * (size_t)std::max<int64_t>(n, 1)), "item scratch");
    int64_t* tot = (int64_t*)P.total.p;
    for (size_t r = P.rounds.size(); r-- > 0;)
      CK(launch_item_totals(L, P.rounds[r].first, P.rounds[r].second, tot, s), "item totals");
    CK(launch_item_counts(L, tot, (int32_t*)P.capped.p, s), "item counts");
    CK(S.scan_tmp.ensure(sizeof(int64_t) * (size_t)(2 * ((n + 4095) / 4096) + 4)), "scan scratch");
    CK(launch_exclusive_scan(counts, n, offsets, (int64_t*)S.scan_tmp.p, s), "scan");
    for (size_t r = 0; r < P.rounds.size(); ++r)
      CK(launch_item_starts(L, P.rounds[r].first, P.rounds[r].second, tot, (int64_t*)P.rel_start.p, s),
         "item starts");
    int64_t total = 0;
    CK(cudaMemcpyAsync(&total, offsets + n, sizeof(int64_t), cudaMemcpyDeviceToHost, s), "read total");
    CK(cudaMemcpyAsync(&hc, S.ctr.p, sizeof(hc), cudaMemcpyDeviceToHost, s), "read counters");
    CK(cudaStreamSynchronize(s), "assembly");
    if (req->enable_statistics && hc.capped_split > 0) {
      // queries split across items and capped at num_max_contacts ran past FCL's stop
      // point; their statistics come from an exact serial traversal
      CK(cudaMemsetAsync(&L.ctr->work, 0, sizeof(unsigned long long), s), "counters");
      CK(launch_collide_stats(L, (const int32_t*)P.capped.p, (int64_t)hc.capped_split, req->precision, stack, s),
         "stats pass");
    }
    P.last = L;
    *total_out = total;
    return FCLGPU_OK;
  }
  return fail(FCLGPU_ERR_OUT_OF_MEMORY, "batch scratch kept overflowing");
}

int collide_scatter(const int64_t* offsets, int32_t* contacts, cudaStream_t s) {
  CK(launch_scatter_items(g_split.last, g_split.last_nrec, (const int64_t*)g_split.rel_start.p, offsets, contacts, s),
     "scatter");
  return FCLGPU_OK;
}

// ---------------------------------------------------------------------------------
// Collide with contact geometry (enable_contact): the pair traversal lists the
// intersecting triangle pairs; mesh_contact.cu turns them into contacts.
// ---------------------------------------------------------------------------------
struct ContactScratch {
  DevBuf pcounts, poff, plist, qid, nc, info, G, flag, scan_tmp;
  ContactLaunch last{};
};
ContactScratch g_contact;

// Per-query contact counts and offsets (n + 1) of the batch; the pairs and their contact
// geometry stay in g_contact for contacts_emit.
int contacts_core(int64_t n, const int32_t* pair_of_query, const double* tf1, const double* tf2,
                  const fclgpu_collide_request* req, int stack, int32_t* counts, int64_t* offsets, cudaStream_t s,
                  int64_t* total_out) {
  ContactScratch& C = g_contact;
  const int64_t maxc = std::max<int64_t>(req->num_max_contacts, 0);
  int64_t pair_cap = maxc;
  CK(C.pcounts.ensure(4 * (size_t)n), "contact scratch");
  CK(C.poff.ensure(8 * (size_t)(n + 1)), "contact scratch");
  CK(C.flag.ensure(sizeof(unsigned int)), "contact scratch");
  for (int attempt = 0; attempt < 40; ++attempt) {
    fclgpu_collide_request r = *req;
    r.num_max_contacts = (int32_t)pair_cap;
    r.enable_statistics = 0;
    int64_t npairs = 0;
    int rc = collide_core(n, pair_of_query, tf1, tf2, &r, (int32_t*)C.pcounts.p, (int64_t*)C.poff.p, nullptr,
                          nullptr, nullptr, stack, s, &npairs);
    if (rc) return rc;
    const size_t np = (size_t)std::max<int64_t>(npairs, 1);
    CK(C.plist.ensure(8 * np), "contact scratch");
    CK(C.qid.ensure(4 * np), "contact scratch");
    CK(C.nc.ensure(4 * np), "contact scratch");
    CK(C.info.ensure(80 * np), "contact scratch");
    CK(C.G.ensure(8 * (np + 1)), "contact scratch");
    const int64_t scan_n = std::max<int64_t>(npairs, n);
    CK(C.scan_tmp.ensure(sizeof(int64_t) * (size_t)(2 * ((scan_n + 4095) / 4096) + 4)), "scan scratch");
    rc = collide_scatter((const int64_t*)C.poff.p, (int32_t*)C.plist.p, s);
    if (rc) return rc;
    ContactLaunch L{};
    L.meshes = (const DevMesh*)g_scratch.meshes.p;
    L.pairs = (const int2*)g_scratch.pairs.p;
    L.pair_of_query = pair_of_query;
    L.tf1 = tf1;
    L.tf2 = tf2;
    L.n = n;
    L.poff = (const int64_t*)C.poff.p;
    L.plist = (const int2*)C.plist.p;
    L.npairs = npairs;
    L.max_contacts = (int32_t)std::min<int64_t>(maxc, INT32_MAX);
    L.pair_cap = (int32_t)pair_cap;
    L.qid = (int32_t*)C.qid.p;
    L.nc = (int32_t*)C.nc.p;
    L.info = (double*)C.info.p;
    L.G = (const int64_t*)C.G.p;
    CK(launch_contact_info(L, s), "contact info");
    CK(launch_exclusive_scan(L.nc, npairs, (int64_t*)C.G.p, (int64_t*)C.scan_tmp.p, s), "contact scan");
    CK(cudaMemsetAsync(C.flag.p, 0, sizeof(unsigned int), s), "contact flag");
    CK(launch_contact_counts(L, (const int32_t*)C.pcounts.p, counts, (unsigned int*)C.flag.p, s), "contact counts");
    unsigned int incomplete = 0;
    CK(cudaMemcpyAsync(&incomplete, C.flag.p, sizeof(incomplete), cudaMemcpyDeviceToHost, s), "contact flag");
    CK(cudaStreamSynchronize(s), "contact counts");
    C.last = L;
    if (incomplete == 0 || pair_cap >= INT32_MAX) break;
    // some query's pair list ended at the cap with fewer contacts than it may hold (pairs
    // without a contact point): list more pairs
    pair_cap = std::min<int64_t>(2 * std::max<int64_t>(pair_cap, 1), INT32_MAX);
  }
  CK(launch_exclusive_scan(counts, n, offsets, (int64_t*)C.scan_tmp.p, s), "contact offsets");
  int64_t total = 0;
  CK(cudaMemcpyAsync(&total, offsets + n, sizeof(int64_t), cudaMemcpyDeviceToHost, s), "read total");
  CK(cudaStreamSynchronize(s), "contact offsets");
  *total_out = total;
  return FCLGPU_OK;
}

int contacts_emit(const int64_t* offsets, int32_t* ids, double* pos, double* normal, double* depth,
                  cudaStream_t s) {
  CK(launch_contact_emit(g_contact.last, offsets, ids, pos, normal, depth, s), "contact emit");
  return FCLGPU_OK;
}

}  // namespace

void fclgpu::set_error_detail(const std::string& what) { g_detail = what; }

extern "C" {

const char* fclgpu_status_string(int status) {
  switch (status) {
    case FCLGPU_OK: return "ok";
    case FCLGPU_ERR_INVALID_ARGUMENT: return "invalid argument";
    case FCLGPU_ERR_CUDA: return "CUDA error";
    case FCLGPU_ERR_OUT_OF_MEMORY: return "out of device memory";
    case FCLGPU_ERR_CAPACITY: return "output capacity too small";
    case FCLGPU_ERR_EMPTY_MODEL: return "model has no triangles or vertices";
    case FCLGPU_ERR_STACK_DEPTH: return "BVH too deep for the traversal stack";
    case FCLGPU_ERR_DEVICE_STATUS: return "kernel reported an internal error";
    case FCLGPU_ERR_NOT_INITIALIZED: return "not initialized";
    case FCLGPU_ERR_UNSUPPORTED: return "unsupported";
    case FCLGPU_ERR_PENDING: return "request not finished";
    case FCLGPU_ERR_INCORRECT_DATA: return "incorrect data";
    default: return "unknown status";
  }
}

const char* fclgpu_last_error_detail(void) { return g_detail.c_str(); }

int fclgpu_init(int device) {
  std::lock_guard<std::recursive_mutex> lk(g_mu);
  int n = 0;
  CK(cudaGetDeviceCount(&n), "cudaGetDeviceCount");
  if (device < 0 || device >= n) return fail(FCLGPU_ERR_INVALID_ARGUMENT, "no such device");
  CK(cudaSetDevice(device), "cudaSetDevice");
  CK(cudaFree(nullptr), "context");
  g_device = device;
  return FCLGPU_OK;
}

int64_t fclgpu_kernel_launch_count(void) { return g_kernel_launches; }

int fclgpu_last_kernel_time(double* ms) {
  if (!ms) return fail(FCLGPU_ERR_INVALID_ARGUMENT, "null argument");
  if (g_last_kernel_ms < 0) return fail(FCLGPU_ERR_NOT_INITIALIZED, "no batch has run");
  *ms = g_last_kernel_ms;
  return FCLGPU_OK;
}

int fclgpu_set_collide_tuning(int32_t budget, int32_t leaf_batch_steps, int32_t variant) {
  if (budget < 16 || budget > (1 << 24) || leaf_batch_steps < 1 || leaf_batch_steps > 256 || variant < 0 ||
      variant > 1)
    return fail(FCLGPU_ERR_INVALID_ARGUMENT, "tuning value out of range");
  std::lock_guard<std::recursive_mutex> lk(g_mu);
  g_default_budget = budget;
  g_wb_steps = leaf_batch_steps;
  g_wb_variant = variant;
  return FCLGPU_OK;
}

int fclgpu_set_collide_persistent(int32_t enable, int64_t barrier_timeout_ns, int32_t test_missing_blocks) {
  if (enable < 0 || enable > 1 || barrier_timeout_ns < 1000 || test_missing_blocks < 0 || test_missing_blocks > 1)
    return fail(FCLGPU_ERR_INVALID_ARGUMENT, "persistent-launch setting out of range");
  std::lock_guard<std::recursive_mutex> lk(g_mu);
  g_persist = enable;
  g_barrier_timeout_ns = barrier_timeout_ns;
  g_test_missing_blocks = test_missing_blocks;
  return FCLGPU_OK;
}

int64_t fclgpu_collide_persistent_fallbacks(void) { return g_persist_fallbacks; }

int fclgpu_set_collide_test_limits(int64_t initial_records, int64_t initial_items, int32_t stack_limit) {
  if (initial_records < 0 || initial_items < 0 || stack_limit < 0)
    return fail(FCLGPU_ERR_INVALID_ARGUMENT, "test limits must be >= 0");
  std::lock_guard<std::recursive_mutex> lk(g_mu);
  g_test_records = initial_records;
  g_test_items = initial_items;
  g_test_stack = stack_limit;
  if (initial_records > 0) g_scratch.record_hint = 0;
  if (initial_items > 0) g_split.item_hint = 0;
  return FCLGPU_OK;
}

int fclgpu_get_collide_tuning(int32_t* budget, int32_t* leaf_batch_steps, int32_t* variant) {
  if (!budget || !leaf_batch_steps || !variant) return fail(FCLGPU_ERR_INVALID_ARGUMENT, "null argument");
  std::lock_guard<std::recursive_mutex> lk(g_mu);
  *budget = (int32_t)g_default_budget;
  *leaf_batch_steps = g_wb_steps;
  *variant = g_wb_variant;
  return FCLGPU_OK;
}

}  // extern "C"

namespace {
// BVHModel::computeLocalAABB (geometry/bvh/BVH_model-inl.h:1080-1100) and the first vertex
void set_local_aabb(fclgpu_mesh_s* m, const double* verts, int64_t nv) {
  double lo[3], hi[3];
  for (int k = 0; k < 3; ++k) {
    lo[k] = std::numeric_limits<double>::max();
    hi[k] = -std::numeric_limits<double>::max();
  }
  for (int64_t i = 0; i < nv; ++i)
    for (int k = 0; k < 3; ++k) {
      lo[k] = std::min(lo[k], verts[3 * i + k]);
      hi[k] = std::max(hi[k], verts[3 * i + k]);
    }
  double c[3], r = 0;
  for (int k = 0; k < 3; ++k) c[k] = (lo[k] + hi[k]) * 0.5;
  for (int64_t i = 0; i < nv; ++i) {
    const double dx = c[0] - verts[3 * i], dy = c[1] - verts[3 * i + 1], dz = c[2] - verts[3 * i + 2];
    const double q = (dx * dx + dy * dy) + dz * dz;
    if (q > r) r = q;
  }
  for (int k = 0; k < 3; ++k) {
    m->aabb_local[k] = lo[k];
    m->aabb_local[3 + k] = hi[k];
    m->aabb_center[k] = c[k];
    m->first_vertex[k] = verts[k];
  }
  m->aabb_radius = std::sqrt(r);
}

int check_model(const double* verts, int64_t nv, const int32_t* tris, int64_t nt, fclgpu_mesh* out) {
  if (!out) return fail(FCLGPU_ERR_INVALID_ARGUMENT, "out is null");
  *out = nullptr;
  if (nv <= 0 || nt <= 0 || !verts || !tris) return fail(FCLGPU_ERR_EMPTY_MODEL, "empty model");
  if (nt > (1 << 29)) return fail(FCLGPU_ERR_INVALID_ARGUMENT, "too many triangles");
  for (int64_t i = 0; i < 3 * nt; ++i)
    if (tris[i] < 0 || tris[i] >= nv) return fail(FCLGPU_ERR_INVALID_ARGUMENT, "triangle index out of range");
  return FCLGPU_OK;
}
}  // namespace

extern "C" {

int fclgpu_mesh_create_on_device(const double* verts, int64_t nv, const int32_t* tris, int64_t nt, fclgpu_mesh* out,
                                 void* stream) {
  int rc = check_model(verts, nv, tris, nt, out);
  if (rc) return rc;
  std::lock_guard<std::recursive_mutex> lk(g_mu);
  rc = ensure_init();
  if (rc) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  fclgpu_mesh_s* m = new fclgpu_mesh_s();
  const size_t nn = 2 * (size_t)nt - 1;
  auto alloc = [&](void** p, size_t bytes) -> cudaError_t {
    cudaError_t e = cudaMalloc(p, std::max<size_t>(bytes, 16));
    if (e == cudaSuccess) m->allocations.push_back(*p);
    return e;
  };
  void *p_n64, *p_r64, *p_v64, *p_t, *p_n32, *p_s64, *p_r32, *p_t32, *p_lv;
  cudaError_t e = cudaSuccess;
  if (e == cudaSuccess) e = alloc(&p_n64, sizeof(NodeD) * nn);
  if (e == cudaSuccess) e = alloc(&p_r64, sizeof(RssD) * nn);
  if (e == cudaSuccess) e = alloc(&p_v64, sizeof(double) * 3 * nv);
  if (e == cudaSuccess) e = alloc(&p_t, sizeof(int32_t) * 3 * nt);
  if (e == cudaSuccess) e = alloc(&p_n32, sizeof(float) * 16 * nn);
  if (e == cudaSuccess) e = alloc(&p_s64, sizeof(double) * nn);
  if (e == cudaSuccess) e = alloc(&p_r32, sizeof(float) * 20 * nn);
  if (e == cudaSuccess) e = alloc(&p_t32, sizeof(float) * 12 * nt);
  if (e == cudaSuccess) e = alloc(&p_lv, sizeof(int32_t) * std::max<size_t>(nn / 2, 1));
  if (e == cudaSuccess) e = cudaMemcpyAsync(p_v64, verts, sizeof(double) * 3 * nv, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(p_t, tris, sizeof(int32_t) * 3 * nt, cudaMemcpyHostToDevice, s);
  int maxd = 0;
  std::vector<int64_t> off;
  if (e == cudaSuccess)
    e = build_bvh_device((const double*)p_v64, (const int32_t*)p_t, (int)nt, (NodeD*)p_n64, (RssD*)p_r64, off,
                         (int32_t*)p_lv, &maxd, s);
  if (e != cudaSuccess) {
    cudaStreamSynchronize(s);
    for (void* p : m->allocations) cudaFree(p);
    delete m;
    return cuda_fail(e, "device build");
  }
  DevMesh& d = m->dev;
  d.nodes64 = (const NodeD*)p_n64;
  d.rss64 = (const RssD*)p_r64;
  d.verts64 = (const double*)p_v64;
  d.tris = (const int32_t*)p_t;
  d.nodes32 = p_n32;
  d.size64 = (const double*)p_s64;
  d.rss32 = p_r32;
  d.tri32 = p_t32;
  d.n_nodes = (int32_t)nn;
  d.n_tris = (int32_t)nt;
  d.n_verts = (int32_t)nv;
  d.max_depth = maxd;
  d.refitted = 0;
  d.pad2 = 0;
  m->levels = (int32_t*)p_lv;
  m->level_off = off;
  rc = repack_mesh(m, s);
  if (rc) {
    for (void* p : m->allocations) cudaFree(p);
    delete m;
    return rc;
  }
  set_local_aabb(m, verts, nv);
  m->info.num_vertices = nv;
  m->info.num_tris = nt;
  m->info.num_nodes = (int64_t)nn;
  m->info.max_depth = maxd;
  m->info.reserved = 0;
  m->info.device_bytes = (int64_t)(nn * (sizeof(NodeD) + sizeof(RssD) + 64 + 8 + 80) + nv * 24 + nt * (12 + 48));
  *out = m;
  return FCLGPU_OK;
}

int fclgpu_mesh_create(const double* verts, int64_t nv, const int32_t* tris, int64_t nt, fclgpu_mesh* out) {
  {
    const int rc0 = check_model(verts, nv, tris, nt, out);
    if (rc0) return rc0;
  }
  // the host build runs outside the lock so several meshes can be built in parallel
  HostBVH bvh;
  if (build_obbrss(verts, nv, tris, nt, bvh) != 0) return fail(FCLGPU_ERR_EMPTY_MODEL, "empty model");
  PackedF32 pk;
  pack_fp32(verts, tris, nt, bvh, pk);
  std::lock_guard<std::recursive_mutex> lk(g_mu);
  int rc = ensure_init();
  if (rc) return rc;

  fclgpu_mesh_s* m = new fclgpu_mesh_s();
  auto alloc = [&](void** p, size_t bytes, const void* src) -> cudaError_t {
    cudaError_t e = cudaMalloc(p, std::max<size_t>(bytes, 16));
    if (e != cudaSuccess) return e;
    m->allocations.push_back(*p);
    return cudaMemcpy(*p, src, bytes, cudaMemcpyHostToDevice);
  };
  const size_t nn = bvh.nodes.size();
  void *p_n64, *p_r64, *p_v64, *p_t, *p_n32, *p_s64, *p_r32, *p_t32;
  cudaError_t e = cudaSuccess;
  if (e == cudaSuccess) e = alloc(&p_n64, sizeof(NodeD) * nn, bvh.nodes.data());
  if (e == cudaSuccess) e = alloc(&p_r64, sizeof(RssD) * nn, bvh.rss.data());
  if (e == cudaSuccess) e = alloc(&p_v64, sizeof(double) * 3 * nv, verts);
  if (e == cudaSuccess) e = alloc(&p_t, sizeof(int32_t) * 3 * nt, tris);
  if (e == cudaSuccess) e = alloc(&p_n32, sizeof(float) * pk.nodes32.size(), pk.nodes32.data());
  if (e == cudaSuccess) e = alloc(&p_s64, sizeof(double) * pk.size64.size(), pk.size64.data());
  if (e == cudaSuccess) e = alloc(&p_r32, sizeof(float) * pk.rss32.size(), pk.rss32.data());
  if (e == cudaSuccess) e = alloc(&p_t32, sizeof(float) * pk.tri32.size(), pk.tri32.data());
  if (e != cudaSuccess) {
    for (void* p : m->allocations) cudaFree(p);
    delete m;
    return cuda_fail(e, "mesh upload");
  }
  double vmax = 0.0;
  for (int64_t i = 0; i < 3 * nv; ++i) vmax = std::max(vmax, std::fabs(verts[i]));
  DevMesh& d = m->dev;
  d.nodes64 = (const NodeD*)p_n64;
  d.rss64 = (const RssD*)p_r64;
  d.verts64 = (const double*)p_v64;
  d.tris = (const int32_t*)p_t;
  d.nodes32 = p_n32;
  d.size64 = (const double*)p_s64;
  d.rss32 = p_r32;
  d.tri32 = p_t32;
  d.n_nodes = (int32_t)nn;
  d.n_tris = (int32_t)nt;
  d.n_verts = (int32_t)nv;
  d.max_depth = bvh.max_depth;
  // inflate the magnitude constants slightly so they bound the FP64 values after rounding
  d.vmax = vmax * (1.0 + 1e-12);
  d.cmax = pk.cmax * (1.0 + 1e-12);
  d.rmax = pk.rmax * (1.0 + 1e-12);
  d.refitted = 0;
  d.pad2 = 0;
  set_local_aabb(m, verts, nv);
  {
    // internal nodes by depth, for the level-by-level refit
    std::vector<int32_t> depth(nn, 0);
    int maxd = 0;
    for (size_t b = 0; b < nn; ++b) {  // children always follow their parent
      const int c = bvh.nodes[b].child;
      if (c >= 0) {
        depth[c] = depth[c + 1] = depth[b] + 1;
        maxd = std::max(maxd, depth[b]);
      }
    }
    std::vector<int64_t> off(maxd + 2, 0);
    for (size_t b = 0; b < nn; ++b)
      if (bvh.nodes[b].child >= 0) ++off[depth[b] + 1];
    for (int l = 0; l <= maxd; ++l) off[l + 1] += off[l];
    std::vector<int32_t> ids(std::max<int64_t>(off[maxd + 1], 1));
    std::vector<int64_t> fill(off.begin(), off.end() - 1);
    for (size_t b = 0; b < nn; ++b)
      if (bvh.nodes[b].child >= 0) ids[fill[depth[b]]++] = (int32_t)b;
    void* p_lv = nullptr;
    e = alloc(&p_lv, sizeof(int32_t) * ids.size(), ids.data());
    if (e != cudaSuccess) {
      for (void* p : m->allocations) cudaFree(p);
      delete m;
      return cuda_fail(e, "mesh upload");
    }
    m->levels = (int32_t*)p_lv;
    m->level_off = off;
  }
  m->info.num_vertices = nv;
  m->info.num_tris = nt;
  m->info.num_nodes = (int64_t)nn;
  m->info.max_depth = bvh.max_depth;
  m->info.reserved = 0;
  m->info.max_abs_coord = vmax;
  m->info.device_bytes = (int64_t)(nn * (sizeof(NodeD) + sizeof(RssD) + 64 + 8 + 80) + nv * 24 + nt * (12 + 48));
  *out = m;
  return FCLGPU_OK;
}

int fclgpu_mesh_destroy(fclgpu_mesh mesh) {
  if (!mesh) return FCLGPU_OK;
  std::lock_guard<std::recursive_mutex> lk(g_mu);
  for (void* p : mesh->allocations) cudaFree(p);
  delete mesh;
  return FCLGPU_OK;
}

int fclgpu_mesh_get_info(fclgpu_mesh mesh, fclgpu_mesh_info* info) {
  if (!mesh || !info) return fail(FCLGPU_ERR_INVALID_ARGUMENT, "null argument");
  *info = mesh->info;
  return FCLGPU_OK;
}

int fclgpu_mesh_get_nodes(fclgpu_mesh mesh, double* nodes30, int32_t* first_child) {
  if (!mesh || !nodes30 || !first_child) return fail(FCLGPU_ERR_INVALID_ARGUMENT, "null argument");
  const size_t nn = (size_t)mesh->dev.n_nodes;
  std::vector<NodeD> nd(nn);
  std::vector<RssD> rs(nn);
  CK(cudaMemcpy(nd.data(), mesh->dev.nodes64, sizeof(NodeD) * nn, cudaMemcpyDeviceToHost), "read nodes");
  CK(cudaMemcpy(rs.data(), mesh->dev.rss64, sizeof(RssD) * nn, cudaMemcpyDeviceToHost), "read rss");
  for (size_t i = 0; i < nn; ++i) {
    double* o = nodes30 + 30 * i;
    for (int k = 0; k < 9; ++k) o[k] = nd[i].axis[k];
    for (int k = 0; k < 3; ++k) o[9 + k] = nd[i].To[k];
    for (int k = 0; k < 3; ++k) o[12 + k] = nd[i].ext[k];
    for (int k = 0; k < 9; ++k) o[15 + k] = rs[i].axis[k];
    for (int k = 0; k < 3; ++k) o[24 + k] = rs[i].To[k];
    o[27] = rs[i].l[0];
    o[28] = rs[i].l[1];
    o[29] = rs[i].r;
    first_child[i] = nd[i].child;
  }
  return FCLGPU_OK;
}

int fclgpu_collide_batch_device(const fclgpu_mesh* meshes, int32_t num_meshes, const int32_t* pairs_host,
                                int32_t num_pairs, int64_t n, const int32_t* pair_of_query, const double* tf1,
                                const double* tf2, const fclgpu_collide_request* req, fclgpu_collide_result* res,
                                void* stream) {
  if (!req || !res || n < 0 || (n > 0 && (!tf2 || !res->counts)))
    return fail(FCLGPU_ERR_INVALID_ARGUMENT, "missing request, result, tf2 or counts");
  if (n >= (int64_t)1 << 31) return fail(FCLGPU_ERR_INVALID_ARGUMENT, "batch too large");
  if (req->precision != FCLGPU_PLAIN_FP64 && req->precision != FCLGPU_FP32_RECHECK)
    return fail(FCLGPU_ERR_INVALID_ARGUMENT, "unknown precision");
  std::lock_guard<std::recursive_mutex> lk(g_mu);
  int rc = ensure_init();
  if (rc) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  int stack = 64;
  rc = prepare_tables(meshes, num_meshes, pairs_host, num_pairs, s, &stack);
  if (rc) return rc;
  res->total_contacts = 0;
  if (n == 0) {
    if (res->offsets) CK(cudaMemsetAsync(res->offsets, 0, sizeof(int64_t), s), "offsets");
    return FCLGPU_OK;
  }
  int64_t* offsets = res->offsets;
  if (!offsets) {
    CK(g_scratch.offsets.ensure(sizeof(int64_t) * (size_t)(n + 1)), "offsets scratch");
    offsets = (int64_t*)g_scratch.offsets.p;
  }
  int64_t total = 0;
  rc = collide_core(n, pair_of_query, tf1, tf2, req, res->counts, offsets, res->num_bv_tests,
                    res->num_leaf_tests, res->num_rechecks, stack, s, &total);
  if (rc) return rc;
  res->total_contacts = total;
  if (!res->contacts) return FCLGPU_OK;
  if (total > res->contacts_capacity) return fail(FCLGPU_ERR_CAPACITY, "contacts buffer too small");
  return collide_scatter(offsets, res->contacts, s);
}

int fclgpu_collide_batch(const fclgpu_mesh* meshes, int32_t num_meshes, const int32_t* pairs_host,
                         int32_t num_pairs, int64_t n, const int32_t* pair_of_query, const double* tf1,
                         const double* tf2, const fclgpu_collide_request* req, fclgpu_collide_result* res,
                         void* stream) {
  if (!req || !res || n < 0 || (n > 0 && (!tf2 || !res->counts)))
    return fail(FCLGPU_ERR_INVALID_ARGUMENT, "missing request, result, tf2 or counts");
  cudaStream_t s = (cudaStream_t)stream;
  Scratch& S = g_scratch;
  const size_t nn = (size_t)std::max<int64_t>(n, 1);
  std::lock_guard<std::recursive_mutex> lk(g_mu);  // held across the device call and the copies
  {
    int rc = ensure_init();
    if (rc) return rc;
    if (pair_of_query) CK(S.in_pair.ensure(4 * nn), "inputs");
    if (tf1) CK(S.in_tf1.ensure(96 * nn), "inputs");
    CK(S.in_tf2.ensure(96 * nn), "inputs");
    CK(S.counts.ensure(4 * nn), "outputs");
    CK(S.offsets.ensure(8 * (nn + 1)), "outputs");
    if (res->num_bv_tests) CK(S.out_nbv.ensure(8 * nn), "outputs");
    if (res->num_leaf_tests) CK(S.out_nleaf.ensure(8 * nn), "outputs");
    if (res->num_rechecks) CK(S.out_nrc.ensure(8 * nn), "outputs");
    if (pair_of_query) CK(cudaMemcpyAsync(S.in_pair.p, pair_of_query, 4 * n, cudaMemcpyHostToDevice, s), "h2d");
    if (tf1) CK(cudaMemcpyAsync(S.in_tf1.p, tf1, 96 * n, cudaMemcpyHostToDevice, s), "h2d");
    CK(cudaMemcpyAsync(S.in_tf2.p, tf2, 96 * n, cudaMemcpyHostToDevice, s), "h2d");
  }
  fclgpu_collide_result dr = *res;
  dr.counts = (int32_t*)S.counts.p;
  dr.offsets = (int64_t*)S.offsets.p;
  dr.contacts = nullptr;
  dr.num_bv_tests = res->num_bv_tests ? (int64_t*)S.out_nbv.p : nullptr;
  dr.num_leaf_tests = res->num_leaf_tests ? (int64_t*)S.out_nleaf.p : nullptr;
  dr.num_rechecks = res->num_rechecks ? (int64_t*)S.out_nrc.p : nullptr;
  // first pass computes counts and offsets; contacts are scattered into device scratch
  // sized from the total, then copied out
  int rc = fclgpu_collide_batch_device(meshes, num_meshes, pairs_host, num_pairs, n,
                                       pair_of_query ? (const int32_t*)S.in_pair.p : nullptr,
                                       tf1 ? (const double*)S.in_tf1.p : nullptr, (const double*)S.in_tf2.p, req,
                                       &dr, stream);
  if (rc) return rc;
  res->total_contacts = dr.total_contacts;
  if (res->contacts) {
    if (dr.total_contacts > res->contacts_capacity) return fail(FCLGPU_ERR_CAPACITY, "contacts buffer too small");
    CK(S.out_contacts.ensure(8 * (size_t)std::max<int64_t>(dr.total_contacts, 1)), "contacts scratch");
    // records of the batch are still in scratch: scatter them now
    rc = collide_scatter((const int64_t*)S.offsets.p, (int32_t*)S.out_contacts.p, s);
    if (rc) return rc;
    if (dr.total_contacts)
      CK(cudaMemcpyAsync(res->contacts, S.out_contacts.p, 8 * dr.total_contacts, cudaMemcpyDeviceToHost, s), "d2h");
  }
  CK(cudaMemcpyAsync(res->counts, S.counts.p, 4 * n, cudaMemcpyDeviceToHost, s), "d2h");
  if (res->offsets) CK(cudaMemcpyAsync(res->offsets, S.offsets.p, 8 * (n + 1), cudaMemcpyDeviceToHost, s), "d2h");
  if (res->num_bv_tests) CK(cudaMemcpyAsync(res->num_bv_tests, S.out_nbv.p, 8 * n, cudaMemcpyDeviceToHost, s), "d2h");
  if (res->num_leaf_tests)
    CK(cudaMemcpyAsync(res->num_leaf_tests, S.out_nleaf.p, 8 * n, cudaMemcpyDeviceToHost, s), "d2h");
  if (res->num_rechecks) CK(cudaMemcpyAsync(res->num_rechecks, S.out_nrc.p, 8 * n, cudaMemcpyDeviceToHost, s), "d2h");
  CK(cudaStreamSynchronize(s), "collide batch");
  return FCLGPU_OK;
}

int fclgpu_collide_contacts_device(const fclgpu_mesh* meshes, int32_t num_meshes, const int32_t* pairs_host,
                                   int32_t num_pairs, int64_t n, const int32_t* pair_of_query, const double* tf1,
                                   const double* tf2, const fclgpu_collide_request* req, fclgpu_contact_result* res,
                                   void* stream) {
  if (!req || !res || n < 0 || (n > 0 && (!tf2 || !res->counts || !res->offsets)))
    return fail(FCLGPU_ERR_INVALID_ARGUMENT, "missing request, result, tf2, counts or offsets");
  if (n >= (int64_t)1 << 31) return fail(FCLGPU_ERR_INVALID_ARGUMENT, "batch too large");
  if (req->precision != FCLGPU_PLAIN_FP64 && req->precision != FCLGPU_FP32_RECHECK)
    return fail(FCLGPU_ERR_INVALID_ARGUMENT, "unknown precision");
  if (req->enable_statistics) return fail(FCLGPU_ERR_UNSUPPORTED, "statistics are not produced with contacts");
  std::lock_guard<std::recursive_mutex> lk(g_mu);
  int rc = ensure_init();
  if (rc) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  int stack = 64;
  rc = prepare_tables(meshes, num_meshes, pairs_host, num_pairs, s, &stack);
  if (rc) return rc;
  res->total_contacts = 0;
  if (n == 0) {
    CK(cudaMemsetAsync(res->offsets, 0, sizeof(int64_t), s), "offsets");
    CK(cudaStreamSynchronize(s), "contacts");
    return FCLGPU_OK;
  }
  int64_t total = 0;
  rc = contacts_core(n, pair_of_query, tf1, tf2, req, stack, res->counts, res->offsets, s, &total);
  if (rc) return rc;
  res->total_contacts = total;
  if (!res->ids && !res->pos && !res->normal && !res->depth) return FCLGPU_OK;
  if (total > res->capacity) return fail(FCLGPU_ERR_CAPACITY, "contact buffers too small");
  rc = contacts_emit(res->offsets, res->ids, res->pos, res->normal, res->depth, s);
  if (rc) return rc;
  CK(cudaStreamSynchronize(s), "contacts");
  return FCLGPU_OK;
}

int fclgpu_collide_contacts(const fclgpu_mesh* meshes, int32_t num_meshes, const int32_t* pairs_host,
                            int32_t num_pairs, int64_t n, const int32_t* pair_of_query, const double* tf1,
                            const double* tf2, const fclgpu_collide_request* req, fclgpu_contact_result* res,
                            void* stream) {
  if (!req || !res || n < 0 || (n > 0 && (!tf2 || !res->counts)))
    return fail(FCLGPU_ERR_INVALID_ARGUMENT, "missing request, result, tf2 or counts");
  cudaStream_t s = (cudaStream_t)stream;
  Scratch& S = g_scratch;
  const size_t nn = (size_t)std::max<int64_t>(n, 1);
  std::lock_guard<std::recursive_mutex> lk(g_mu);
  {
    int rc = ensure_init();
    if (rc) return rc;
    if (pair_of_query) CK(S.in_pair.ensure(4 * nn), "inputs");
    if (tf1) CK(S.in_tf1.ensure(96 * nn), "inputs");
    CK(S.in_tf2.ensure(96 * nn), "inputs");
    CK(S.counts.ensure(4 * nn), "outputs");
    CK(S.offsets.ensure(8 * (nn + 1)), "outputs");
    if (n > 0) {
      if (pair_of_query) CK(cudaMemcpyAsync(S.in_pair.p, pair_of_query, 4 * n, cudaMemcpyHostToDevice, s), "h2d");
      if (tf1) CK(cudaMemcpyAsync(S.in_tf1.p, tf1, 96 * n, cudaMemcpyHostToDevice, s), "h2d");
      CK(cudaMemcpyAsync(S.in_tf2.p, tf2, 96 * n, cudaMemcpyHostToDevice, s), "h2d");
    }
  }
  fclgpu_contact_result dr{};
  dr.counts = (int32_t*)S.counts.p;
  dr.offsets = (int64_t*)S.offsets.p;
  int rc = fclgpu_collide_contacts_device(meshes, num_meshes, pairs_host, num_pairs, n,
                                          pair_of_query ? (const int32_t*)S.in_pair.p : nullptr,
                                          tf1 ? (const double*)S.in_tf1.p : nullptr, (const double*)S.in_tf2.p, req,
                                          &dr, stream);
  if (rc) return rc;
  const int64_t total = dr.total_contacts;
  res->total_contacts = total;
  const bool want = res->ids || res->pos || res->normal || res->depth;
  if (want && total > res->capacity) return fail(FCLGPU_ERR_CAPACITY, "contact buffers too small");
  if (want && total > 0) {
    // output scratch: ids 8 B, pos 24 B, normal 24 B, depth 8 B per contact
    const size_t nt = (size_t)total;
    CK(S.out_contacts.ensure(64 * nt), "contacts scratch");
    char* base = (char*)S.out_contacts.p;
    int32_t* ids = (int32_t*)base;
    double* pos = (double*)(base + 8 * nt);
    double* nrm = (double*)(base + 32 * nt);
    double* dep = (double*)(base + 56 * nt);
    rc = contacts_emit((const int64_t*)S.offsets.p, ids, pos, nrm, dep, s);
    if (rc) return rc;
    if (res->ids) CK(cudaMemcpyAsync(res->ids, ids, 8 * nt, cudaMemcpyDeviceToHost, s), "d2h");
    if (res->pos) CK(cudaMemcpyAsync(res->pos, pos, 24 * nt, cudaMemcpyDeviceToHost, s), "d2h");
    if (res->normal) CK(cudaMemcpyAsync(res->normal, nrm, 24 * nt, cudaMemcpyDeviceToHost, s), "d2h");
    if (res->depth) CK(cudaMemcpyAsync(res->depth, dep, 8 * nt, cudaMemcpyDeviceToHost, s), "d2h");
  }
  if (n > 0) {
    CK(cudaMemcpyAsync(res->counts, S.counts.p, 4 * n, cudaMemcpyDeviceToHost, s), "d2h");
    if (res->offsets) CK(cudaMemcpyAsync(res->offsets, S.offsets.p, 8 * (n + 1), cudaMemcpyDeviceToHost, s), "d2h");
  } else if (res->offsets) {
    res->offsets[0] = 0;
  }
  CK(cudaStreamSynchronize(s), "collide contacts");
  return FCLGPU_OK;
}

// ---- continuous collide (naive solver; translation, linear or screw motion) --------
namespace {
struct CcdScratch {
  DevBuf tfa, tfb, pq, counts, offsets, in_pq, in_a0, in_a1, in_b0, in_b1, out_hit, out_toc, out_tf1, out_tf2;
  DevBuf status, out_iter;
};
CcdScratch g_ccd;

int ccd_samples(const fclgpu_ccd_request* req, int64_t* n_iter) {
  if (req->solver_type != FCLGPU_CCDC_NAIVE && req->solver_type != FCLGPU_CCDC_CONSERVATIVE_ADVANCEMENT)
    return fail(FCLGPU_ERR_UNSUPPORTED,
                "only the naive and conservative-advancement continuous-collision solvers are on the GPU path");
  if (req->solver_type == FCLGPU_CCDC_CONSERVATIVE_ADVANCEMENT) {  // samples nothing; t_err is FCL's 1e-5
    if (req->motion_type != FCLGPU_CCDM_TRANS && req->motion_type != FCLGPU_CCDM_LINEAR &&
        req->motion_type != FCLGPU_CCDM_SCREW)
      return fail(FCLGPU_ERR_UNSUPPORTED, "the spline motion is not on the GPU path");
    *n_iter = 0;
    return FCLGPU_OK;
  }
  if (req->motion_type != FCLGPU_CCDM_TRANS && req->motion_type != FCLGPU_CCDM_LINEAR &&
      req->motion_type != FCLGPU_CCDM_SCREW)
    return fail(FCLGPU_ERR_UNSUPPORTED, "the spline motion is not on the GPU path");
  if (req->num_max_iterations < 0 || !(req->toc_err > 0))
    return fail(FCLGPU_ERR_INVALID_ARGUMENT, "num_max_iterations must be >= 0 and toc_err > 0");
  // continuous_collision-inl.h:144: min(num_max_iterations, (size_t)ceil(1 / toc_err))
  const double c = std::ceil(1.0 / req->toc_err);
  const int64_t k = c >= 9.0e18 ? INT64_MAX : (int64_t)c;
  *n_iter = std::min<int64_t>(req->num_max_iterations, k);
  if (*n_iter == 1) return fail(FCLGPU_ERR_INVALID_ARGUMENT, "one sample: FCL computes t = 0/0");
  return FCLGPU_OK;
}
}  // namespace

int fclgpu_continuous_collide_batch_device(const fclgpu_mesh* meshes, int32_t num_meshes, const int32_t* pairs_host,
                                           int32_t num_pairs, int64_t n, const int32_t* pair_of_query,
                                           const double* tf1_beg, const double* tf1_end, const double* tf2_beg,
                                           const double* tf2_end, const fclgpu_ccd_request* req,
                                           fclgpu_ccd_result* res, void* stream) {
  if (!req || !res || n < 0 || (n > 0 && (!tf2_beg || !tf2_end || !res->is_collide || !res->time_of_contact)))
    return fail(FCLGPU_ERR_INVALID_ARGUMENT, "missing request, result, tf2 or outputs");
  if ((tf1_beg == nullptr) != (tf1_end == nullptr))
    return fail(FCLGPU_ERR_INVALID_ARGUMENT, "tf1_beg and tf1_end must both be given or both be NULL");
  if (req->precision != FCLGPU_PLAIN_FP64 && req->precision != FCLGPU_FP32_RECHECK)
    return fail(FCLGPU_ERR_INVALID_ARGUMENT, "unknown precision");
  int64_t n_iter = 0;
  int rc = ccd_samples(req, &n_iter);
  if (rc) return rc;
  if (req->solver_type == FCLGPU_CCDC_CONSERVATIVE_ADVANCEMENT) {
    if (n >= (int64_t)1 << 31) return fail(FCLGPU_ERR_INVALID_ARGUMENT, "batch too large");
    std::lock_guard<std::recursive_mutex> lk(g_mu);
    rc = ensure_init();
    if (rc) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    int stack = 64;
    rc = prepare_tables(meshes, num_meshes, pairs_host, num_pairs, s, &stack);
    if (rc) return rc;
    if (n == 0) return FCLGPU_OK;
    CK(g_ccd.counts.ensure(4 * (size_t)n), "ccd scratch");
    CK(g_ccd.offsets.ensure(8 * (size_t)(n + 1)), "ccd scratch");
    CK(g_ccd.status.ensure(4), "ccd scratch");
    CK(cudaMemsetAsync(g_ccd.status.p, 0, 4, s), "ccd scratch");
    // the discrete collide at the start poses (the motions' transforms before integrate)
    fclgpu_collide_request cr{};
    cr.num_max_contacts = 1;
    cr.precision = req->precision;
    int64_t total = 0;
    rc = collide_core(n, pair_of_query, tf1_beg, tf2_beg, &cr, (int32_t*)g_ccd.counts.p, (int64_t*)g_ccd.offsets.p,
                      nullptr, nullptr, nullptr, stack, s, &total);
    if (rc) return rc;
    CcdLaunch L{};
    L.pair_of_query = pair_of_query;
    L.tf1_beg = tf1_beg;
    L.tf1_end = tf1_end;
    L.tf2_beg = tf2_beg;
    L.tf2_end = tf2_end;
    L.n = n;
    L.motion = req->motion_type;
    L.is_collide = res->is_collide;
    L.toc = res->time_of_contact;
    L.contact_tf1 = res->contact_tf1;
    L.contact_tf2 = res->contact_tf2;
    L.meshes = (const DevMesh*)g_scratch.meshes.p;
    L.pairs = (const int2*)g_scratch.pairs.p;
    L.num_pairs = num_pairs;
    L.hit0 = (const int32_t*)g_ccd.counts.p;
    // each iteration that does not end the loop advances t by more than 1e-5
    L.max_iterations = 200000;
    L.iterations = res->iterations;
    L.status = (unsigned*)g_ccd.status.p;
    CK(launch_ccd_ca(L, stack, s), "conservative advancement");
    unsigned st = 0;
    CK(cudaMemcpyAsync(&st, g_ccd.status.p, 4, cudaMemcpyDeviceToHost, s), "status");
    CK(cudaStreamSynchronize(s), "conservative advancement");
    if (st & DEV_ERR_PAIR) return fail(FCLGPU_ERR_DEVICE_STATUS, "a query's pair index lies outside the pair table");
    if (st & DEV_ERR_STACK) return fail(FCLGPU_ERR_DEVICE_STATUS, "traversal stack overflow");
    if (st & DEV_ERR_ITERATIONS) return fail(FCLGPU_ERR_DEVICE_STATUS, "conservative advancement iteration cap");
    return FCLGPU_OK;
  }
  if (n * std::max<int64_t>(n_iter, 1) >= (int64_t)1 << 31)
    return fail(FCLGPU_ERR_INVALID_ARGUMENT, "queries x samples must stay below 2^31");
  std::lock_guard<std::recursive_mutex> lk(g_mu);
  rc = ensure_init();
  if (rc) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  int stack = 64;
  rc = prepare_tables(meshes, num_meshes, pairs_host, num_pairs, s, &stack);
  if (rc) return rc;
  if (n == 0) return FCLGPU_OK;
  CcdLaunch L{};
  L.pair_of_query = pair_of_query;
  L.tf1_beg = tf1_beg;
  L.tf1_end = tf1_end;
  L.tf2_beg = tf2_beg;
  L.tf2_end = tf2_end;
  L.n = n;
  L.n_iter = n_iter;
  L.motion = req->motion_type;
  L.is_collide = res->is_collide;
  L.toc = res->time_of_contact;
  L.contact_tf1 = res->contact_tf1;
  L.contact_tf2 = res->contact_tf2;
  if (n_iter == 0) {  // no sample: is_collide = false, time_of_contact = 1
    CK(g_ccd.counts.ensure(4), "ccd scratch");
    CK(launch_ccd_reduce(L, (const int32_t*)g_ccd.counts.p, s), "ccd reduce");
    CK(cudaStreamSynchronize(s), "ccd");
    return FCLGPU_OK;
  }
  const size_t N = (size_t)(n * n_iter);
  CK(g_ccd.tfa.ensure(96 * N), "ccd scratch");
  CK(g_ccd.tfb.ensure(96 * N), "ccd scratch");
  CK(g_ccd.pq.ensure(4 * N), "ccd scratch");
  CK(g_ccd.counts.ensure(4 * N), "ccd scratch");
  CK(g_ccd.offsets.ensure(8 * (N + 1)), "ccd scratch");
  L.tfa = (double*)g_ccd.tfa.p;
  L.tfb = (double*)g_ccd.tfb.p;
  L.pq_expanded = (int32_t*)g_ccd.pq.p;
  CK(launch_ccd_poses(L, s), "ccd poses");
  // the discrete collides: default CollisionRequest (one contact, no contact geometry)
  fclgpu_collide_request cr{};
  cr.num_max_contacts = 1;
  cr.precision = req->precision;
  int64_t total = 0;
  rc = collide_core((int64_t)N, L.pq_expanded, L.tfa, L.tfb, &cr, (int32_t*)g_ccd.counts.p,
                    (int64_t*)g_ccd.offsets.p, nullptr, nullptr, nullptr, stack, s, &total);
  if (rc) return rc;
  CK(launch_ccd_reduce(L, (const int32_t*)g_ccd.counts.p, s), "ccd reduce");
  CK(cudaStreamSynchronize(s), "ccd");
  return FCLGPU_OK;
}

int fclgpu_continuous_collide_batch(const fclgpu_mesh* meshes, int32_t num_meshes, const int32_t* pairs_host,
                                    int32_t num_pairs, int64_t n, const int32_t* pair_of_query,
                                    const double* tf1_beg, const double* tf1_end, const double* tf2_beg,
                                    const double* tf2_end, const fclgpu_ccd_request* req, fclgpu_ccd_result* res,
                                    void* stream) {
  if (!req || !res || n < 0 || (n > 0 && (!tf2_beg || !tf2_end || !res->is_collide || !res->time_of_contact)))
    return fail(FCLGPU_ERR_INVALID_ARGUMENT, "missing request, result, tf2 or outputs");
  cudaStream_t s = (cudaStream_t)stream;
  CcdScratch& G = g_ccd;
  const size_t nn = (size_t)std::max<int64_t>(n, 1);
  std::lock_guard<std::recursive_mutex> lk(g_mu);
  int rc = ensure_init();
  if (rc) return rc;
  if (pair_of_query) CK(G.in_pq.ensure(4 * nn), "inputs");
  if (tf1_beg) CK(G.in_a0.ensure(96 * nn), "inputs");
  if (tf1_end) CK(G.in_a1.ensure(96 * nn), "inputs");
  CK(G.in_b0.ensure(96 * nn), "inputs");
  CK(G.in_b1.ensure(96 * nn), "inputs");
  CK(G.out_hit.ensure(4 * nn), "outputs");
  CK(G.out_toc.ensure(8 * nn), "outputs");
  CK(G.out_tf1.ensure(96 * nn), "outputs");
  CK(G.out_tf2.ensure(96 * nn), "outputs");
  if (n > 0) {
    if (pair_of_query) CK(cudaMemcpyAsync(G.in_pq.p, pair_of_query, 4 * n, cudaMemcpyHostToDevice, s), "h2d");
    if (tf1_beg) CK(cudaMemcpyAsync(G.in_a0.p, tf1_beg, 96 * n, cudaMemcpyHostToDevice, s), "h2d");
    if (tf1_end) CK(cudaMemcpyAsync(G.in_a1.p, tf1_end, 96 * n, cudaMemcpyHostToDevice, s), "h2d");
    CK(cudaMemcpyAsync(G.in_b0.p, tf2_beg, 96 * n, cudaMemcpyHostToDevice, s), "h2d");
    CK(cudaMemcpyAsync(G.in_b1.p, tf2_end, 96 * n, cudaMemcpyHostToDevice, s), "h2d");
    // entries of non-colliding queries are left unchanged: start from the caller's values
    if (res->contact_tf1) CK(cudaMemcpyAsync(G.out_tf1.p, res->contact_tf1, 96 * n, cudaMemcpyHostToDevice, s), "h2d");
    if (res->contact_tf2) CK(cudaMemcpyAsync(G.out_tf2.p, res->contact_tf2, 96 * n, cudaMemcpyHostToDevice, s), "h2d");
  }
  fclgpu_ccd_result dr{};
  dr.is_collide = (int32_t*)G.out_hit.p;
  dr.time_of_contact = (double*)G.out_toc.p;
  dr.contact_tf1 = res->contact_tf1 ? (double*)G.out_tf1.p : nullptr;
  dr.contact_tf2 = res->contact_tf2 ? (double*)G.out_tf2.p : nullptr;
  if (res->iterations) {
    CK(G.out_iter.ensure(4 * nn), "outputs");
    dr.iterations = (int32_t*)G.out_iter.p;
  }
  rc = fclgpu_continuous_collide_batch_device(meshes, num_meshes, pairs_host, num_pairs, n,
                                              pair_of_query ? (const int32_t*)G.in_pq.p : nullptr,
                                              tf1_beg ? (const double*)G.in_a0.p : nullptr,
                                              tf1_end ? (const double*)G.in_a1.p : nullptr,
                                              (const double*)G.in_b0.p, (const double*)G.in_b1.p, req, &dr, stream);
  if (rc) return rc;
  if (n > 0) {
    CK(cudaMemcpyAsync(res->is_collide, G.out_hit.p, 4 * n, cudaMemcpyDeviceToHost, s), "d2h");
    CK(cudaMemcpyAsync(res->time_of_contact, G.out_toc.p, 8 * n, cudaMemcpyDeviceToHost, s), "d2h");
    if (res->contact_tf1) CK(cudaMemcpyAsync(res->contact_tf1, G.out_tf1.p, 96 * n, cudaMemcpyDeviceToHost, s), "d2h");
    if (res->contact_tf2) CK(cudaMemcpyAsync(res->contact_tf2, G.out_tf2.p, 96 * n, cudaMemcpyDeviceToHost, s), "d2h");
    if (res->iterations) CK(cudaMemcpyAsync(res->iterations, dr.iterations, 4 * n, cudaMemcpyDeviceToHost, s), "d2h");
  }
  CK(cudaStreamSynchronize(s), "continuous collide");
  return FCLGPU_OK;
}

int fclgpu_distance_batch_device(const fclgpu_mesh* meshes, int32_t num_meshes, const int32_t* pairs_host,
                                 int32_t num_pairs, int64_t n, const int32_t* pair_of_query, const double* tf1,
                                 const double* tf2, const fclgpu_distance_request* req, fclgpu_distance_result* res,
                                 void* stream) {
  if (!req || !res || n < 0 || (n > 0 && (!tf2 || !res->min_distance)))
    return fail(FCLGPU_ERR_INVALID_ARGUMENT, "missing request, result, tf2 or min_distance");
  if (req->precision != FCLGPU_PLAIN_FP64 && req->precision != FCLGPU_FP32_RECHECK)
    return fail(FCLGPU_ERR_INVALID_ARGUMENT, "unknown precision");
  std::lock_guard<std::recursive_mutex> lk(g_mu);
  int rc = ensure_init();
  if (rc) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  int stack = 64;
  rc = prepare_tables(meshes, num_meshes, pairs_host, num_pairs, s, &stack);
  if (rc) return rc;
  if (n == 0) return FCLGPU_OK;
  Scratch& S = g_scratch;
  CK(S.ctr.ensure(sizeof(BatchCounters)), "counters");
  CK(cudaMemsetAsync(S.ctr.p, 0, sizeof(BatchCounters), s), "counters");
  DistanceLaunch L;
  L.meshes = (const DevMesh*)S.meshes.p;
  L.pairs = (const int2*)S.pairs.p;
  L.num_pairs = num_pairs;
  L.pair_of_query = pair_of_query;
  L.tf1 = tf1;
  L.tf2 = tf2;
  L.n = n;
  L.nearest = req->enable_nearest_points;
  L.want_stats = req->enable_statistics;
  L.ctr = (BatchCounters*)S.ctr.p;
  L.dist = res->min_distance;
  L.ids = res->ids;
  L.points = res->nearest_points;
  L.margins = res->margins;
  L.within = res->within_margin;
  L.nbv = res->num_bv_tests;
  L.nleaf = res->num_leaf_tests;
  L.nrecheck = res->num_rechecks;
  const int block = 128;
  const int grid = distance_grid(req->precision, stack, block);
  rc = ensure_events();
  if (rc) return rc;
  CK(cudaEventRecord(g_ev[0], s), "event");
  CK(launch_mesh_distance(L, req->precision, stack, grid, block, s), "distance kernel");
  CK(cudaEventRecord(g_ev[1], s), "event");
  BatchCounters hc;
  CK(cudaMemcpyAsync(&hc, S.ctr.p, sizeof(hc), cudaMemcpyDeviceToHost, s), "read counters");
  CK(cudaStreamSynchronize(s), "distance kernel");
  {
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, g_ev[0], g_ev[1]), "event");
    g_last_kernel_ms = ms;
  }
  if (hc.status) return fail(FCLGPU_ERR_DEVICE_STATUS, "distance kernel status word set");
  return FCLGPU_OK;
}

int fclgpu_distance_batch(const fclgpu_mesh* meshes, int32_t num_meshes, const int32_t* pairs_host,
                          int32_t num_pairs, int64_t n, const int32_t* pair_of_query, const double* tf1,
                          const double* tf2, const fclgpu_distance_request* req, fclgpu_distance_result* res,
                          void* stream) {
  if (!req || !res || n < 0 || (n > 0 && (!tf2 || !res->min_distance)))
    return fail(FCLGPU_ERR_INVALID_ARGUMENT, "missing request, result, tf2 or min_distance");
  cudaStream_t s = (cudaStream_t)stream;
  Scratch& S = g_scratch;
  const size_t nn = (size_t)std::max<int64_t>(n, 1);
  std::lock_guard<std::recursive_mutex> lk(g_mu);
  {
    int rc = ensure_init();
    if (rc) return rc;
    if (pair_of_query) CK(S.in_pair.ensure(4 * nn), "inputs");
    if (tf1) CK(S.in_tf1.ensure(96 * nn), "inputs");
    CK(S.in_tf2.ensure(96 * nn), "inputs");
    if (res->margins) CK(S.in_margin.ensure(8 * nn), "inputs");
    CK(S.out_dist.ensure(8 * nn), "outputs");
    if (res->ids) CK(S.out_ids.ensure(8 * nn), "outputs");
    if (res->nearest_points) CK(S.out_pts.ensure(48 * nn), "outputs");
    if (res->within_margin) CK(S.out_within.ensure(4 * nn), "outputs");
    if (res->num_bv_tests) CK(S.out_nbv.ensure(8 * nn), "outputs");
    if (res->num_leaf_tests) CK(S.out_nleaf.ensure(8 * nn), "outputs");
    if (res->num_rechecks) CK(S.out_nrc.ensure(8 * nn), "outputs");
    if (pair_of_query) CK(cudaMemcpyAsync(S.in_pair.p, pair_of_query, 4 * n, cudaMemcpyHostToDevice, s), "h2d");
    if (tf1) CK(cudaMemcpyAsync(S.in_tf1.p, tf1, 96 * n, cudaMemcpyHostToDevice, s), "h2d");
    CK(cudaMemcpyAsync(S.in_tf2.p, tf2, 96 * n, cudaMemcpyHostToDevice, s), "h2d");
    if (res->margins) CK(cudaMemcpyAsync(S.in_margin.p, res->margins, 8 * n, cudaMemcpyHostToDevice, s), "h2d");
  }
  fclgpu_distance_result dr;
  dr.min_distance = (double*)S.out_dist.p;
  dr.ids = res->ids ? (int32_t*)S.out_ids.p : nullptr;
  dr.nearest_points = res->nearest_points ? (double*)S.out_pts.p : nullptr;
  dr.margins = res->margins ? (const double*)S.in_margin.p : nullptr;
  dr.within_margin = res->within_margin ? (int32_t*)S.out_within.p : nullptr;
  dr.num_bv_tests = res->num_bv_tests ? (int64_t*)S.out_nbv.p : nullptr;
  dr.num_leaf_tests = res->num_leaf_tests ? (int64_t*)S.out_nleaf.p : nullptr;
  dr.num_rechecks = res->num_rechecks ? (int64_t*)S.out_nrc.p : nullptr;
  int rc = fclgpu_distance_batch_device(meshes, num_meshes, pairs_host, num_pairs, n,
                                        pair_of_query ? (const int32_t*)S.in_pair.p : nullptr,
                                        tf1 ? (const double*)S.in_tf1.p : nullptr, (const double*)S.in_tf2.p, req,
                                        &dr, stream);
  if (rc) return rc;
  CK(cudaMemcpyAsync(res->min_distance, dr.min_distance, 8 * n, cudaMemcpyDeviceToHost, s), "d2h");
  if (res->ids) CK(cudaMemcpyAsync(res->ids, dr.ids, 8 * n, cudaMemcpyDeviceToHost, s), "d2h");
  if (res->nearest_points)
    CK(cudaMemcpyAsync(res->nearest_points, dr.nearest_points, 48 * n, cudaMemcpyDeviceToHost, s), "d2h");
  if (res->within_margin)
    CK(cudaMemcpyAsync(res->within_margin, dr.within_margin, 4 * n, cudaMemcpyDeviceToHost, s), "d2h");
  if (res->num_bv_tests) CK(cudaMemcpyAsync(res->num_bv_tests, dr.num_bv_tests, 8 * n, cudaMemcpyDeviceToHost, s), "d2h");
  if (res->num_leaf_tests)
    CK(cudaMemcpyAsync(res->num_leaf_tests, dr.num_leaf_tests, 8 * n, cudaMemcpyDeviceToHost, s), "d2h");
  if (res->num_rechecks) CK(cudaMemcpyAsync(res->num_rechecks, dr.num_rechecks, 8 * n, cudaMemcpyDeviceToHost, s), "d2h");
  CK(cudaStreamSynchronize(s), "distance batch");
  return FCLGPU_OK;
}

// ---------------------------------------------------------------------------------
// Front-list collide (mesh_front.cu): a count launch, scans, a fill launch.
// ---------------------------------------------------------------------------------
}  // extern "C"

namespace {
struct FrontScratch {
  DevBuf ncont, nseg, flen, status, scan_tmp, coff, foff;
  DevBuf in_pq, in_tf1, in_tf2, in_foff, in_front, out_counts, out_coff, out_cont, out_foff, out_front, out_nbv,
      out_nleaf;
};
FrontScratch g_front;
}  // namespace

extern "C" {

int fclgpu_collide_front_batch_device(const fclgpu_mesh* meshes, int32_t num_meshes, const int32_t* pairs_host,
                                      int32_t num_pairs, int64_t n, const int32_t* pair_of_query, const double* tf1,
                                      const double* tf2, const int64_t* front_in_offsets, const int32_t* front_in,
                                      const fclgpu_front_request* req, fclgpu_front_result* res, void* stream) {
  if (!req || !res || n < 0 || (n > 0 && (!tf2 || !res->counts || !res->contact_offsets || !res->front_offsets)))
    return fail(FCLGPU_ERR_INVALID_ARGUMENT, "missing request, result, tf2 or outputs");
  if (n >= (int64_t)1 << 31) return fail(FCLGPU_ERR_INVALID_ARGUMENT, "batch too large");
  if (req->num_max_contacts < 1) return fail(FCLGPU_ERR_INVALID_ARGUMENT, "num_max_contacts must be >= 1");
  if (req->precision != FCLGPU_PLAIN_FP64 && req->precision != FCLGPU_FP32_RECHECK)
    return fail(FCLGPU_ERR_INVALID_ARGUMENT, "unknown precision");
  if ((front_in_offsets == nullptr) != (front_in == nullptr))
    return fail(FCLGPU_ERR_INVALID_ARGUMENT, "front_in_offsets and front_in go together");
  if ((res->contacts_capacity > 0 && !res->contacts) || (res->front_capacity > 0 && !res->front) ||
      res->contacts_capacity < 0 || res->front_capacity < 0)
    return fail(FCLGPU_ERR_INVALID_ARGUMENT, "missing contact or front buffer");
  std::lock_guard<std::recursive_mutex> lk(g_mu);
  int rc = ensure_init();
  if (rc) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  int stack = 64;
  rc = prepare_tables(meshes, num_meshes, pairs_host, num_pairs, s, &stack);
  if (rc) return rc;
  res->total_contacts = 0;
  res->total_front = 0;
  if (n == 0) {
    CK(cudaMemsetAsync(res->contact_offsets, 0, 8, s), "offsets");
    CK(cudaMemsetAsync(res->front_offsets, 0, 8, s), "offsets");
    CK(cudaStreamSynchronize(s), "front collide");
    return FCLGPU_OK;
  }
  FrontScratch& F = g_front;
  const size_t nn = (size_t)n;
  CK(F.nseg.ensure(12 * nn), "front scratch");
  CK(F.flen.ensure(4 * nn), "front scratch");
  CK(F.status.ensure(4), "front scratch");
  CK(F.scan_tmp.ensure(sizeof(int64_t) * (size_t)(2 * ((n + 4095) / 4096) + 4)), "scan scratch");
  CK(cudaMemsetAsync(F.status.p, 0, 4, s), "front scratch");
  FrontLaunch L{};
  L.meshes = (const DevMesh*)g_scratch.meshes.p;
  L.pairs = (const int2*)g_scratch.pairs.p;
  L.num_pairs = num_pairs;
  L.pair_of_query = pair_of_query;
  L.tf1 = tf1;
  L.tf2 = tf2;
  L.n = n;
  L.num_max_contacts = req->num_max_contacts;
  L.front_in_off = front_in_offsets;
  L.front_in = front_in;
  L.ncont = res->counts;
  L.nseg = (int32_t*)F.nseg.p;
  L.status = (unsigned*)F.status.p;
  CK(launch_collide_front(L, req->precision, stack, false, s), "front count");
  CK(launch_exclusive_scan(res->counts, n, res->contact_offsets, (int64_t*)F.scan_tmp.p, s), "scan");
  CK(launch_front_lengths(L.nseg, n, (int32_t*)F.flen.p, s), "front lengths");
  CK(launch_exclusive_scan((const int32_t*)F.flen.p, n, res->front_offsets, (int64_t*)F.scan_tmp.p, s), "scan");
  int64_t tot[2] = {0, 0};
  unsigned st = 0;
  CK(cudaMemcpyAsync(&tot[0], res->contact_offsets + n, 8, cudaMemcpyDeviceToHost, s), "totals");
  CK(cudaMemcpyAsync(&tot[1], res->front_offsets + n, 8, cudaMemcpyDeviceToHost, s), "totals");
  CK(cudaMemcpyAsync(&st, F.status.p, 4, cudaMemcpyDeviceToHost, s), "status");
  CK(cudaStreamSynchronize(s), "front count");
  if (st & DEV_ERR_PAIR) return fail(FCLGPU_ERR_DEVICE_STATUS, "a query's pair index lies outside the pair table");
  if (st & DEV_ERR_STACK) return fail(FCLGPU_ERR_DEVICE_STATUS, "traversal stack overflow");
  res->total_contacts = tot[0];
  res->total_front = tot[1];
  if (tot[0] > res->contacts_capacity || tot[1] > res->front_capacity)
    return fail(FCLGPU_ERR_CAPACITY, "contact or front buffer too small");
  L.cont_off = res->contact_offsets;
  L.contacts = res->contacts;
  L.front_out_off = res->front_offsets;
  L.front_out = res->front;
  L.nbv = res->num_bv_tests;
  L.nleaf = res->num_leaf_tests;
  CK(launch_collide_front(L, req->precision, stack, true, s), "front fill");
  CK(cudaStreamSynchronize(s), "front fill");
  return FCLGPU_OK;
}

int fclgpu_collide_front_batch(const fclgpu_mesh* meshes, int32_t num_meshes, const int32_t* pairs_host,
                               int32_t num_pairs, int64_t n, const int32_t* pair_of_query, const double* tf1,
                               const double* tf2, const int64_t* front_in_offsets, const int32_t* front_in,
                               const fclgpu_front_request* req, fclgpu_front_result* res, void* stream) {
  if (!req || !res || n < 0 || (n > 0 && (!tf2 || !res->counts || !res->contact_offsets || !res->front_offsets)))
    return fail(FCLGPU_ERR_INVALID_ARGUMENT, "missing request, result, tf2 or outputs");
  if ((front_in_offsets == nullptr) != (front_in == nullptr))
    return fail(FCLGPU_ERR_INVALID_ARGUMENT, "front_in_offsets and front_in go together");
  if ((res->contacts_capacity > 0 && !res->contacts) || (res->front_capacity > 0 && !res->front) ||
      res->contacts_capacity < 0 || res->front_capacity < 0)
    return fail(FCLGPU_ERR_INVALID_ARGUMENT, "missing contact or front buffer");
  cudaStream_t s = (cudaStream_t)stream;
  FrontScratch& F = g_front;
  const size_t nn = (size_t)std::max<int64_t>(n, 1);
  std::lock_guard<std::recursive_mutex> lk(g_mu);
  int rc = ensure_init();
  if (rc) return rc;
  const int64_t nfin = front_in_offsets && n > 0 ? front_in_offsets[n] : 0;
  if (nfin < 0) return fail(FCLGPU_ERR_INVALID_ARGUMENT, "negative front length");
  if (pair_of_query) CK(F.in_pq.ensure(4 * nn), "inputs");
  if (tf1) CK(F.in_tf1.ensure(96 * nn), "inputs");
  CK(F.in_tf2.ensure(96 * nn), "inputs");
  if (front_in) {
    CK(F.in_foff.ensure(8 * (nn + 1)), "inputs");
    CK(F.in_front.ensure(8 * (size_t)std::max<int64_t>(nfin, 1)), "inputs");
  }
  CK(F.out_counts.ensure(4 * nn), "outputs");
  CK(F.out_coff.ensure(8 * (nn + 1)), "outputs");
  CK(F.out_foff.ensure(8 * (nn + 1)), "outputs");
  CK(F.out_cont.ensure(8 * (size_t)std::max<int64_t>(res->contacts_capacity, 1)), "outputs");
  CK(F.out_front.ensure(8 * (size_t)std::max<int64_t>(res->front_capacity, 1)), "outputs");
  if (res->num_bv_tests) CK(F.out_nbv.ensure(8 * nn), "outputs");
  if (res->num_leaf_tests) CK(F.out_nleaf.ensure(8 * nn), "outputs");
  if (n > 0) {
    if (pair_of_query) CK(cudaMemcpyAsync(F.in_pq.p, pair_of_query, 4 * n, cudaMemcpyHostToDevice, s), "h2d");
    if (tf1) CK(cudaMemcpyAsync(F.in_tf1.p, tf1, 96 * n, cudaMemcpyHostToDevice, s), "h2d");
    CK(cudaMemcpyAsync(F.in_tf2.p, tf2, 96 * n, cudaMemcpyHostToDevice, s), "h2d");
    if (front_in) {
      CK(cudaMemcpyAsync(F.in_foff.p, front_in_offsets, 8 * (n + 1), cudaMemcpyHostToDevice, s), "h2d");
      if (nfin > 0) CK(cudaMemcpyAsync(F.in_front.p, front_in, 8 * nfin, cudaMemcpyHostToDevice, s), "h2d");
    }
  }
  fclgpu_front_result dr{};
  dr.counts = (int32_t*)F.out_counts.p;
  dr.contact_offsets = (int64_t*)F.out_coff.p;
  dr.contacts = (int32_t*)F.out_cont.p;
  dr.contacts_capacity = res->contacts_capacity;
  dr.front_offsets = (int64_t*)F.out_foff.p;
  dr.front = (int32_t*)F.out_front.p;
  dr.front_capacity = res->front_capacity;
  dr.num_bv_tests = res->num_bv_tests ? (int64_t*)F.out_nbv.p : nullptr;
  dr.num_leaf_tests = res->num_leaf_tests ? (int64_t*)F.out_nleaf.p : nullptr;
  rc = fclgpu_collide_front_batch_device(meshes, num_meshes, pairs_host, num_pairs, n,
                                         pair_of_query ? (const int32_t*)F.in_pq.p : nullptr,
                                         tf1 ? (const double*)F.in_tf1.p : nullptr, (const double*)F.in_tf2.p,
                                         front_in ? (const int64_t*)F.in_foff.p : nullptr,
                                         front_in ? (const int32_t*)F.in_front.p : nullptr, req, &dr, stream);
  res->total_contacts = dr.total_contacts;
  res->total_front = dr.total_front;
  if (rc != FCLGPU_OK && rc != FCLGPU_ERR_CAPACITY) return rc;
  if (n > 0) {
    CK(cudaMemcpyAsync(res->counts, dr.counts, 4 * n, cudaMemcpyDeviceToHost, s), "d2h");
    CK(cudaMemcpyAsync(res->contact_offsets, dr.contact_offsets, 8 * (n + 1), cudaMemcpyDeviceToHost, s), "d2h");
    CK(cudaMemcpyAsync(res->front_offsets, dr.front_offsets, 8 * (n + 1), cudaMemcpyDeviceToHost, s), "d2h");
  } else {
    res->contact_offsets[0] = 0;
    res->front_offsets[0] = 0;
  }
  if (rc == FCLGPU_OK && n > 0) {
    if (dr.total_contacts > 0)
      CK(cudaMemcpyAsync(res->contacts, dr.contacts, 8 * dr.total_contacts, cudaMemcpyDeviceToHost, s), "d2h");
    if (dr.total_front > 0)
      CK(cudaMemcpyAsync(res->front, dr.front, 8 * dr.total_front, cudaMemcpyDeviceToHost, s), "d2h");
    if (res->num_bv_tests) CK(cudaMemcpyAsync(res->num_bv_tests, dr.num_bv_tests, 8 * n, cudaMemcpyDeviceToHost, s), "d2h");
    if (res->num_leaf_tests)
      CK(cudaMemcpyAsync(res->num_leaf_tests, dr.num_leaf_tests, 8 * n, cudaMemcpyDeviceToHost, s), "d2h");
  }
  CK(cudaStreamSynchronize(s), "front collide");
  return rc;
}

}  // extern "C"
