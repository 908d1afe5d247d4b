// Batched mesh distance that allocates no memory.
//
// Who needs it: callers that must not (or cannot) allocate GPU memory at query time.
// A motion-planning or control loop with a hard per-cycle deadline cannot afford the
// synchronisation and unbounded latency of cudaMalloc/cudaFree; a process whose device
// memory is owned by another allocator (a framework's caching allocator that has
// reserved the free HBM, or a memory pool shared with other work) may see cudaMalloc
// fail or fragment that pool.  fclgpu_distance_batch_device grows internal scratch with
// cudaMalloc on first use; this entry point never does.
//
// How: the only scratch the distance kernel needs -- the work counter and status word,
// and the mesh and pair tables it reads -- lives in one file-scope __device__ array of
// fixed size (every GPU that loads the library keeps it until the process exits).  The
// caller passes all per-query inputs and outputs.  Limits: at most kNoAllocMaxMeshes
// meshes and kNoAllocMaxPairs pairs per call; larger requests are rejected with
// FCLGPU_ERR_INVALID_ARGUMENT before any work is queued.
//
// Sharing: every call uses the same array and leaves its contents behind; the counter
// is cleared at the start of each call.  Calls that overlap on the GPU (from several
// host threads, or on several streams without ordering between them) race on the
// array, so they must be serialised by the caller.
//
// Set-up: the first call on a device, with that device current, looks up the array's
// device address with cudaGetSymbolAddress (the host-side name of a __device__ variable
// is not a device address) and caches it for that device; make that first call before
// starting any stream capture.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "../../include/fclgpu.h"
#include "kernels.h"
#include "mesh_handle.h"

using namespace fclgpu;

namespace fclgpu {
void set_error_detail(const std::string& what);
}

namespace {

constexpr int kNoAllocMaxMeshes = 64;
constexpr int kNoAllocMaxPairs = 256;
constexpr int kNoAllocMaxDevices = 64;

struct NoAllocScratch {
  BatchCounters ctr;
  DevMesh meshes[kNoAllocMaxMeshes];
  int2 pairs[kNoAllocMaxPairs];
};

// 256-byte aligned so the counters and tables start on their natural boundaries.
static __device__ __align__(256) unsigned char g_noalloc_scratch[sizeof(NoAllocScratch)];

std::mutex g_noalloc_mu;
void* g_noalloc_ptr[kNoAllocMaxDevices] = {};

// Every error return sets the per-thread detail message (fclgpu_last_error_detail).
int fail(int code, const char* why) {
  set_error_detail(std::string("fclgpu_distance_batch_noalloc: ") + why);
  return code;
}
int cuda_fail(cudaError_t e, const char* where) {
  set_error_detail(std::string("fclgpu_distance_batch_noalloc: ") + where + ": " + cudaGetErrorString(e));
  return FCLGPU_ERR_CUDA;
}

}  // namespace

extern "C" int fclgpu_distance_batch_noalloc(const fclgpu_mesh* meshes, int32_t num_meshes,
                                             const int32_t* pairs_host, int32_t num_pairs, int64_t n,
                                             const int32_t* pair_of_query, const double* tf1, const double* tf2,
                                             const fclgpu_distance_request* req, fclgpu_distance_result* res,
                                             void* stream) {
  if (!req || !res || n < 0 || (n > 0 && (!tf2 || !res->min_distance)))
    return fail(FCLGPU_ERR_INVALID_ARGUMENT, "missing request, result, tf2 or min_distance");
  if (req->precision != FCLGPU_PLAIN_FP64 && req->precision != FCLGPU_FP32_RECHECK)
    return fail(FCLGPU_ERR_INVALID_ARGUMENT, "unknown precision");
  if (!meshes || num_meshes <= 0 || num_meshes > kNoAllocMaxMeshes)
    return fail(FCLGPU_ERR_INVALID_ARGUMENT, "needs 1 to 64 meshes per call");
  if (!pairs_host || num_pairs <= 0 || num_pairs > kNoAllocMaxPairs)
    return fail(FCLGPU_ERR_INVALID_ARGUMENT, "needs 1 to 256 pairs per call");
  // tables are staged in fixed-size host arrays (no heap allocation either)
  DevMesh tab[kNoAllocMaxMeshes];
  int2 pr[kNoAllocMaxPairs];
  int need = 0;
  for (int i = 0; i < num_meshes; ++i) {
    if (!meshes[i]) return fail(FCLGPU_ERR_INVALID_ARGUMENT, "null mesh handle");
    tab[i] = meshes[i]->dev;
  }
  for (int p = 0; p < num_pairs; ++p) {
    const int a = pairs_host[2 * p], b = pairs_host[2 * p + 1];
    if (a < 0 || a >= num_meshes || b < 0 || b >= num_meshes)
      return fail(FCLGPU_ERR_INVALID_ARGUMENT, "pair index out of range");
    pr[p] = make_int2(a, b);
    const int d = tab[a].max_depth + tab[b].max_depth + 2;
    need = d > need ? d : need;
  }
  if (need > 256) return fail(FCLGPU_ERR_STACK_DEPTH, "BVH pair deeper than 256 levels");
  const int stack = need <= 64 ? 64 : 256;
  if (n == 0) return FCLGPU_OK;

  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
  if (dev < 0 || dev >= kNoAllocMaxDevices) return fail(FCLGPU_ERR_CUDA, "device ordinal beyond 63");
  void* base = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
      void* p = nullptr;
      const cudaError_t es = cudaGetSymbolAddress(&p, g_noalloc_scratch);
      if (es != cudaSuccess) return cuda_fail(es, "cudaGetSymbolAddress");
      if (!p) return fail(FCLGPU_ERR_CUDA, "cudaGetSymbolAddress returned null");
      g_noalloc_ptr[dev] = p;
    }
    base = g_noalloc_ptr[dev];
  }
  NoAllocScratch* S = static_cast<NoAllocScratch*>(base);
  cudaStream_t s = (cudaStream_t)stream;
  if ((e = cudaMemsetAsync(&S->ctr, 0, sizeof(BatchCounters), s)) != cudaSuccess) return cuda_fail(e, "clear counters");
  if ((e = cudaMemcpyAsync(S->meshes, tab, sizeof(DevMesh) * num_meshes, cudaMemcpyHostToDevice, s)) != cudaSuccess)
    return cuda_fail(e, "stage mesh table");
  if ((e = cudaMemcpyAsync(S->pairs, pr, sizeof(int2) * num_pairs, cudaMemcpyHostToDevice, s)) != cudaSuccess)
    return cuda_fail(e, "stage pair table");

  DistanceLaunch L;
  L.meshes = S->meshes;
  L.pairs = S->pairs;
  L.num_pairs = num_pairs;
  L.pair_of_query = pair_of_query;
  L.tf1 = tf1;
  L.tf2 = tf2;
  L.n = n;
  L.nearest = req->enable_nearest_points;
  L.want_stats = req->enable_statistics;
  L.ctr = &S->ctr;
  L.dist = res->min_distance;
  L.ids = res->ids;
  L.points = res->nearest_points;
  L.margins = res->margins;
  L.within = res->within_margin;
  L.nbv = res->num_bv_tests;
  L.nleaf = res->num_leaf_tests;
  L.nrecheck = res->num_rechecks;
  const int block = 128;
  if ((e = launch_mesh_distance(L, req->precision, stack, distance_grid(req->precision, stack, block), block, s)) !=
      cudaSuccess)
    return cuda_fail(e, "distance kernel launch");
  BatchCounters hc;
  if ((e = cudaMemcpyAsync(&hc, &S->ctr, sizeof(hc), cudaMemcpyDeviceToHost, s)) != cudaSuccess)
    return cuda_fail(e, "read counters");
  if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return cuda_fail(e, "stream synchronize");
  if (hc.status) return fail(FCLGPU_ERR_DEVICE_STATUS, "device reported a traversal error (stack overflow or bad pair index)");
  return FCLGPU_OK;
}
