// Batched BVHModel<OBBRSS> x convex shape collide / distance (one pair per thread) and
// its C ABI (fclgpu_mesh_shape_batch*).
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/fclgpu.h"
#include "kernels.h"
#include "mesh_handle.h"
#include "mesh_shape.cuh"
#include "mesh_shape.h"
#include "shapeset_handle.h"

namespace fclgpu {
namespace {

template <int STACK>
__global__ void __launch_bounds__(128) k_mesh_shape(MeshShapeLaunch L) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < L.n; i += stride) {
    const DevMesh m = L.meshes[L.mesh_idx[i]];
    ShapeRef A;
    A.s = L.shapes[L.shape_idx[i]];
    A.verts = L.sverts;
    M3<double> Rm, Rs;
    D3v tm, ts;
    load_tf(L.tfm + 12 * i, Rm, tm);
    load_tf(L.tfs + 12 * i, Rs, ts);
    MeshShapeOut o;
    o.count = 0;
    o.tri = -1;
    o.dist = 0;
    o.pmesh = o.pshape = v3(0.0, 0.0, 0.0);
    o.nbv = o.nleaf = 0;
    o.status = 0;
    if (L.mode == 0) {
      mesh_shape_collide<STACK>(m, Rm, tm, A, Rs, ts, L.max_contacts, o);
      L.counts[i] = o.count;
    } else {
      mesh_shape_distance<STACK>(m, Rm, tm, A, Rs, ts, o);
      L.dist[i] = o.dist;
      if (L.tri) L.tri[i] = o.tri;
      if (L.pts) {
        double* p = L.pts + 6 * i;
        p[0] = o.pmesh.x;
        p[1] = o.pmesh.y;
        p[2] = o.pmesh.z;
        p[3] = o.pshape.x;
        p[4] = o.pshape.y;
        p[5] = o.pshape.z;
      }
    }
    if (L.nbv) L.nbv[i] = o.nbv;
    if (L.nleaf) L.nleaf[i] = o.nleaf;
    if (o.status) atomicOr(L.status, 1u);
  }
}

}  // namespace

cudaError_t launch_mesh_shape(const MeshShapeLaunch& L, int stack_entries, cudaStream_t s) {
  if (L.n <= 0) return cudaSuccess;
  const long long want = (L.n + 127) / 128;
  const int grid = (int)std::min<long long>(std::max<long long>(want, 1), 152 * 32);
  if (stack_entries <= 64)
    k_mesh_shape<64><<<grid, 128, 0, s>>>(L);
  else
    k_mesh_shape<256><<<grid, 128, 0, s>>>(L);
  ++g_kernel_launches;
  return cudaGetLastError();
}

}  // namespace fclgpu

using namespace fclgpu;

namespace {

std::mutex g_ms_mu;

struct MsBuf {
  void* p = nullptr;
  size_t cap = 0;
  cudaError_t ensure(size_t bytes) {
    if (bytes <= cap) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
    const size_t want = std::max<size_t>(bytes, 256);
    cudaError_t e = cudaMalloc(&p, want);
    if (e == cudaSuccess) cap = want;
    return e;
  }
};
MsBuf g_ms_meshes, g_ms_status;

int ms_fail(int code, const std::string& why) {
  set_error_detail(why);
  return code;
}
int ms_cuda(cudaError_t e, const char* where) {
  set_error_detail(std::string(where) + ": " + cudaGetErrorString(e));
  return e == cudaErrorMemoryAllocation ? FCLGPU_ERR_OUT_OF_MEMORY : FCLGPU_ERR_CUDA;
}

}  // namespace

extern "C" {

int fclgpu_mesh_shape_batch_device(const fclgpu_mesh* meshes, int32_t num_meshes, fclgpu_shapeset shapes, int64_t n,
                                   const int32_t* mesh_idx, const int32_t* shape_idx, const double* tf_mesh,
                                   const double* tf_shape, const fclgpu_mesh_shape_request* req,
                                   fclgpu_mesh_shape_result* res, void* stream) {
  if (!req || !res || n < 0 || !meshes || num_meshes <= 0 || !shapes)
    return ms_fail(FCLGPU_ERR_INVALID_ARGUMENT, "missing mesh-shape argument");
  if (req->mode != FCLGPU_MESH_SHAPE_COLLIDE && req->mode != FCLGPU_MESH_SHAPE_DISTANCE)
    return ms_fail(FCLGPU_ERR_INVALID_ARGUMENT, "unknown mode");
  if (n > 0 && (!mesh_idx || !shape_idx || !tf_mesh || !tf_shape ||
                (req->mode == FCLGPU_MESH_SHAPE_COLLIDE ? !res->counts : !res->min_distance)))
    return ms_fail(FCLGPU_ERR_INVALID_ARGUMENT, "missing mesh-shape input or output");
  if (req->mode == FCLGPU_MESH_SHAPE_COLLIDE && req->num_max_contacts < 1)
    return ms_fail(FCLGPU_ERR_INVALID_ARGUMENT, "num_max_contacts must be >= 1");
  std::vector<DevMesh> table(num_meshes);
  int depth = 0;
  for (int32_t i = 0; i < num_meshes; ++i) {
    if (!meshes[i]) return ms_fail(FCLGPU_ERR_INVALID_ARGUMENT, "null mesh handle");
    table[i] = meshes[i]->dev;
    depth = std::max(depth, (int)meshes[i]->dev.max_depth);
  }
  if (depth + 2 > 256) return ms_fail(FCLGPU_ERR_STACK_DEPTH, "BVH deeper than the traversal stack");
  if (n == 0) return FCLGPU_OK;
  std::lock_guard<std::mutex> lk(g_ms_mu);
  cudaStream_t s = (cudaStream_t)stream;
  cudaError_t e = g_ms_meshes.ensure(sizeof(DevMesh) * num_meshes);
  if (e == cudaSuccess) e = g_ms_status.ensure(sizeof(unsigned));
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(g_ms_meshes.p, table.data(), sizeof(DevMesh) * num_meshes, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(g_ms_status.p, 0, sizeof(unsigned), s);
  if (e != cudaSuccess) return ms_cuda(e, "mesh-shape setup");
  MeshShapeLaunch L;
  L.meshes = static_cast<const DevMesh*>(g_ms_meshes.p);
  L.shapes = shapes->shapes;
  L.sverts = shapes->verts;
  L.n = n;
  L.mesh_idx = mesh_idx;
  L.shape_idx = shape_idx;
  L.tfm = tf_mesh;
  L.tfs = tf_shape;
  L.mode = req->mode;
  L.max_contacts = (int32_t)std::min<int64_t>(req->num_max_contacts, INT32_MAX);
  L.counts = res->counts;
  L.dist = res->min_distance;
  L.tri = res->tri;
  L.pts = res->nearest_points;
  L.nbv = res->num_bv_tests;
  L.nleaf = res->num_leaf_tests;
  L.status = static_cast<unsigned*>(g_ms_status.p);
  e = launch_mesh_shape(L, depth + 2, s);
  unsigned st = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&st, g_ms_status.p, sizeof(unsigned), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return ms_cuda(e, "mesh-shape kernel");
  if (st) return ms_fail(FCLGPU_ERR_STACK_DEPTH, "mesh-shape traversal stack overflow");
  return FCLGPU_OK;
}

int fclgpu_mesh_shape_batch(const fclgpu_mesh* meshes, int32_t num_meshes, fclgpu_shapeset shapes, int64_t n,
                            const int32_t* mesh_idx, const int32_t* shape_idx, const double* tf_mesh,
                            const double* tf_shape, const fclgpu_mesh_shape_request* req,
                            fclgpu_mesh_shape_result* res, void* stream) {
  if (!req || !res || n < 0) return ms_fail(FCLGPU_ERR_INVALID_ARGUMENT, "missing mesh-shape argument");
  if (n == 0)
    return fclgpu_mesh_shape_batch_device(meshes, num_meshes, shapes, 0, mesh_idx, shape_idx, tf_mesh, tf_shape, req,
                                          res, stream);
  cudaStream_t s = (cudaStream_t)stream;
  const size_t nn = (size_t)n;
  // one staging block: inputs, then outputs
  const size_t bytes = nn * (4 + 4 + 96 + 96 + 4 + 8 + 4 + 48 + 8 + 8) + 16;  // + alignment padding
  char* d = nullptr;
  cudaError_t e = cudaMalloc(&d, bytes);
  if (e != cudaSuccess) return ms_cuda(e, "staging");
  int32_t* dm = (int32_t*)d;
  int32_t* ds = dm + nn;
  double* dtm = (double*)(ds + nn);
  double* dts = dtm + 12 * nn;
  int32_t* dc = (int32_t*)(dts + 12 * nn);
  double* dd = (double*)(dc + nn + (nn & 1));
  int32_t* dt = (int32_t*)(dd + nn);
  double* dp = (double*)(dt + nn + (nn & 1));
  int64_t* db = (int64_t*)(dp + 6 * nn);
  int64_t* dl = db + nn;
  if (e == cudaSuccess) e = cudaMemcpyAsync(dm, mesh_idx, 4 * nn, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(ds, shape_idx, 4 * nn, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dtm, tf_mesh, 96 * nn, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dts, tf_shape, 96 * nn, cudaMemcpyHostToDevice, s);
  int rc = FCLGPU_OK;
  if (e != cudaSuccess) {
    rc = ms_cuda(e, "h2d");
  } else {
    fclgpu_mesh_shape_result dr = {dc, dd, dt, dp, db, dl};
    rc = fclgpu_mesh_shape_batch_device(meshes, num_meshes, shapes, n, dm, ds, dtm, dts, req, &dr, stream);
    if (rc == FCLGPU_OK) {
      if (req->mode == FCLGPU_MESH_SHAPE_COLLIDE) {
        e = cudaMemcpyAsync(res->counts, dc, 4 * nn, cudaMemcpyDeviceToHost, s);
      } else {
        e = cudaMemcpyAsync(res->min_distance, dd, 8 * nn, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess && res->tri) e = cudaMemcpyAsync(res->tri, dt, 4 * nn, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess && res->nearest_points)
          e = cudaMemcpyAsync(res->nearest_points, dp, 48 * nn, cudaMemcpyDeviceToHost, s);
      }
      if (e == cudaSuccess && res->num_bv_tests)
        e = cudaMemcpyAsync(res->num_bv_tests, db, 8 * nn, cudaMemcpyDeviceToHost, s);
      if (e == cudaSuccess && res->num_leaf_tests)
        e = cudaMemcpyAsync(res->num_leaf_tests, dl, 8 * nn, cudaMemcpyDeviceToHost, s);
      if (e == cudaSuccess) e = cudaStreamSynchronize(s);
      if (e != cudaSuccess) rc = ms_cuda(e, "d2h");
    }
  }
  cudaFree(d);
  return rc;
}

}  // extern "C"
