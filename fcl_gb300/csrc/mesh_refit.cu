// Device refit of a mesh's BVH after its vertices moved, and its C ABI
// (fclgpu_mesh_update*): BVHModel<OBBRSS>::beginUpdateModel, updateVertex for every
// vertex, endUpdateModel(refit = true, bottomup = true)
// (geometry/bvh/BVH_model-inl.h:624-727, 961-1027).  The tree keeps its shape; every
// leaf is refitted to its triangle in the previous and the current frame, then the
// internal nodes level by level, deepest first, as the sum of their children.  The FP32
// store (nodes, sizes, RSS, triangles) and the magnitude bounds the FP32 filters use are
// rebuilt from the new FP64 values.  The local AABB is kept: FCL's endUpdateModel does
// not recompute it.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/fclgpu.h"
#include "kernels.h"
#include "mesh_handle.h"
#include "refit.cuh"

namespace fclgpu {
void set_error_detail(const std::string& what);
}

using namespace fclgpu;

namespace {

std::mutex g_refit_mu;

__device__ __forceinline__ D3v vtx(const double* V, int i) { return v3(V[3 * i], V[3 * i + 1], V[3 * i + 2]); }

__global__ void k_refit_leaves(DevMesh m, const double* prev, NodeD* nodes, RssD* rss) {
  const int stride = gridDim.x * blockDim.x;
  for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < m.n_nodes; b += stride) {
    const int child = nodes[b].child;
    if (child >= 0) continue;
    const int t = -(child + 1);
    const int i0 = m.tris[3 * t], i1 = m.tris[3 * t + 1], i2 = m.tris[3 * t + 2];
    NodeD nd;
    RssD rs;
    if (prev) {  // both frames: fit over six points (fitn)
      const D3v v[6] = {vtx(prev, i0), vtx(prev, i1), vtx(prev, i2),
                        vtx(m.verts64, i0), vtx(m.verts64, i1), vtx(m.verts64, i2)};
      auto pts = [&](int i) { return v[i]; };
      fit_points_bv(pts, 6, nd, rs.To, rs.l, rs.r);
      for (int k = 0; k < 9; ++k) rs.axis[k] = nd.axis[k];
    } else {     // no previous frame (replaced model): fit3
      const D3v v[3] = {vtx(m.verts64, i0), vtx(m.verts64, i1), vtx(m.verts64, i2)};
      fit3_obbrss(v, nd, rs);
    }
    nd.child = child;
    nodes[b] = nd;
    rss[b] = rs;
  }
}

// internal nodes ids[0..n) (one level: their children are final)
__global__ void k_refit_level(const int32_t* ids, int n, NodeD* nodes, RssD* rss) {
  const int stride = gridDim.x * blockDim.x;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += stride) {
    const int b = ids[k];
    const int c = nodes[b].child;
    NodeD nd = obb_merge(nodes[c], nodes[c + 1]);
    nd.child = c;
    const RssD rs = rss_merge(rss[c], rss[c + 1]);
    nodes[b] = nd;
    rss[b] = rs;
  }
}

__device__ __forceinline__ void atomic_max_nonneg(unsigned long long* p, double x) {
  atomicMax(p, (unsigned long long)__double_as_longlong(x));  // non-negative doubles order as integers
}

// the FP32 store of every node (the layout of pack_fp32) and the centre bounds
__global__ void k_refit_pack(DevMesh m, const NodeD* nodes, const RssD* rss, float4* nodes32, double* size64,
                             float4* rss32, unsigned long long* bounds) {
  const int stride = gridDim.x * blockDim.x;
  for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < m.n_nodes; b += stride) {
    const NodeD n = nodes[b];
    const RssD r = rss[b];
    for (int k = 0; k < 3; ++k)
      nodes32[4 * b + k] = make_float4((float)n.axis[k], (float)n.axis[3 + k], (float)n.axis[6 + k], (float)n.To[k]);
    nodes32[4 * b + 3] = make_float4((float)n.ext[0], (float)n.ext[1], (float)n.ext[2], __int_as_float(n.child));
    size64[b] = (n.ext[0] * n.ext[0] + n.ext[1] * n.ext[1]) + n.ext[2] * n.ext[2];
    rss32[5 * b] = make_float4((float)r.To[0], (float)r.To[1], (float)r.To[2], (float)r.r);
    rss32[5 * b + 1] = make_float4((float)r.l[0], (float)r.l[1], 0.f, 0.f);
    for (int k = 0; k < 3; ++k)
      rss32[5 * b + 2 + k] = make_float4((float)r.axis[k], (float)r.axis[3 + k], (float)r.axis[6 + k], 0.f);
    atomic_max_nonneg(bounds + 1, sqrt((n.To[0] * n.To[0] + n.To[1] * n.To[1]) + n.To[2] * n.To[2]));
    atomic_max_nonneg(bounds + 2, sqrt((r.To[0] * r.To[0] + r.To[1] * r.To[1]) + r.To[2] * r.To[2]));
  }
}

// FP32 triangles (first vertex as a float pair, then the FP64 differences rounded) and
// the largest vertex coordinate
__global__ void k_refit_tris(DevMesh m, float4* tri32, unsigned long long* bounds) {
  const int stride = gridDim.x * blockDim.x;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < m.n_tris; t += stride) {
    const double* p1 = m.verts64 + 3 * m.tris[3 * t];
    const double* p2 = m.verts64 + 3 * m.tris[3 * t + 1];
    const double* p3 = m.verts64 + 3 * m.tris[3 * t + 2];
    float hi[3], lo[3], d2[3], d3[3];
    for (int k = 0; k < 3; ++k) {
      hi[k] = (float)p1[k];
      lo[k] = (float)(p1[k] - (double)hi[k]);
      d2[k] = (float)(p2[k] - p1[k]);
      d3[k] = (float)(p3[k] - p1[k]);
    }
    tri32[3 * t] = make_float4(hi[0], hi[1], hi[2], lo[0]);
    tri32[3 * t + 1] = make_float4(lo[1], lo[2], d2[0], d2[1]);
    tri32[3 * t + 2] = make_float4(d2[2], d3[0], d3[1], d3[2]);
  }
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < 3 * m.n_verts; i += stride)
    atomic_max_nonneg(bounds, fabs(m.verts64[i]));
}

int grid_for(long long n, int block) {
  return (int)std::max<long long>(1, std::min<long long>((n + block - 1) / block, 152LL * 16));
}

int refit_fail(int code, const std::string& why) {
  set_error_detail(why);
  return code;
}
int refit_cuda(cudaError_t e, const char* where) {
  set_error_detail(std::string(where) + ": " + cudaGetErrorString(e));
  return e == cudaErrorMemoryAllocation ? FCLGPU_ERR_OUT_OF_MEMORY : FCLGPU_ERR_CUDA;
}

}  // namespace

// The FP32 store (nodes, sizes, RSS, triangles) from the FP64 nodes and vertices, and the
// magnitude bounds the FP32 filters use.  Synchronises s.
int repack_mesh(fclgpu_mesh m, cudaStream_t s) {
  DevMesh& d = m->dev;
  cudaError_t e;
  if (!m->bounds) {
    if ((e = cudaMalloc(&m->bounds, 4 * sizeof(unsigned long long)))) return refit_cuda(e, "refit bounds");
    m->allocations.push_back(m->bounds);
  }
  if ((e = cudaMemsetAsync(m->bounds, 0, 4 * sizeof(unsigned long long), s))) return refit_cuda(e, "bounds");
  k_refit_pack<<<grid_for(d.n_nodes, 128), 128, 0, s>>>(d, d.nodes64, d.rss64, (float4*)d.nodes32,
                                                          const_cast<double*>(d.size64), (float4*)d.rss32,
                                                          (unsigned long long*)m->bounds);
  k_refit_tris<<<grid_for(std::max(d.n_tris, 3 * d.n_verts), 128), 128, 0, s>>>(d, (float4*)d.tri32,
                                                                                (unsigned long long*)m->bounds);
  g_kernel_launches += 2;
  if ((e = cudaGetLastError())) return refit_cuda(e, "refit kernels");
  unsigned long long hb[4];
  if ((e = cudaMemcpyAsync(hb, m->bounds, sizeof(hb), cudaMemcpyDeviceToHost, s)) || (e = cudaStreamSynchronize(s)))
    return refit_cuda(e, "refit");
  double bd[3];
  std::memcpy(bd, hb, sizeof(bd));
  // same inflation as at creation: the bounds must hold the FP64 values after rounding
  d.vmax = bd[0] * (1.0 + 1e-12);
  d.cmax = bd[1] * (1.0 + 1e-12);
  d.rmax = bd[2] * (1.0 + 1e-12);
  m->info.max_abs_coord = bd[0];
  return FCLGPU_OK;
}

namespace {

// verts: device pointer with the new positions (3 doubles per vertex).  replace = false:
// update (the current frame becomes the previous one, leaves fit both frames); true:
// replace (FCL drops the previous frame, leaves fit the new triangle alone).  rebuild:
// endUpdateModel / endReplaceModel with refit = false (BVH_model-inl.h:594-620, 703-734):
// buildTree on the new vertices (the device build, bvh_build_device.cu), followed for an
// update by the bottom-up refit over both frames, as FCL does.
int refit_from_device(fclgpu_mesh m, const double* verts, cudaStream_t s, bool replace, bool rebuild) {
  DevMesh& d = m->dev;
  const size_t vbytes = sizeof(double) * 3 * (size_t)d.n_verts;
  cudaError_t e = cudaSuccess;
  if (!m->prev_verts) {
    e = cudaMalloc(&m->prev_verts, vbytes);
    if (e != cudaSuccess) return refit_cuda(e, "previous-frame vertices");
    m->allocations.push_back(m->prev_verts);
  }
  double* cur = const_cast<double*>(d.verts64);
  // beginUpdateModel: the current frame becomes the previous one; updateVertex: the new
  // positions become the current frame
  if (!replace && (e = cudaMemcpyAsync(m->prev_verts, cur, vbytes, cudaMemcpyDeviceToDevice, s)))
    return refit_cuda(e, "frames");
  if ((e = cudaMemcpyAsync(cur, verts, vbytes, cudaMemcpyDeviceToDevice, s))) return refit_cuda(e, "frames");
  NodeD* nodes = const_cast<NodeD*>(d.nodes64);
  RssD* rss = const_cast<RssD*>(d.rss64);
  if (rebuild) {
    int maxd = 0;
    std::vector<int64_t> off;
    if ((e = build_bvh_device(cur, d.tris, d.n_tris, nodes, rss, off, m->levels, &maxd, s)))
      return refit_cuda(e, "device build");
    m->level_off = off;
    d.max_depth = maxd;
    m->info.max_depth = maxd;
  }
  if (!(rebuild && replace)) {
    k_refit_leaves<<<grid_for(d.n_nodes, 128), 128, 0, s>>>(d, replace ? nullptr : (const double*)m->prev_verts,
                                                             nodes, rss);
    ++g_kernel_launches;
    for (size_t l = m->level_off.size() - 1; l-- > 0;) {  // deepest level first
      const int64_t a = m->level_off[l], b = m->level_off[l + 1];
      if (b > a) {
        k_refit_level<<<grid_for(b - a, 128), 128, 0, s>>>(m->levels + a, (int)(b - a), nodes, rss);
        ++g_kernel_launches;
      }
    }
  }
  int rc = repack_mesh(m, s);
  if (rc) return rc;
  d.refitted = (rebuild && replace) ? 0 : 1;  // a fresh build's volumes contain their geometry
  if ((e = cudaMemcpyAsync(m->first_vertex, cur, 3 * sizeof(double), cudaMemcpyDeviceToHost, s)) ||
      (e = cudaStreamSynchronize(s)))
    return refit_cuda(e, "refit");
  return FCLGPU_OK;
}

}  // namespace

extern "C" {

namespace {
int move_vertices_device(fclgpu_mesh mesh, const double* verts, int64_t nv, void* stream, bool replace,
                         bool rebuild = false) {
  if (!mesh || !verts) return refit_fail(FCLGPU_ERR_INVALID_ARGUMENT, "null argument");
  if (nv != mesh->dev.n_verts)
    return refit_fail(FCLGPU_ERR_INCORRECT_DATA, "the updated model must have the same number of vertices");
  std::lock_guard<std::mutex> lk(g_refit_mu);
  return refit_from_device(mesh, verts, (cudaStream_t)stream, replace, rebuild);
}

int move_vertices_host(fclgpu_mesh mesh, const double* verts, int64_t nv, void* stream, bool replace,
                       bool rebuild = false) {
  if (!mesh || !verts) return refit_fail(FCLGPU_ERR_INVALID_ARGUMENT, "null argument");
  if (nv != mesh->dev.n_verts)
    return refit_fail(FCLGPU_ERR_INCORRECT_DATA, "the updated model must have the same number of vertices");
  std::lock_guard<std::mutex> lk(g_refit_mu);
  cudaStream_t s = (cudaStream_t)stream;
  const size_t vbytes = sizeof(double) * 3 * (size_t)nv;
  double* staging = nullptr;
  cudaError_t e = cudaMalloc(&staging, vbytes);
  if (e != cudaSuccess) return refit_cuda(e, "staging");
  e = cudaMemcpyAsync(staging, verts, vbytes, cudaMemcpyHostToDevice, s);
  int rc = e == cudaSuccess ? refit_from_device(mesh, staging, s, replace, rebuild) : refit_cuda(e, "h2d");
  cudaStreamSynchronize(s);
  cudaFree(staging);
  return rc;
}
}  // namespace

int fclgpu_mesh_update_device(fclgpu_mesh mesh, const double* verts, int64_t nv, void* stream) {
  return move_vertices_device(mesh, verts, nv, stream, false);
}

int fclgpu_mesh_update(fclgpu_mesh mesh, const double* verts, int64_t nv, void* stream) {
  return move_vertices_host(mesh, verts, nv, stream, false);
}

int fclgpu_mesh_replace_device(fclgpu_mesh mesh, const double* verts, int64_t nv, int32_t refit, void* stream) {
  return move_vertices_device(mesh, verts, nv, stream, true, refit == 0);
}

int fclgpu_mesh_replace(fclgpu_mesh mesh, const double* verts, int64_t nv, int32_t refit, void* stream) {
  return move_vertices_host(mesh, verts, nv, stream, true, refit == 0);
}

int fclgpu_mesh_update_model_device(fclgpu_mesh mesh, const double* verts, int64_t nv, int32_t refit, void* stream) {
  return move_vertices_device(mesh, verts, nv, stream, false, refit == 0);
}

int fclgpu_mesh_update_model(fclgpu_mesh mesh, const double* verts, int64_t nv, int32_t refit, void* stream) {
  return move_vertices_host(mesh, verts, nv, stream, false, refit == 0);
}

}  // extern "C"
