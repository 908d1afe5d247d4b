// C ABI for convex shape sets and batched shape-pair queries (include/fclgpu.h).
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/fclgpu.h"
#include "shapes.h"
#include "shapeset_handle.h"

using namespace fclgpu;

namespace {

std::mutex g_mu;

struct Buf {
  void* p = nullptr;
  size_t cap = 0;
  cudaError_t ensure(size_t bytes) {
    if (bytes <= cap) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
    cudaError_t e = cudaMalloc(&p, std::max<size_t>(bytes, 256));
    if (e == cudaSuccess) cap = std::max<size_t>(bytes, 256);
    return e;
  }
};
Buf g_ctr, g_ia, g_ib, g_tf1, g_tf2, g_hit, g_nrm, g_pt, g_dep, g_dist, g_p1, g_p2, g_st, g_order, g_epa, g_bins;
cudaEvent_t g_ev[2] = {nullptr, nullptr};

int cfail(cudaError_t e, const char* where) {
  set_error_detail(std::string(where) + ": " + cudaGetErrorString(e));
  return e == cudaErrorMemoryAllocation ? FCLGPU_ERR_OUT_OF_MEMORY : FCLGPU_ERR_CUDA;
}
#define CKS(expr, where)                          \
  do {                                            \
    cudaError_t e_ = (expr);                      \
    if (e_ != cudaSuccess) return cfail(e_, where); \
  } while (0)

}  // namespace

namespace {
std::mutex g_solver_mu;
SolverParams g_solver = FCLG_SOLVER_DEFAULTS;
}  // namespace

SolverParams fclgpu::current_solver_params() {
  std::lock_guard<std::mutex> lk(g_solver_mu);
  return g_solver;
}

extern "C" {

int fclgpu_shapeset_create(const fclgpu_shape* shapes, int32_t n, const double* verts, int64_t nv,
                           fclgpu_shapeset* out) {
  if (!out || n <= 0 || !shapes || (nv > 0 && !verts)) return FCLGPU_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  std::vector<DevShape> h(n);
  for (int i = 0; i < n; ++i) {
    const fclgpu_shape& s = shapes[i];
    if (s.type < FCLGPU_SHAPE_BOX || s.type > FCLGPU_SHAPE_CONVEX) return FCLGPU_ERR_INVALID_ARGUMENT;
    if (s.type == FCLGPU_SHAPE_CONVEX &&
        (s.vertex_count <= 0 || s.vertex_offset < 0 || s.vertex_offset + (int64_t)s.vertex_count > nv))
      return FCLGPU_ERR_INVALID_ARGUMENT;
    h[i].type = s.type;
    h[i].voff = s.vertex_offset;
    h[i].vcnt = s.vertex_count;
    h[i].pad = 0;
    for (int k = 0; k < 3; ++k) h[i].p[k] = s.params[k];
  }
  // vertex pool: the FP64 vertices, then (16-byte aligned) an FP32 float4 copy that the
  // convex support functions filter with; no copy if a coordinate is outside FP32 range
  // or the offset does not fit the shape record
  const int64_t off32 = (3 * nv + 1) & ~int64_t(1);
  bool use32 = nv > 0 && off32 < INT32_MAX;
  for (int64_t k = 0; use32 && k < 3 * nv; ++k) use32 = std::fabs(verts[k]) < 1e30;
  std::vector<float> v32(use32 ? 4 * nv : 0);
  for (int64_t k = 0; use32 && k < nv; ++k) {
    for (int c = 0; c < 3; ++c) v32[4 * k + c] = (float)verts[3 * k + c];
    v32[4 * k + 3] = 0.f;
  }
  if (use32)
    for (auto& d : h)
      if (d.type == FCLGPU_SHAPE_CONVEX) d.pad = (int32_t)off32;
  // a Convex's params are unused by FCL; params[0] holds the largest vertex norm (its
  // radius about the frame origin), rounded up, for the FP32 separation certificates
  for (auto& d : h)
    if (d.type == FCLGPU_SHAPE_CONVEX) {
      double r = 0.0;
      for (int i = 0; i < d.vcnt; ++i) {
        const double* v = verts + 3 * ((int64_t)d.voff + i);
        r = std::max(r, std::sqrt((v[0] * v[0] + v[1] * v[1]) + v[2] * v[2]));
      }
      d.p[0] = r * (1.0 + 1e-6);
    }
  const size_t pool_bytes = sizeof(double) * (use32 ? off32 : 3 * std::max<int64_t>(nv, 1)) + v32.size() * 4;
  fclgpu_shapeset_s* ss = new fclgpu_shapeset_s();
  cudaError_t e = cudaMalloc(&ss->shapes, sizeof(DevShape) * n);
  if (e == cudaSuccess) e = cudaMemcpy(ss->shapes, h.data(), sizeof(DevShape) * n, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMalloc(&ss->verts, pool_bytes);
  if (e == cudaSuccess && nv > 0) e = cudaMemcpy(ss->verts, verts, sizeof(double) * 3 * nv, cudaMemcpyHostToDevice);
  if (e == cudaSuccess && use32)
    e = cudaMemcpy(ss->verts + off32, v32.data(), v32.size() * 4, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    if (ss->shapes) cudaFree(ss->shapes);
    if (ss->verts) cudaFree(ss->verts);
    delete ss;
    return cfail(e, "shapeset upload");
  }
  ss->n = n;
  ss->nv = nv;
  ss->host = h;
  if (nv > 0) ss->host_verts.assign(verts, verts + 3 * nv);
  *out = ss;
  return FCLGPU_OK;
}

int fclgpu_shapeset_destroy(fclgpu_shapeset s) {
  if (!s) return FCLGPU_OK;
  cudaFree(s->shapes);
  cudaFree(s->verts);
  delete s;
  return FCLGPU_OK;
}

int fclgpu_shape_batch_device(fclgpu_shapeset set, int64_t n, const int32_t* ia, const int32_t* ib,
                              const double* tf1, const double* tf2, fclgpu_shape_result* res, void* stream) {
  if (!set || !res || n < 0 || (n > 0 && (!ia || !ib || !tf1 || !tf2 || !res->hit || !res->distance)))
    return FCLGPU_ERR_INVALID_ARGUMENT;
  if (n == 0) return FCLGPU_OK;
  std::lock_guard<std::mutex> lk(g_mu);
  cudaStream_t s = (cudaStream_t)stream;
  CKS(g_ctr.ensure(sizeof(BatchCounters)), "counters");
  CKS(cudaMemsetAsync(g_ctr.p, 0, sizeof(BatchCounters), s), "counters");
  // optional outputs default to scratch
  const size_t nn = (size_t)n;
  CKS(g_nrm.ensure(24 * nn), "scratch");
  CKS(g_pt.ensure(24 * nn), "scratch");
  CKS(g_dep.ensure(8 * nn), "scratch");
  CKS(g_p1.ensure(24 * nn), "scratch");
  CKS(g_p2.ensure(24 * nn), "scratch");
  ShapeLaunch L;
  L.shapes = set->shapes;
  L.verts = set->verts;
  L.ia = ia;
  L.ib = ib;
  L.tf1 = tf1;
  L.tf2 = tf2;
  L.n = n;
  L.ctr = (BatchCounters*)g_ctr.p;
  L.hit = res->hit;
  L.normal = res->normal ? res->normal : (double*)g_nrm.p;
  L.point = res->point ? res->point : (double*)g_pt.p;
  L.depth = res->depth ? res->depth : (double*)g_dep.p;
  L.dist = res->distance;
  L.p1 = res->p1 ? res->p1 : (double*)g_p1.p;
  L.p2 = res->p2 ? res->p2 : (double*)g_p2.p;
  L.status = res->status;
  CKS(g_order.ensure(4 * nn), "scratch");
  CKS(g_epa.ensure(4 * nn), "scratch");
  CKS(g_bins.ensure(64 * 4 + 16), "scratch");  // bins, EPA count, distance work counter
  L.order = (int32_t*)g_order.p;
  L.epa_list = (int32_t*)g_epa.p;
  L.epa_count = (unsigned long long*)((char*)g_bins.p + 64 * 4);
  if (!g_ev[0]) {
    CKS(cudaEventCreate(&g_ev[0]), "event");
    CKS(cudaEventCreate(&g_ev[1]), "event");
  }
  CKS(cudaEventRecord(g_ev[0], s), "event");
  CKS(launch_shape_batch(L, (unsigned*)g_bins.p, s), "shape kernel");
  CKS(cudaEventRecord(g_ev[1], s), "event");
  CKS(cudaStreamSynchronize(s), "shape kernel");
  float ms = 0.f;
  CKS(cudaEventElapsedTime(&ms, g_ev[0], g_ev[1]), "event");
  g_last_shape_ms = ms;
  return FCLGPU_OK;
}

int fclgpu_shape_batch(fclgpu_shapeset set, int64_t n, const int32_t* ia, const int32_t* ib, const double* tf1,
                       const double* tf2, fclgpu_shape_result* res, void* stream) {
  if (!set || !res || n < 0 || (n > 0 && (!ia || !ib || !tf1 || !tf2 || !res->hit || !res->distance)))
    return FCLGPU_ERR_INVALID_ARGUMENT;
  if (n == 0) return FCLGPU_OK;
  cudaStream_t s = (cudaStream_t)stream;
  const size_t nn = (size_t)n;
  {
    std::lock_guard<std::mutex> lk(g_mu);
    CKS(g_ia.ensure(4 * nn), "inputs");
    CKS(g_ib.ensure(4 * nn), "inputs");
    CKS(g_tf1.ensure(96 * nn), "inputs");
    CKS(g_tf2.ensure(96 * nn), "inputs");
    CKS(g_hit.ensure(4 * nn), "outputs");
    CKS(g_dist.ensure(8 * nn), "outputs");
    CKS(g_st.ensure(8 * nn), "outputs");
    CKS(cudaMemcpyAsync(g_ia.p, ia, 4 * nn, cudaMemcpyHostToDevice, s), "h2d");
    CKS(cudaMemcpyAsync(g_ib.p, ib, 4 * nn, cudaMemcpyHostToDevice, s), "h2d");
    CKS(cudaMemcpyAsync(g_tf1.p, tf1, 96 * nn, cudaMemcpyHostToDevice, s), "h2d");
    CKS(cudaMemcpyAsync(g_tf2.p, tf2, 96 * nn, cudaMemcpyHostToDevice, s), "h2d");
  }
  fclgpu_shape_result d{};
  d.hit = (int32_t*)g_hit.p;
  d.distance = (double*)g_dist.p;
  d.status = res->status ? (int32_t*)g_st.p : nullptr;
  // optional per-pair vectors land in scratch owned by the device entry point
  int rc = fclgpu_shape_batch_device(set, n, (const int32_t*)g_ia.p, (const int32_t*)g_ib.p,
                                     (const double*)g_tf1.p, (const double*)g_tf2.p, &d, stream);
  if (rc) return rc;
  std::lock_guard<std::mutex> lk(g_mu);
  CKS(cudaMemcpyAsync(res->hit, g_hit.p, 4 * nn, cudaMemcpyDeviceToHost, s), "d2h");
  CKS(cudaMemcpyAsync(res->distance, g_dist.p, 8 * nn, cudaMemcpyDeviceToHost, s), "d2h");
  if (res->normal) CKS(cudaMemcpyAsync(res->normal, g_nrm.p, 24 * nn, cudaMemcpyDeviceToHost, s), "d2h");
  if (res->point) CKS(cudaMemcpyAsync(res->point, g_pt.p, 24 * nn, cudaMemcpyDeviceToHost, s), "d2h");
  if (res->depth) CKS(cudaMemcpyAsync(res->depth, g_dep.p, 8 * nn, cudaMemcpyDeviceToHost, s), "d2h");
  if (res->p1) CKS(cudaMemcpyAsync(res->p1, g_p1.p, 24 * nn, cudaMemcpyDeviceToHost, s), "d2h");
  if (res->p2) CKS(cudaMemcpyAsync(res->p2, g_p2.p, 24 * nn, cudaMemcpyDeviceToHost, s), "d2h");
  if (res->status) CKS(cudaMemcpyAsync(res->status, g_st.p, 8 * nn, cudaMemcpyDeviceToHost, s), "d2h");
  CKS(cudaStreamSynchronize(s), "shape batch");
  return FCLGPU_OK;
}

int fclgpu_last_shape_kernel_time(double* ms) {
  if (!ms) return FCLGPU_ERR_INVALID_ARGUMENT;
  *ms = fclgpu::g_last_shape_ms;
  return FCLGPU_OK;
}

int fclgpu_shape_collide_batch(fclgpu_shapeset set, int64_t n, const int32_t* ia, const int32_t* ib,
                               const double* tf1, const double* tf2, int32_t* hit, void* stream) {
  if (!set || n < 0 || (n > 0 && (!ia || !ib || !tf1 || !tf2 || !hit))) return FCLGPU_ERR_INVALID_ARGUMENT;
  if (n == 0) return FCLGPU_OK;
  cudaStream_t s = (cudaStream_t)stream;
  const size_t nn = (size_t)n;
  std::lock_guard<std::mutex> lk(g_mu);
  CKS(g_ia.ensure(4 * nn), "inputs");
  CKS(g_ib.ensure(4 * nn), "inputs");
  CKS(g_tf1.ensure(96 * nn), "inputs");
  CKS(g_tf2.ensure(96 * nn), "inputs");
  CKS(g_hit.ensure(4 * nn), "outputs");
  CKS(cudaMemcpyAsync(g_ia.p, ia, 4 * nn, cudaMemcpyHostToDevice, s), "h2d");
  CKS(cudaMemcpyAsync(g_ib.p, ib, 4 * nn, cudaMemcpyHostToDevice, s), "h2d");
  CKS(cudaMemcpyAsync(g_tf1.p, tf1, 96 * nn, cudaMemcpyHostToDevice, s), "h2d");
  CKS(cudaMemcpyAsync(g_tf2.p, tf2, 96 * nn, cudaMemcpyHostToDevice, s), "h2d");
  ShapeLaunch L{};
  L.shapes = set->shapes;
  L.verts = set->verts;
  L.ia = (const int32_t*)g_ia.p;
  L.ib = (const int32_t*)g_ib.p;
  L.tf1 = (const double*)g_tf1.p;
  L.tf2 = (const double*)g_tf2.p;
  L.n = n;
  L.hit = (int32_t*)g_hit.p;
  CKS(launch_shape_collide_only(L, s), "shape collide");
  CKS(cudaMemcpyAsync(hit, g_hit.p, 4 * nn, cudaMemcpyDeviceToHost, s), "d2h");
  CKS(cudaStreamSynchronize(s), "shape collide");
  return FCLGPU_OK;
}

int fclgpu_set_gjk_solver_params(const fclgpu_gjk_solver_params* p) {
  SolverParams v = FCLG_SOLVER_DEFAULTS;
  if (p) {
    if (!(p->gjk_tolerance > 0.0) || !(p->epa_tolerance > 0.0) || !(p->gjk_tolerance < 1e300) ||
        !(p->epa_tolerance < 1e300) || p->gjk_max_iterations < 1 || p->epa_max_iterations < 1)
      return FCLGPU_ERR_INVALID_ARGUMENT;
    v = SolverParams{p->gjk_tolerance, p->epa_tolerance, p->gjk_max_iterations, p->epa_max_iterations};
  }
  std::lock_guard<std::mutex> lk(g_solver_mu);
  g_solver = v;
  return FCLGPU_OK;
}

int fclgpu_get_gjk_solver_params(fclgpu_gjk_solver_params* p) {
  if (!p) return FCLGPU_ERR_INVALID_ARGUMENT;
  const SolverParams v = current_solver_params();
  *p = fclgpu_gjk_solver_params{v.gjk_tolerance, v.epa_tolerance, v.gjk_max_iterations, v.epa_max_iterations};
  return FCLGPU_OK;
}

}  // extern "C"
