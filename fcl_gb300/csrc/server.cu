// Motion-checking request loop (include/fclgpu.h, fclgpu_server_*): continuous
// batching of robot-sweep requests over a resident device broadphase.
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <chrono>
#include <climits>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/fclgpu.h"
#include "kernels.h"
#include "shapeset_handle.h"

namespace fclgpu {
namespace {

constexpr int kMaxLinks = 64;
// waypoints of one request per step: the first chunk is one waypoint and each next one
// twice as long up to kRequestChunk, so a request checks at most about twice the
// waypoints up to its first contact (in a cluttered scene most requests collide at
// their first waypoints), and a long contact-free request needs few steps
constexpr int kFirstChunk = 1;
constexpr int kRequestChunk = 512;

struct RobotDev {
  int32_t L;
  const int32_t* axis;
  const double* offset;  // L x 3
  const double* gtf;     // L x 12
  const int2* refs;      // L
};

// Forward kinematics of one waypoint per thread: R <- R * Rot(axis_i, q_i); link i's
// geometry pose = (R * G_R, t + R * G_t); then t <- t + R * offset_i.
__global__ void k_robot_fk(RobotDev rb, int64_t W, const double* q, const int32_t* slot, const double* bases,
                           double* qtf, int2* qrefs) {
  const long long w = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= W) return;
  const double* b = bases + 12 * (long long)slot[w];
  double R[3][3], t[3];
#pragma unroll
  for (int r = 0; r < 3; ++r) {
    for (int c = 0; c < 3; ++c) R[r][c] = b[4 * r + c];
    t[r] = b[4 * r + 3];
  }
  for (int i = 0; i < rb.L; ++i) {
    double s, c;
    sincos(q[w * rb.L + i], &s, &c);
    const int ax = rb.axis[i];
    // R * J with J the rotation about axis ax: only two columns change
    const int a = ax == 0 ? 1 : 0, bcol = ax == 2 ? 1 : 2;  // the plane of rotation (a, bcol)
#pragma unroll
    for (int r = 0; r < 3; ++r) {
      const double ra = R[r][a], rbv = R[r][bcol];
      // J[a][a] = c, J[bcol][a] = s (x: y->z, y: z->x, z: x->y with sign per axis)
      if (ax == 1) {
        // rotation about y: [[c,0,s],[0,1,0],[-s,0,c]]; plane (x=0, z=2)
        R[r][a] = ra * c - rbv * s;
        R[r][bcol] = ra * s + rbv * c;
      } else {
        // about x: [[1,0,0],[0,c,-s],[0,s,c]] plane (1,2); about z: [[c,-s,0],[s,c,0],[0,0,1]] plane (0,1)
        R[r][a] = ra * c + rbv * s;
        R[r][bcol] = rbv * c - ra * s;
      }
    }
    const double* g = rb.gtf + 12 * i;
    double* o = qtf + 12 * (w * rb.L + i);
#pragma unroll
    for (int r = 0; r < 3; ++r) {
#pragma unroll
      for (int cc = 0; cc < 3; ++cc) o[4 * r + cc] = (R[r][0] * g[cc] + R[r][1] * g[4 + cc]) + R[r][2] * g[8 + cc];
      o[4 * r + 3] = t[r] + ((R[r][0] * g[3] + R[r][1] * g[7]) + R[r][2] * g[11]);
    }
    const double* off = rb.offset + 3 * i;
    double nt[3];
#pragma unroll
    for (int r = 0; r < 3; ++r) nt[r] = t[r] + ((R[r][0] * off[0] + R[r][1] * off[1]) + R[r][2] * off[2]);
#pragma unroll
    for (int r = 0; r < 3; ++r) t[r] = nt[r];
    qrefs[w * rb.L + i] = rb.refs[i];
  }
}

cudaError_t launch_robot_fk(const RobotDev& rb, int64_t W, const double* q, const int32_t* slot,
                            const double* bases, double* qtf, int2* qrefs, cudaStream_t s) {
  if (W <= 0) return cudaSuccess;
  k_robot_fk<<<(unsigned)((W + 127) / 128), 128, 0, s>>>(rb, W, q, slot, bases, qtf, qrefs);
  ++g_kernel_launches;
  return cudaGetLastError();
}

// The queries listed in idx, compacted for the clearance pass.
__global__ void k_gather_queries(long long n, const int32_t* idx, const int2* refs, const double* tf, int2* orefs,
                                 double* otf) {
  const long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  const long long i = idx[j];
  orefs[j] = refs[i];
  for (int k = 0; k < 12; ++k) otf[12 * j + k] = tf[12 * i + k];
}

using Clock = std::chrono::steady_clock;

struct Request {
  int64_t id;
  int32_t K;
  std::vector<double> base;
  std::vector<double> q;
  int32_t next_wp = 0;  // next waypoint to schedule
  int32_t done_wp = 0;
  int32_t chunk = kFirstChunk;  // waypoints of its next chunk
  fclgpu_motion_result res;
  Clock::time_point submit;
  bool started = false;
  bool done = false;
};

double ms_between(Clock::time_point a, Clock::time_point b) {
  return std::chrono::duration<double, std::milli>(b - a).count();
}

}  // namespace
}  // namespace fclgpu

using namespace fclgpu;

struct fclgpu_server_s {
  fclgpu_broadphase scene = nullptr;
  int32_t L = 0;
  std::vector<int32_t> axis;
  std::vector<double> offset, gtf;
  std::vector<fclgpu_geometry_ref> refs;
  fclgpu_server_config cfg;
  // device robot and step buffers
  int32_t* d_axis = nullptr;
  double* d_offset = nullptr;
  double* d_gtf = nullptr;
  int2* d_refs = nullptr;
  int64_t cap_wp = 0;
  double* d_q = nullptr;
  int32_t* d_slot = nullptr;
  double* d_bases = nullptr;
  double* d_qtf = nullptr;
  int2* d_qrefs = nullptr;
  int64_t* d_nc = nullptr;
  double* d_dist = nullptr;
  int32_t* d_obj = nullptr;
  int2* d_frefs = nullptr;   // compacted contact-free queries
  double* d_ftf = nullptr;
  int32_t* d_fmap = nullptr;
  double* d_fdist = nullptr;
  int32_t* d_fobj = nullptr;
  unsigned long long* d_fcount = nullptr;
  // pinned host staging
  double* h_q = nullptr;
  int32_t* h_slot = nullptr;
  double* h_bases = nullptr;
  int64_t* h_nc = nullptr;
  double* h_dist = nullptr;
  int32_t* h_obj = nullptr;
  int32_t* h_fidx = nullptr;
  cudaStream_t stream = nullptr;
  // queue
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  bool stop = false;
  std::deque<Request*> pending;
  std::vector<Request*> active;
  std::unordered_map<int64_t, std::unique_ptr<Request>> reqs;
  int64_t next_id = 1;
  int waiters = 0;  // threads inside fclgpu_server_wait (destroy waits for them to leave)
  fclgpu_server_stats stats;
  double cand_per_query = 8.0;  // running estimate for the memory admission
  std::thread worker;
  int device = 0;
  int last_error = FCLGPU_OK;
};

namespace {

RobotDev robot_dev(const fclgpu_server_s* s) {
  RobotDev r;
  r.L = s->L;
  r.axis = s->d_axis;
  r.offset = s->d_offset;
  r.gtf = s->d_gtf;
  r.refs = s->d_refs;
  return r;
}

// Waypoints one step may take under the free-memory budget: per waypoint, L queries of
// about 400 bytes of fixed scratch plus ~160 bytes per broadphase candidate.
int64_t memory_cap(fclgpu_server_s* s) {
  size_t freeb = 0, total = 0;
  if (cudaMemGetInfo(&freeb, &total) != cudaSuccess) return s->cap_wp;
  const double budget = s->cfg.memory_budget_bytes > 0 ? (double)s->cfg.memory_budget_bytes : 0.5 * (double)freeb;
  const double per_wp = (double)s->L * (400.0 + 160.0 * s->cand_per_query);
  const int64_t cap = (int64_t)(budget / per_wp);
  return std::max<int64_t>(1, std::min<int64_t>(cap, s->cap_wp));
}

struct Chunk {
  Request* r;
  int32_t k0, k1;
};

int run_step(fclgpu_server_s* s, const std::vector<Chunk>& chunks, int64_t W) {
  const int L = s->L;
  int64_t w = 0;
  for (size_t c = 0; c < chunks.size(); ++c) {
    const Chunk& ch = chunks[c];
    std::memcpy(s->h_bases + 12 * c, ch.r->base.data(), 96);
    const int32_t n = ch.k1 - ch.k0;
    std::memcpy(s->h_q + w * L, ch.r->q.data() + (size_t)ch.k0 * L, sizeof(double) * (size_t)n * L);
    for (int32_t k = 0; k < n; ++k) s->h_slot[w + k] = (int32_t)c;
    w += n;
  }
  cudaStream_t st = s->stream;
  const int64_t nq = W * L;
  if (cudaMemcpyAsync(s->d_q, s->h_q, sizeof(double) * nq, cudaMemcpyHostToDevice, st) != cudaSuccess ||
      cudaMemcpyAsync(s->d_slot, s->h_slot, 4 * W, cudaMemcpyHostToDevice, st) != cudaSuccess ||
      cudaMemcpyAsync(s->d_bases, s->h_bases, 96 * chunks.size(), cudaMemcpyHostToDevice, st) != cudaSuccess ||
      launch_robot_fk(robot_dev(s), W, s->d_q, s->d_slot, s->d_bases, s->d_qtf, s->d_qrefs, st) != cudaSuccess)
    return FCLGPU_ERR_CUDA;
  const auto tc0 = Clock::now();
  fclgpu_broadphase_collide_request creq = {1, s->cfg.precision, 0};
  fclgpu_broadphase_collide_result cres = {s->d_nc, nullptr, nullptr, 0, 0};
  int rc = fclgpu_broadphase_collide_device(s->scene, reinterpret_cast<const fclgpu_geometry_ref*>(s->d_qrefs), nq,
                                            s->d_qtf, &creq, &cres, st);
  if (rc) return rc;
  int64_t cand = cres.total_candidates;
  if (cudaMemcpyAsync(s->h_nc, s->d_nc, 8 * nq, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return FCLGPU_ERR_CUDA;
  const auto tc1 = Clock::now();
  // first colliding waypoint (and its smallest link) per request
  w = 0;
  for (const Chunk& ch : chunks) {
    fclgpu_motion_result& r = ch.r->res;
    for (int32_t k = ch.k0; k < ch.k1; ++k, ++w)
      for (int i = 0; i < L; ++i)
        if (s->h_nc[w * L + i] > 0 && (r.first_colliding_waypoint < 0 || k < r.first_colliding_waypoint)) {
          r.first_colliding_waypoint = k;
          r.clearance_link = i;
        }
  }
  if (s->cfg.compute_clearance) {
    // a request in contact has clearance 0; the queries of the others go through
    // the distance pass
    int64_t nfree = 0;
    w = 0;
    for (const Chunk& ch : chunks) {
      const int32_t n = ch.k1 - ch.k0;
      if (ch.r->res.first_colliding_waypoint < 0)
        for (int64_t qi = w * L; qi < (w + n) * L; ++qi) s->h_fidx[nfree++] = (int32_t)qi;
      w += n;
    }
    const auto td0 = Clock::now();
    if (nfree > 0) {
      if (cudaMemcpyAsync(s->d_fmap, s->h_fidx, 4 * nfree, cudaMemcpyHostToDevice, st) != cudaSuccess)
        return FCLGPU_ERR_CUDA;
      k_gather_queries<<<(unsigned)((nfree + 255) / 256), 256, 0, st>>>(nfree, s->d_fmap, s->d_qrefs, s->d_qtf,
                                                                        s->d_frefs, s->d_ftf);
      ++g_kernel_launches;
      if (cudaGetLastError() != cudaSuccess) return FCLGPU_ERR_CUDA;
      fclgpu_broadphase_distance_request dreq = {0, s->cfg.precision};
      fclgpu_broadphase_distance_result dres = {s->d_fdist, s->d_fobj, nullptr, nullptr, 0, 0};
      rc = fclgpu_broadphase_distance_device(s->scene, reinterpret_cast<const fclgpu_geometry_ref*>(s->d_frefs),
                                             nfree, s->d_ftf, &dreq, &dres, st);
      if (rc) return rc;
      cand = std::max<int64_t>(cand, dres.total_candidates);
      if (cudaMemcpyAsync(s->h_dist, s->d_fdist, 8 * nfree, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
          cudaMemcpyAsync(s->h_obj, s->d_fobj, 4 * nfree, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
          cudaStreamSynchronize(st) != cudaSuccess)
        return FCLGPU_ERR_CUDA;
    }
    s->stats.distance_ms += ms_between(td0, Clock::now());
    // clearance: minimum over the contact-free queries (ties: smallest waypoint, then
    // link); 0 at the first contact
    int64_t f = 0;
    w = 0;
    for (const Chunk& ch : chunks) {
      fclgpu_motion_result& r = ch.r->res;
      const int32_t n = ch.k1 - ch.k0;
      if (r.first_colliding_waypoint >= 0) {
        r.min_clearance = 0.0;
        r.clearance_waypoint = r.first_colliding_waypoint;
        r.clearance_object = -1;
      } else {
        for (int32_t k = ch.k0; k < ch.k1; ++k)
          for (int i = 0; i < L; ++i, ++f) {
            const double d = s->h_dist[f];
            const bool better = d < r.min_clearance ||
                                (d == r.min_clearance && (k < r.clearance_waypoint ||
                                                          (k == r.clearance_waypoint && i < r.clearance_link)));
            if (better) {
              r.min_clearance = d;
              r.clearance_waypoint = k;
              r.clearance_link = i;
              r.clearance_object = s->h_obj[f];
            }
          }
      }
      w += n;
    }
  }
  s->cand_per_query = 0.5 * s->cand_per_query + 0.5 * std::max(1.0, (double)cand / (double)std::max<int64_t>(nq, 1));
  s->stats.queries += nq;
  s->stats.candidates += cand;
  s->stats.collide_ms += ms_between(tc0, tc1);
  return FCLGPU_OK;
}

void worker_loop(fclgpu_server_s* s) {
  cudaSetDevice(s->device);
  for (;;) {
    std::vector<Chunk> chunks;
    int64_t W = 0;
    {
      std::unique_lock<std::mutex> lk(s->mu);
      s->cv_work.wait(lk, [&] { return s->stop || !s->pending.empty() || !s->active.empty(); });
      if (s->stop) break;
      const int64_t cap = memory_cap(s);
      // admit queued requests (FIFO) while the step has room for at least a chunk each
      while (!s->pending.empty() && (int64_t)s->active.size() < cap) {
        s->active.push_back(s->pending.front());
        s->pending.pop_front();
      }
      // fair share of the step among admitted requests, in admission order
      int64_t left = cap;
      size_t remaining = s->active.size();
      for (Request* r : s->active) {
        if (left <= 0) break;
        const int64_t share = std::max<int64_t>(1, left / (int64_t)remaining);
        --remaining;
        const int32_t n = (int32_t)std::min<int64_t>(std::min<int64_t>(share, r->chunk), r->K - r->next_wp);
        if (n <= 0) continue;
        r->chunk = std::min(2 * r->chunk, kRequestChunk);
        chunks.push_back(Chunk{r, r->next_wp, r->next_wp + n});
        r->next_wp += n;
        left -= n;
        W += n;
        if (!r->started) {
          r->started = true;
          r->res.queue_ms = ms_between(r->submit, Clock::now());
        }
      }
    }
    if (chunks.empty()) continue;
    const auto t0 = Clock::now();
    const int rc = run_step(s, chunks, W);
    const auto t1 = Clock::now();
    {
      std::lock_guard<std::mutex> lk(s->mu);
      s->stats.steps += 1;
      s->stats.waypoints += W;
      s->stats.busy_ms += ms_between(t0, t1);
      s->stats.max_step_waypoints = std::max<int64_t>(s->stats.max_step_waypoints, W);
      if (rc) s->last_error = rc;
      for (const Chunk& ch : chunks) {
        ch.r->done_wp += ch.k1 - ch.k0;
        ch.r->res.num_steps += 1;
      }
      std::vector<Request*> keep;
      for (Request* r : s->active) {
        // a request ends at its first contact: later waypoints change neither its
        // first colliding waypoint nor its clearance (0)
        if (r->done_wp >= r->K || r->res.first_colliding_waypoint >= 0 || rc) {
          r->done = true;
          r->res.reserved = rc;
          r->res.latency_ms = ms_between(r->submit, t1);
        } else {
          keep.push_back(r);
        }
      }
      s->active.swap(keep);
    }
    s->cv_done.notify_all();
  }
}

void free_server(fclgpu_server_s* s) {
  for (void* p : {(void*)s->d_axis, (void*)s->d_offset, (void*)s->d_gtf, (void*)s->d_refs, (void*)s->d_q,
                  (void*)s->d_slot, (void*)s->d_bases, (void*)s->d_qtf, (void*)s->d_qrefs, (void*)s->d_nc,
                  (void*)s->d_dist, (void*)s->d_obj, (void*)s->d_frefs, (void*)s->d_ftf, (void*)s->d_fmap,
                  (void*)s->d_fdist, (void*)s->d_fobj, (void*)s->d_fcount})
    if (p) cudaFree(p);
  for (void* p : {(void*)s->h_q, (void*)s->h_slot, (void*)s->h_bases, (void*)s->h_nc, (void*)s->h_dist,
                  (void*)s->h_obj, (void*)s->h_fidx})
    if (p) cudaFreeHost(p);
  if (s->stream) cudaStreamDestroy(s->stream);
  delete s;
}

}  // namespace

extern "C" {

int fclgpu_server_create(fclgpu_broadphase scene, const fclgpu_robot_desc* robot, const fclgpu_server_config* cfg,
                         fclgpu_server* out) {
  if (!out || !scene || !robot || robot->num_links <= 0 || robot->num_links > kMaxLinks || !robot->joint_axis ||
      !robot->link_offset || !robot->link_geometry || !robot->link_geometry_tf) {
    set_error_detail("bad server arguments");
    return FCLGPU_ERR_INVALID_ARGUMENT;
  }
  *out = nullptr;
  const int L = robot->num_links;
  for (int i = 0; i < L; ++i)
    if (robot->joint_axis[i] < 0 || robot->joint_axis[i] > 2) {
      set_error_detail("joint axis must be 0, 1 or 2");
      return FCLGPU_ERR_INVALID_ARGUMENT;
    }
  fclgpu_server_s* s = new fclgpu_server_s();
  s->scene = scene;
  s->L = L;
  s->axis.assign(robot->joint_axis, robot->joint_axis + L);
  s->offset.assign(robot->link_offset, robot->link_offset + 3 * L);
  s->gtf.assign(robot->link_geometry_tf, robot->link_geometry_tf + 12 * L);
  s->refs.assign(robot->link_geometry, robot->link_geometry + L);
  s->cfg = cfg ? *cfg : fclgpu_server_config{0, 0, FCLGPU_FP32_RECHECK, 1};
  if (s->cfg.max_waypoints_per_step <= 0) s->cfg.max_waypoints_per_step = 4096;
  s->cap_wp = s->cfg.max_waypoints_per_step;
  std::memset(&s->stats, 0, sizeof(s->stats));
  const int64_t W = s->cap_wp, nq = W * L;
  cudaError_t e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
  auto dm = [&](void** p, size_t b) {
    if (e == cudaSuccess) e = cudaMalloc(p, std::max<size_t>(b, 16));
  };
  auto hm = [&](void** p, size_t b) {
    if (e == cudaSuccess) e = cudaMallocHost(p, std::max<size_t>(b, 16));
  };
  dm((void**)&s->d_axis, 4 * L);
  dm((void**)&s->d_offset, 24 * L);
  dm((void**)&s->d_gtf, 96 * L);
  dm((void**)&s->d_refs, 8 * L);
  dm((void**)&s->d_q, 8 * nq);
  dm((void**)&s->d_slot, 4 * W);
  dm((void**)&s->d_bases, 96 * W);
  dm((void**)&s->d_qtf, 96 * nq);
  dm((void**)&s->d_qrefs, 8 * nq);
  dm((void**)&s->d_nc, 8 * nq);
  dm((void**)&s->d_dist, 8 * nq);
  dm((void**)&s->d_obj, 4 * nq);
  dm((void**)&s->d_frefs, 8 * nq);
  dm((void**)&s->d_ftf, 96 * nq);
  dm((void**)&s->d_fmap, 4 * nq);
  dm((void**)&s->d_fdist, 8 * nq);
  dm((void**)&s->d_fobj, 4 * nq);
  dm((void**)&s->d_fcount, 8);
  hm((void**)&s->h_q, 8 * nq);
  hm((void**)&s->h_slot, 4 * W);
  hm((void**)&s->h_bases, 96 * W);
  hm((void**)&s->h_nc, 8 * nq);
  hm((void**)&s->h_dist, 8 * nq);
  hm((void**)&s->h_obj, 4 * nq);
  hm((void**)&s->h_fidx, 4 * nq);
  if (e == cudaSuccess) e = cudaMemcpy(s->d_axis, s->axis.data(), 4 * L, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(s->d_offset, s->offset.data(), 24 * L, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(s->d_gtf, s->gtf.data(), 96 * L, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(s->d_refs, s->refs.data(), 8 * L, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    set_error_detail(std::string("server setup: ") + cudaGetErrorString(e));
    free_server(s);
    return e == cudaErrorMemoryAllocation ? FCLGPU_ERR_OUT_OF_MEMORY : FCLGPU_ERR_CUDA;
  }
  cudaGetDevice(&s->device);
  s->worker = std::thread(worker_loop, s);
  *out = s;
  return FCLGPU_OK;
}

int fclgpu_server_submit(fclgpu_server s, const double* base_tf, const double* q, int32_t num_waypoints,
                         int64_t* request_id) {
  if (!s || !base_tf || !q || num_waypoints <= 0 || !request_id) {
    set_error_detail("bad submit arguments");
    return FCLGPU_ERR_INVALID_ARGUMENT;
  }
  std::unique_ptr<Request> r(new Request());
  r->K = num_waypoints;
  r->base.assign(base_tf, base_tf + 12);
  r->q.assign(q, q + (size_t)num_waypoints * s->L);
  std::memset(&r->res, 0, sizeof(r->res));
  r->res.first_colliding_waypoint = -1;
  r->res.clearance_waypoint = -1;
  r->res.clearance_link = -1;
  r->res.clearance_object = -1;
  r->res.min_clearance = DBL_MAX;
  r->submit = Clock::now();
  {
    std::lock_guard<std::mutex> lk(s->mu);
    r->id = s->next_id++;
    *request_id = r->id;
    s->pending.push_back(r.get());
    s->reqs[r->id] = std::move(r);
  }
  s->cv_work.notify_one();
  return FCLGPU_OK;
}

int fclgpu_server_wait(fclgpu_server s, int64_t id, double timeout_ms, fclgpu_motion_result* out) {
  if (!s || !out) return FCLGPU_ERR_INVALID_ARGUMENT;
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->reqs.find(id);
  if (it == s->reqs.end()) {
    set_error_detail("unknown request id");
    return FCLGPU_ERR_INVALID_ARGUMENT;
  }
  Request* r = it->second.get();
  auto ready = [&] { return r->done; };
  struct WaiterCount {  // lets destroy wait until no thread is left inside this call
    fclgpu_server_s* s;
    explicit WaiterCount(fclgpu_server_s* s_) : s(s_) { ++s->waiters; }
    ~WaiterCount() {
      --s->waiters;
      s->cv_done.notify_all();
    }
  } counted(s);
  if (timeout_ms < 0)
    s->cv_done.wait(lk, ready);
  else if (!s->cv_done.wait_for(lk, std::chrono::duration<double, std::milli>(timeout_ms), ready))
    return FCLGPU_ERR_PENDING;
  if (s->stop && r->res.reserved == FCLGPU_ERR_NOT_INITIALIZED) {
    set_error_detail("the server was destroyed before this request finished");
    return FCLGPU_ERR_NOT_INITIALIZED;
  }
  *out = r->res;
  const int rc = r->res.reserved;
  out->reserved = 0;
  s->reqs.erase(it);
  if (rc) set_error_detail("the step that processed this request failed");
  return rc;
}

int fclgpu_server_get_stats(fclgpu_server s, fclgpu_server_stats* out) {
  if (!s || !out) return FCLGPU_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lk(s->mu);
  *out = s->stats;
  return FCLGPU_OK;
}

int fclgpu_server_link_poses(fclgpu_server s, const double* base_tf, const double* q, int32_t K, double* out_tf) {
  if (!s || !base_tf || !q || K <= 0 || !out_tf) return FCLGPU_ERR_INVALID_ARGUMENT;
  const int L = s->L;
  const size_t nq = (size_t)K * L;
  double *dq = nullptr, *db = nullptr, *dt = nullptr;
  int32_t* ds = nullptr;
  int2* dr = nullptr;
  cudaError_t e = cudaMalloc(&dq, 8 * nq);
  if (e == cudaSuccess) e = cudaMalloc(&db, 96);
  if (e == cudaSuccess) e = cudaMalloc(&dt, 96 * nq);
  if (e == cudaSuccess) e = cudaMalloc(&ds, 4 * (size_t)K);
  if (e == cudaSuccess) e = cudaMalloc(&dr, 8 * nq);
  std::vector<int32_t> zero(K, 0);
  if (e == cudaSuccess) e = cudaMemcpy(dq, q, 8 * nq, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(db, base_tf, 96, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(ds, zero.data(), 4 * (size_t)K, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = launch_robot_fk(robot_dev(s), K, dq, ds, db, dt, dr, nullptr);
  if (e == cudaSuccess) e = cudaMemcpy(out_tf, dt, 96 * nq, cudaMemcpyDeviceToHost);
  for (void* p : {(void*)dq, (void*)db, (void*)dt, (void*)ds, (void*)dr})
    if (p) cudaFree(p);
  if (e != cudaSuccess) {
    set_error_detail(std::string("link poses: ") + cudaGetErrorString(e));
    return FCLGPU_ERR_CUDA;
  }
  return FCLGPU_OK;
}

int fclgpu_server_destroy(fclgpu_server s) {
  if (!s) return FCLGPU_OK;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
  }
  s->cv_work.notify_all();
  if (s->worker.joinable()) s->worker.join();
  cudaStreamSynchronize(s->stream);
  {
    // unfinished requests end with an error, and every thread blocked in
    // fclgpu_server_wait returns before the server's memory is released
    std::unique_lock<std::mutex> lk(s->mu);
    for (auto& kv : s->reqs) {
      Request* r = kv.second.get();
      if (!r->done) {
        r->res.reserved = FCLGPU_ERR_NOT_INITIALIZED;
        r->done = true;
      }
    }
    s->pending.clear();
    s->active.clear();
    s->cv_done.notify_all();
    s->cv_done.wait(lk, [&] { return s->waiters == 0; });
  }
  free_server(s);
  return FCLGPU_OK;
}

}  // extern "C"
