// Continuous collision of mesh pairs, FCL's default solver: continuousCollideNaive
// (narrowphase/continuous_collision-inl.h:134-171) with the translation (default), linear
// or screw motion (math/motion/, motion.cuh).  FCL samples the motion at
// n_iter = min(num_max_iterations, ceil(1 / toc_err)) times t_i = i / (n_iter - 1) and
// returns the first t_i at which the discrete collide() (default request: one contact)
// reports a collision.
//
// On the device every (query, sample) pair becomes one query of the collide batch:
// k_ccd_poses writes the sampled transforms, the batch runs with num_max_contacts = 1,
// and k_ccd_reduce takes the first colliding sample of each query.  Samples after the
// first colliding one are evaluated although FCL would skip them; they change nothing.
#include <cuda_runtime.h>

#include "geom.cuh"
#include "kernels.h"
#include "motion.cuh"

namespace fclgpu {

namespace {

__global__ void k_ccd_poses(CcdLaunch L) {
  const int64_t total = L.n * L.n_iter;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < total; k += stride) {
    const int64_t q = k / L.n_iter;
    const int64_t i = k - q * L.n_iter;
    const double t = (double)i / (double)(L.n_iter - 1);
    double a0[12], a1[12], b0[12], b1[12];
    for (int j = 0; j < 12; ++j) {
      if (L.tf1_beg) {
        a0[j] = __ldg(L.tf1_beg + 12 * q + j);
        a1[j] = __ldg(L.tf1_end + 12 * q + j);
      } else {
        a0[j] = a1[j] = (j == 0 || j == 5 || j == 10) ? 1.0 : 0.0;
      }
      b0[j] = __ldg(L.tf2_beg + 12 * q + j);
      b1[j] = __ldg(L.tf2_end + 12 * q + j);
    }
    motion_at(L.motion, a0, a1, t, L.tfa + 12 * k);
    motion_at(L.motion, b0, b1, t, L.tfb + 12 * k);
    L.pq_expanded[k] = L.pair_of_query ? __ldg(L.pair_of_query + q) : 0;
  }
}

__global__ void k_ccd_reduce(CcdLaunch L, const int32_t* counts) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < L.n; q += stride) {
    int64_t hit = -1;
    for (int64_t i = 0; i < L.n_iter; ++i)
      if (counts[q * L.n_iter + i] > 0) {
        hit = i;
        break;
      }
    L.is_collide[q] = hit >= 0 ? 1 : 0;
    L.toc[q] = hit >= 0 ? (double)hit / (double)(L.n_iter - 1) : 1.0;
    if (hit >= 0) {
      const int64_t k = q * L.n_iter + hit;
      if (L.contact_tf1)
        for (int j = 0; j < 12; ++j) L.contact_tf1[12 * q + j] = L.tfa[12 * k + j];
      if (L.contact_tf2)
        for (int j = 0; j < 12; ++j) L.contact_tf2[12 * q + j] = L.tfb[12 * k + j];
    }
  }
}

// ---------------------------------------------------------------------------------
// Conservative advancement (continuousCollide with CCDC_CONSERVATIVE_ADVANCEMENT) as FCL's
// oriented OBBRSS node computes it: conservativeAdvancementMeshOriented
// (conservative_advancement_func_matrix-inl.h:149-218) with
// MeshConservativeAdvancementTraversalNodeOBBRSS (mesh_conservative_advancement_
// traversal_node-inl.h:417-747).  After a discrete collide at the start poses (a batch
// before this kernel), each iteration runs FCL's distance traversal (no first-triangle
// seed; canStop c >= min_distance) under tf1^-1 tf2 of the motions' current transforms;
// every tested triangle pair gives d / (bound1 + bound2), the bounds being the
// TriangleMotionBoundVisitor visits of the two motions along the pair's direction turned
// into the world frame by motion 1's rotation; delta_t is their minimum (1 where the
// bound is <= d).  The BV motion bound of an OBBRSS node is 0 in FCL (its visitor has
// visits for RSS only), so the nodes never lower delta_t.  t advances by delta_t until
// delta_t <= 1e-5 (contact at t) or t > 1 (no contact).  FP64 in FCL's operation order.
// ---------------------------------------------------------------------------------
struct MotionCa {
  int type;
  double beg[12], end[12], cur[12];
  D3v vel;     // translation: trans_range; linear: linear_vel
  D3v axis;    // linear: angular axis; screw: axis
  double ang;  // angular velocity
  double lin;  // screw: linear velocity
  D3v p;       // screw: axis origin
};

__device__ void motion_ca_init(MotionCa& m, int type, const double* beg, const double* end) {
  m.type = type;
  for (int j = 0; j < 12; ++j) {
    m.beg[j] = beg[j];
    m.end[j] = end[j];
    m.cur[j] = beg[j];
  }
  m.ang = m.lin = 0.0;
  m.vel = m.axis = m.p = v3(0.0, 0.0, 0.0);
  const D3v t1 = trans_of_tf(beg), t2 = trans_of_tf(end);
  if (type == MOTION_TRANS) {
    m.vel = t2 - t1;
  } else if (type == MOTION_LINEAR) {
    relative_angle_axis(beg, end, m.ang, m.axis);
    double R1[9], R2[9];
    rot_of_tf(beg, R1);
    rot_of_tf(end, R2);
    M3<double> M1, M2;
    for (int k = 0; k < 9; ++k) {
      M1.m[k] = R1[k];
      M2.m[k] = R2[k];
    }
    const D3v o = v3(0.0, 0.0, 0.0);
    m.vel = (mulv(M2, o) + t2) - (mulv(M1, o) + t1);
  } else {
    relative_angle_axis(beg, end, m.ang, m.axis);
    if (m.ang < 1e-10) {
      m.ang = 0.0;
      m.axis = t2 - t1;
      m.lin = sqrt(sqnorm(m.axis));
      m.p = t1;
    } else {
      const D3v o = t2 - t1;
      m.p = d3scale((t1 + t2) + d3scale(cross(m.axis, o), 1.0 / tan(m.ang / 2.0)), 0.5);
      m.lin = dot(o, m.axis);
    }
  }
}

// TriangleMotionBoundVisitor::visit (math/motion/triangle_motion_bound_visitor-inl.h)
__device__ double tri_motion_bound(const MotionCa& m, const D3v* v, const D3v& n) {
  if (m.type == MOTION_TRANS) return dot(m.vel, n);
  M3<double> R;
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) R(r, c) = m.cur[4 * r + c];
  const D3v t = trans_of_tf(m.cur);
  double pm = 0.0;
  for (int k = 0; k < 3; ++k) {
    const D3v w = m.type == MOTION_LINEAR ? mulv(R, v[k] - v3(0.0, 0.0, 0.0)) : (mulv(R, v[k]) + t) - m.p;
    const double s = sqnorm(cross(w, m.axis));
    if (k == 0 || s > pm) pm = s;
  }
  pm = sqrt(pm);
  const double v_dot_n = m.type == MOTION_LINEAR ? dot(m.vel, n) : dot(m.axis, n) * m.lin;
  const double w_cross_n = sqrt(sqnorm(cross(m.axis, n))) * m.ang;
  return v_dot_n + w_cross_n * pm;
}

__device__ __forceinline__ double ca_rss_distance(const DevMesh& A, const DevMesh& B, int b1, int b2,
                                                  const M3<double>& R, const V3<double>& T) {
  const RssD& r1 = A.rss64[b1];
  const RssD& r2 = B.rss64[b2];
  M3<double> A1, A2;
  for (int i = 0; i < 9; ++i) {
    A1.m[i] = r1.axis[i];
    A2.m[i] = r2.axis[i];
  }
  const double l1[2] = {r1.l[0], r1.l[1]};
  const double l2[2] = {r2.l[0], r2.l[1]};
  return rss_distance<double>(R, T, A1, v3(r1.To[0], r1.To[1], r1.To[2]), l1, r1.r, A2,
                              v3(r2.To[0], r2.To[1], r2.To[2]), l2, r2.r);
}

struct CaStack {
  int b1, b2;
  double d;
};

// One CA iteration: FCL's distanceRecurse on the CA node; returns false on stack overflow.
template <int STACK>
__device__ bool ca_iteration(const DevMesh& A, const DevMesh& B, const MotionCa& m1, const MotionCa& m2,
                             double& delta_t) {
  M3<double> R;
  V3<double> T;
  rel_distance(m1.cur, m2.cur, R, T);  // tf1.inverse(Isometry) * tf2
  double R1[9];
  rot_of_tf(m1.cur, R1);
  const Quat R0 = quat_of_rotation(R1);
  double min_d = 1.7976931348623157e308;
  delta_t = 1.0;
  CaStack stk[STACK];
  int sp = 0;
  int b1 = 0, b2 = 0;
  for (;;) {
    const int c1 = A.nodes64[b1].child, c2 = B.nodes64[b2].child;
    const bool l1 = c1 < 0, l2 = c2 < 0;
    bool descend = false;
    if (l1 && l2) {
      const int p1 = -(c1 + 1), p2 = -(c2 + 1);
      D3v Al[3], Bl[3], Bw[3];
      for (int k = 0; k < 3; ++k) {
        const double* pa = A.verts64 + 3 * (long long)A.tris[3 * (long long)p1 + k];
        const double* pb = B.verts64 + 3 * (long long)B.tris[3 * (long long)p2 + k];
        Al[k] = v3(pa[0], pa[1], pa[2]);
        Bl[k] = v3(pb[0], pb[1], pb[2]);
        Bw[k] = mulv(R, Bl[k]) + T;
      }
      V3<double> P, Q;
      const double d = tri_distance<double>(Al, Bw, P, Q);
      if (d < min_d) min_d = d;
      D3v n = quat_rotate(R0, Q - P);
      const double z = sqnorm(n);
      if (z > 0) {
        const double s = sqrt(z);
        n = v3(n.x / s, n.y / s, n.z / s);
      }
      const double bound = tri_motion_bound(m1, Al, n) + tri_motion_bound(m2, Bl, v3(-n.x, -n.y, -n.z));
      const double cur = (bound <= d) ? 1.0 : d / bound;
      if (cur < delta_t) delta_t = cur;
    } else {
      int a1, a2, e1, e2;
      const bool fos = l2 ? true : (l1 ? false : size_key(A, b1) > size_key(B, b2));
      if (fos) {
        a1 = c1; a2 = b2; e1 = c1 + 1; e2 = b2;
      } else {
        a1 = b1; a2 = c2; e1 = b1; e2 = c2 + 1;
      }
      const double d1 = ca_rss_distance(A, B, a1, a2, R, T);
      const double d2 = ca_rss_distance(A, B, e1, e2, R, T);
      if (sp >= STACK) return false;
      int f1, f2;
      double fd;
      if (d2 < d1) {
        stk[sp++] = CaStack{a1, a2, d1};
        f1 = e1; f2 = e2; fd = d2;
      } else {
        stk[sp++] = CaStack{e1, e2, d2};
        f1 = a1; f2 = a2; fd = d1;
      }
      if (!(fd >= min_d)) {  // !canStop(fd)
        b1 = f1;
        b2 = f2;
        descend = true;
      }
    }
    if (descend) continue;
    bool found = false;
    while (sp > 0) {
      const CaStack e = stk[--sp];
      if (!(e.d >= min_d)) {
        b1 = e.b1;
        b2 = e.b2;
        found = true;
        break;
      }
    }
    if (!found) break;
  }
  return true;
}

template <int STACK>
__global__ void __launch_bounds__(128) k_ccd_ca(CcdLaunch L) {
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= L.n) return;
  double a0[12], a1[12], b0[12], b1[12];
  for (int j = 0; j < 12; ++j) {
    if (L.tf1_beg) {
      a0[j] = __ldg(L.tf1_beg + 12 * q + j);
      a1[j] = __ldg(L.tf1_end + 12 * q + j);
    } else {
      a0[j] = a1[j] = (j == 0 || j == 5 || j == 10) ? 1.0 : 0.0;
    }
    b0[j] = __ldg(L.tf2_beg + 12 * q + j);
    b1[j] = __ldg(L.tf2_end + 12 * q + j);
  }
  double toc = 0.0;
  bool hit;
  int64_t it = 0;
  if (L.hit0[q] > 0) {  // in collision at the start poses
    hit = true;
  } else {
    const int pi = L.pair_of_query ? __ldg(L.pair_of_query + q) : 0;
    if (pi < 0 || pi >= L.num_pairs) {
      atomicOr(L.status, DEV_ERR_PAIR);
      return;
    }
    const int2 mp = L.pairs[pi];
    const DevMesh A = L.meshes[mp.x];
    const DevMesh B = L.meshes[mp.y];
    MotionCa m1, m2;
    motion_ca_init(m1, L.motion, a0, a1);
    motion_ca_init(m2, L.motion, b0, b1);
    for (;;) {
      if (++it > L.max_iterations) {
        atomicOr(L.status, DEV_ERR_ITERATIONS);
        break;
      }
      double delta_t;
      if (!ca_iteration<STACK>(A, B, m1, m2, delta_t)) {
        atomicOr(L.status, DEV_ERR_STACK);
        break;
      }
      if (delta_t <= 0.00001) break;  // t_err
      toc += delta_t;
      if (toc > 1.0) {
        toc = 1.0;
        break;
      }
      motion_at(L.motion, m1.beg, m1.end, toc, m1.cur);
      motion_at(L.motion, m2.beg, m2.end, toc, m2.cur);
    }
    hit = toc < 1.0;
  }
  L.is_collide[q] = hit ? 1 : 0;
  L.toc[q] = toc;
  if (L.iterations) L.iterations[q] = (int32_t)it;
  if (hit) {  // the motions integrated to the time of contact
    if (L.contact_tf1) motion_at(L.motion, a0, a1, toc, L.contact_tf1 + 12 * q);
    if (L.contact_tf2) motion_at(L.motion, b0, b1, toc, L.contact_tf2 + 12 * q);
  }
}

unsigned ccd_grid(int64_t items, int block) {
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

cudaError_t launch_ccd_poses(const CcdLaunch& L, cudaStream_t s) {
  if (L.n <= 0 || L.n_iter <= 0) return cudaSuccess;
  k_ccd_poses<<<ccd_grid(L.n * L.n_iter, 128), 128, 0, s>>>(L);
  ++g_kernel_launches;
  return cudaGetLastError();
}

cudaError_t launch_ccd_ca(const CcdLaunch& L, int stack_entries, cudaStream_t s) {
  if (L.n <= 0) return cudaSuccess;
  const unsigned grid = (unsigned)((L.n + 127) / 128);
  if (stack_entries <= 64)
    k_ccd_ca<64><<<grid, 128, 0, s>>>(L);
  else
    k_ccd_ca<256><<<grid, 128, 0, s>>>(L);
  ++g_kernel_launches;
  return cudaGetLastError();
}

cudaError_t launch_ccd_reduce(const CcdLaunch& L, const int32_t* counts, cudaStream_t s) {
  if (L.n <= 0) return cudaSuccess;
  k_ccd_reduce<<<ccd_grid(L.n, 256), 256, 0, s>>>(L, counts);
  ++g_kernel_launches;
  return cudaGetLastError();
}

}  // namespace fclgpu
