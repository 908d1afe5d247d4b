// Device construction of a BVHModel<OBBRSS> tree, bit-identical to the host build
// (bvh_build.cpp, which follows BVHModel::buildTree / recursiveBuildTree,
// geometry/bvh/BVH_model-inl.h:833-938, BVFitter<OBBRSS>, BV_fitter-inl.h:448-478, and the
// MEAN splitter, BV_splitter-inl.h:422-546).
//
// The tree is built level by level.  A task is a node: its id, its span [first, first +
// count) of the primitive permutation, and its preorder position and the number of leaves
// before it in preorder, from which the ids of its children follow: FCL allocates two ids
// per internal node in depth-first order, so the children of node v get
// 1 + 2 (internal nodes before v in preorder) = 1 + 2 (pre(v) - leaves_before(v)).
//
// Every sum of the fit runs in the host's order (FP64 addition is not associative): the
// nine covariance sums are nine sequential chains over the span, one lane each; the
// split value reuses the first three (the mean splitter sums the same terms in the same
// order).  Minima and maxima keep the first element among equal values (the host's
// strict comparisons), which matters only for the sign of a zero; argmin/argmax take the
// first index.  The rectangle extents of the RSS fit are order-free minima and maxima
// (a point can lower the running minimum only with a value the final minimum takes
// into account); the corner adjustments are sequential and run over the points outside
// the rectangle in both coordinates, in order.  The Lomuto partition of the span is
// reproduced exactly: the left part is the left elements in order; the right part is the
// tail of a log in which every right element is appended and every left element met
// while the queue of rights is non-empty appends a copy of the log entry at its rotation
// index (the queue's front), so the log resolves front to back.
//
// Tasks with up to kSmallTask primitives run the host algorithm verbatim, one thread
// each; up to kBlockTask, one warp each (lanes share the per-point work, lane 0 the
// sequential parts); larger ones (the top levels, few tasks) one block of kBT threads
// each, so that the per-point passes are not held to one warp's latency.
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <climits>
#include <cstring>
#include <vector>

#include "kernels.h"
#include "refit.cuh"

namespace fclgpu {

namespace {

constexpr int kSmallTask = 16;
constexpr int kBlockTask = 4096;
constexpr int kBT = 512;        // threads of a block task
constexpr int kChainChunk = 512;

struct BuildTask {
  int32_t id, first, count, pre, lb;
};

__device__ __forceinline__ double dotd3(const double* a, double x, double y, double z) {
  return (a[0] * x + a[1] * y) + a[2] * z;
}

// Per triangle: the nine covariance terms in Builder::fit's forms and the centroid the
// splitter tests ((p1 + p2) + p3) / 3.
__global__ void k_bvh_tri_terms(const double* V, const int32_t* T, int nt, double* T9, double* C3) {
  const int stride = gridDim.x * blockDim.x;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nt; t += stride) {
    const double* a = V + 3 * (long long)T[3 * t];
    const double* b = V + 3 * (long long)T[3 * t + 1];
    const double* c = V + 3 * (long long)T[3 * t + 2];
    double* o = T9 + 9 * (long long)t;
    o[0] = (a[0] + b[0]) + c[0];
    o[1] = (a[1] + b[1]) + c[1];
    o[2] = (a[2] + b[2]) + c[2];
    o[3] = (a[0] * a[0] + b[0] * b[0]) + c[0] * c[0];
    o[4] = (a[1] * a[1] + b[1] * b[1]) + c[1] * c[1];
    o[5] = (a[2] * a[2] + b[2] * b[2]) + c[2] * c[2];
    o[6] = (a[0] * a[1] + b[0] * b[1]) + c[0] * c[1];
    o[7] = (a[0] * a[2] + b[0] * b[2]) + c[0] * c[2];
    o[8] = (a[1] * a[2] + b[1] * b[2]) + c[1] * c[2];
    double* q = C3 + 3 * (long long)t;
    q[0] = ((a[0] + b[0]) + c[0]) / 3.0;
    q[1] = ((a[1] + b[1]) + c[1]) / 3.0;
    q[2] = ((a[2] + b[2]) + c[2]) / 3.0;
  }
}

__device__ __forceinline__ void jrot(double& x, double& y, double s, double tau) {
  const double g = x, h = y;
  x = g - s * (h + g * tau);
  y = h + s * (g - h * tau);
}

// Cyclic Jacobi (FCL's eigen_old), evecs[k] = k-th eigenvector; as Builder::jacobi.
__device__ void jacobi3(const double C[3][3], double evals[3], double evecs[3][3]) {
  double R[3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) R[i][j] = C[i][j];
  double v[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
  double b[3], d[3], z[3];
  for (int p = 0; p < 3; ++p) {
    b[p] = d[p] = R[p][p];
    z[p] = 0;
  }
  for (int k = 0; k < 3; ++k) {
    evals[k] = 0;
    for (int j = 0; j < 3; ++j) evecs[k][j] = (k == j) ? 1.0 : 0.0;
  }
  for (int sweep = 0; sweep < 50; ++sweep) {
    double sm = 0;
    for (int p = 0; p < 3; ++p)
      for (int q = p + 1; q < 3; ++q) sm += fabs(R[p][q]);
    if (sm == 0.0) {
      for (int k = 0; k < 3; ++k) {
        evals[k] = d[k];
        for (int j = 0; j < 3; ++j) evecs[k][j] = v[j][k];
      }
      return;
    }
    const double tresh = (sweep < 3) ? 0.2 * sm / (3 * 3) : 0.0;
    for (int p = 0; p < 3; ++p) {
      for (int q = p + 1; q < 3; ++q) {
        const double g = 100.0 * fabs(R[p][q]);
        if (sweep > 3 && fabs(d[p]) + g == fabs(d[p]) && fabs(d[q]) + g == fabs(d[q])) {
          R[p][q] = 0.0;
        } else if (fabs(R[p][q]) > tresh) {
          double h = d[q] - d[p];
          double t;
          if (fabs(h) + g == fabs(h)) {
            t = (R[p][q]) / h;
          } else {
            const double theta = 0.5 * h / (R[p][q]);
            t = 1.0 / (fabs(theta) + sqrt(1.0 + theta * theta));
            if (theta < 0.0) t = -t;
          }
          const double c = 1.0 / sqrt(1 + t * t);
          const double s = t * c;
          const double tau = s / (1.0 + c);
          h = t * R[p][q];
          z[p] -= h;
          z[q] += h;
          d[p] -= h;
          d[q] += h;
          R[p][q] = 0.0;
          for (int j = 0; j < p; ++j) jrot(R[j][p], R[j][q], s, tau);
          for (int j = p + 1; j < q; ++j) jrot(R[p][j], R[j][q], s, tau);
          for (int j = q + 1; j < 3; ++j) jrot(R[p][j], R[q][j], s, tau);
          for (int j = 0; j < 3; ++j) jrot(v[j][p], v[j][q], s, tau);
        }
      }
    }
    for (int p = 0; p < 3; ++p) {
      b[p] += z[p];
      d[p] = b[p];
      z[p] = 0.0;
    }
  }
  // no convergence in 50 sweeps: FCL leaves its outputs unchanged; identity as the host
}

// Covariance sums -> node axes (row-major, column k the k-th axis) as Builder::fit
__device__ void axes_from_sums(const double s[9], int n, double axis[9]) {
  const int np = 3 * n;
  const double s1x = s[0], s1y = s[1], s1z = s[2], sxx = s[3], syy = s[4], szz = s[5], sxy = s[6], sxz = s[7],
               syz = s[8];
  double C[3][3];
  C[0][0] = sxx - s1x * s1x / np;
  C[1][1] = syy - s1y * s1y / np;
  C[2][2] = szz - s1z * s1z / np;
  C[0][1] = sxy - s1x * s1y / np;
  C[1][2] = syz - s1y * s1z / np;
  C[0][2] = sxz - s1x * s1z / np;
  C[1][0] = C[0][1];
  C[2][0] = C[0][2];
  C[2][1] = C[1][2];
  double evals[3], evecs[3][3];
  jacobi3(C, evals, evecs);
  int lo, mid, hi;
  if (evals[0] > evals[1]) {
    hi = 0;
    lo = 1;
  } else {
    lo = 0;
    hi = 1;
  }
  if (evals[2] < evals[lo]) {
    mid = lo;
    lo = 2;
  } else if (evals[2] > evals[hi]) {
    mid = hi;
    hi = 2;
  } else {
    mid = 2;
  }
  const double a0[3] = {evecs[hi][0], evecs[hi][1], evecs[hi][2]};
  const double a1[3] = {evecs[mid][0], evecs[mid][1], evecs[mid][2]};
  const double a2[3] = {a0[1] * a1[2] - a0[2] * a1[1], a0[2] * a1[0] - a0[0] * a1[2], a0[0] * a1[1] - a0[1] * a1[0]};
  for (int r = 0; r < 3; ++r) {
    axis[3 * r + 0] = a0[r];
    axis[3 * r + 1] = a1[r];
    axis[3 * r + 2] = a2[r];
  }
}

__device__ __forceinline__ void proj_point(const double ax[3][3], const double* p, double o[3]) {
  for (int k = 0; k < 3; ++k) o[k] = (ax[k][0] * p[0] + ax[k][1] * p[1]) + ax[k][2] * p[2];
}

// OBB extent and centre from the projections' minima and maxima (getExtentAndCenter)
__device__ void obb_from_extremes(const double mn[3], const double mx[3], NodeD& nd) {
  const double o0 = (mx[0] + mn[0]) / 2, o1 = (mx[1] + mn[1]) / 2, o2 = (mx[2] + mn[2]) / 2;
  for (int r = 0; r < 3; ++r) nd.To[r] = (nd.axis[3 * r] * o0 + nd.axis[3 * r + 1] * o1) + nd.axis[3 * r + 2] * o2;
  nd.ext[0] = (mx[0] - mn[0]) / 2;
  nd.ext[1] = (mx[1] - mn[1]) / 2;
  nd.ext[2] = (mx[2] - mn[2]) / 2;
}

__device__ __forceinline__ double rss_cap(double z, double cz, double radsqr) {
  const double dz = z - cz;
  const double v = radsqr - dz * dz;
  return sqrt(v > 0 ? v : 0.0);
}

// One corner step of getRadiusAndOriginAndRectangleSize (the host's loop body); returns
// whether it moves the rectangle.  APPLY = false evaluates the step without applying it.
template <bool APPLY = true>
__device__ bool rss_corner(double X, double Y, double Z, double cz, double radsqr, double& minx, double& maxx,
                           double& miny, double& maxy) {
  const double a = sqrt(0.5);
  if (X > maxx) {
    if (Y > maxy) {
      const double dx = X - maxx, dy = Y - maxy;
      double u = dx * a + dy * a;
      const double t = (a * u - dx) * (a * u - dx) + (a * u - dy) * (a * u - dy) + (cz - Z) * (cz - Z);
      const double w = radsqr - t;
      u = u - sqrt(w > 0 ? w : 0.0);
      if (u > 0) {
        if (APPLY) {
          maxx += u * a;
          maxy += u * a;
        }
        return true;
      }
    } else if (Y < miny) {
      const double dx = X - maxx, dy = Y - miny;
      double u = dx * a - dy * a;
      const double t = (a * u - dx) * (a * u - dx) + (-a * u - dy) * (-a * u - dy) + (cz - Z) * (cz - Z);
      const double w = radsqr - t;
      u = u - sqrt(w > 0 ? w : 0.0);
      if (u > 0) {
        if (APPLY) {
          maxx += u * a;
          miny -= u * a;
        }
        return true;
      }
    }
  } else if (X < minx) {
    if (Y > maxy) {
      const double dx = X - minx, dy = Y - maxy;
      double u = dy * a - dx * a;
      const double t = (-a * u - dx) * (-a * u - dx) + (a * u - dy) * (a * u - dy) + (cz - Z) * (cz - Z);
      const double w = radsqr - t;
      u = u - sqrt(w > 0 ? w : 0.0);
      if (u > 0) {
        if (APPLY) {
          minx -= u * a;
          maxy += u * a;
        }
        return true;
      }
    } else if (Y < miny) {
      const double dx = X - minx, dy = Y - miny;
      double u = -dx * a - dy * a;
      const double t = (-a * u - dx) * (-a * u - dx) + (-a * u - dy) * (-a * u - dy) + (cz - Z) * (cz - Z);
      const double w = radsqr - t;
      u = u - sqrt(w > 0 ? w : 0.0);
      if (u > 0) {
        if (APPLY) {
          minx -= u * a;
          miny -= u * a;
        }
        return true;
      }
    }
  }
  return false;
}

__device__ void rss_write(const double ax[3][3], double minx, double maxx, double miny, double maxy, double cz,
                          double r, const double axis9[9], RssD& rs) {
  for (int k = 0; k < 3; ++k) {
    const double ox = ax[0][k] * minx, oy = ax[1][k] * miny, oz = ax[2][k] * cz;
    rs.To[k] = (ox + oy) + oz;
  }
  rs.l[0] = maxx - minx;
  if (rs.l[0] < 0) rs.l[0] = 0;
  rs.l[1] = maxy - miny;
  if (rs.l[1] < 0) rs.l[1] = 0;
  rs.r = r;
  for (int k = 0; k < 9; ++k) rs.axis[k] = axis9[k];
}

__device__ __forceinline__ int32_t child_base(const BuildTask& t) { return 1 + 2 * (t.pre - t.lb); }

// ---------------------------------------------------------------------------------
// Small tasks: the host algorithm, one thread per task
// ---------------------------------------------------------------------------------
__global__ void __launch_bounds__(128) k_bvh_small(const BuildTask* tasks, int ntasks, const double* V,
                                                   const int32_t* T, const double* T9, const double* C3,
                                                   uint32_t* prim, NodeD* nodes, RssD* rss, int32_t* left_out) {
  const int ti = blockIdx.x * blockDim.x + threadIdx.x;
  if (ti >= ntasks) return;
  const BuildTask tk = tasks[ti];
  if (tk.count > kSmallTask) return;
  const int n = tk.count;
  uint32_t* span = prim + tk.first;
  double s[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  for (int i = 0; i < n; ++i) {
    const double* o = T9 + 9 * (long long)span[i];
    for (int k = 0; k < 9; ++k) s[k] += o[k];
  }
  NodeD nd;
  axes_from_sums(s, n, nd.axis);
  double ax[3][3];
  for (int k = 0; k < 3; ++k)
    for (int c = 0; c < 3; ++c) ax[k][c] = nd.axis[3 * c + k];
  auto proj = [&](int e, double o[3]) {
    const double* p = V + 3 * (long long)T[3 * (long long)span[e / 3] + e % 3];
    proj_point(ax, p, o);
  };
  const int np = 3 * n;
  const double big = DBL_MAX;
  double mn[3] = {big, big, big}, mx[3] = {-big, -big, -big};
  for (int e = 0; e < np; ++e) {
    double P[3];
    proj(e, P);
    for (int k = 0; k < 3; ++k) {
      if (P[k] > mx[k]) mx[k] = P[k];
      if (P[k] < mn[k]) mn[k] = P[k];
    }
  }
  obb_from_extremes(mn, mx, nd);
  // RSS (getRadiusAndOriginAndRectangleSize) as the host's rss_fit
  double P0[3];
  proj(0, P0);
  double minz = P0[2], maxz = P0[2];
  for (int e = 1; e < np; ++e) {
    double P[3];
    proj(e, P);
    if (P[2] < minz)
      minz = P[2];
    else if (P[2] > maxz)
      maxz = P[2];
  }
  const double r = 0.5 * (maxz - minz);
  const double radsqr = r * r;
  const double cz = 0.5 * (maxz + minz);
  double ext[2][2];  // [x|y][min|max]
  for (int c = 0; c < 2; ++c) {
    int imin = 0, imax = 0;
    double vmin = P0[c], vmax = P0[c];
    for (int e = 1; e < np; ++e) {
      double P[3];
      proj(e, P);
      if (P[c] < vmin) {
        imin = e;
        vmin = P[c];
      } else if (P[c] > vmax) {
        imax = e;
        vmax = P[c];
      }
    }
    double Pm[3], PM[3];
    proj(imin, Pm);
    proj(imax, PM);
    double lo = Pm[c] + rss_cap(Pm[2], cz, radsqr);
    double hi = PM[c] - rss_cap(PM[2], cz, radsqr);
    for (int e = 0; e < np; ++e) {
      double P[3];
      proj(e, P);
      if (P[c] < lo) {
        const double x = P[c] + rss_cap(P[2], cz, radsqr);
        if (x < lo) lo = x;
      }
    }
    for (int e = 0; e < np; ++e) {
      double P[3];
      proj(e, P);
      if (P[c] > hi) {
        const double x = P[c] - rss_cap(P[2], cz, radsqr);
        if (x > hi) hi = x;
      }
    }
    ext[c][0] = lo;
    ext[c][1] = hi;
  }
  double minx = ext[0][0], maxx = ext[0][1], miny = ext[1][0], maxy = ext[1][1];
  for (int e = 0; e < np; ++e) {
    double P[3];
    proj(e, P);
    rss_corner(P[0], P[1], P[2], cz, radsqr, minx, maxx, miny, maxy);
  }
  RssD rs;
  rss_write(ax, minx, maxx, miny, maxy, cz, r, nd.axis, rs);
  rss[tk.id] = rs;
  if (n == 1) {
    nd.child = -((int)span[0] + 1);
    nd.pad = 0;
    nodes[tk.id] = nd;
    left_out[ti] = 0;
    return;
  }
  // mean split along the first axis and the Lomuto partition
  const double split = ((s[0] * ax[0][0] + s[1] * ax[0][1]) + s[2] * ax[0][2]) / (3 * n);
  int left = 0;
  for (int i = 0; i < n; ++i) {
    const double* c = C3 + 3 * (long long)span[i];
    if (!(dotd3(ax[0], c[0], c[1], c[2]) > split)) {
      const uint32_t tmp = span[i];
      span[i] = span[left];
      span[left] = tmp;
      ++left;
    }
  }
  if (left == 0 || left == n) left = n / 2;
  nd.child = child_base(tk);
  nd.pad = 0;
  nodes[tk.id] = nd;
  left_out[ti] = left;
}

// ---------------------------------------------------------------------------------
// Larger tasks: one warp each
// ---------------------------------------------------------------------------------
constexpr int kWarpsPerBlock = 4;

// (value, index) with the smaller index winning among equal values
struct VI {
  double v;
  int i;
};
__device__ __forceinline__ VI vi_min(VI a, VI b) { return (b.v < a.v || (b.v == a.v && b.i < a.i)) ? b : a; }
__device__ __forceinline__ VI vi_max(VI a, VI b) { return (b.v > a.v || (b.v == a.v && b.i < a.i)) ? b : a; }
__device__ __forceinline__ VI shfl_vi(VI a, int off) {
  VI r;
  r.v = __shfl_xor_sync(0xffffffffu, a.v, off);
  r.i = __shfl_xor_sync(0xffffffffu, a.i, off);
  return r;
}
__device__ __forceinline__ VI warp_min(VI a) {
  for (int off = 16; off > 0; off >>= 1) a = vi_min(a, shfl_vi(a, off));
  return a;
}
__device__ __forceinline__ VI warp_max(VI a) {
  for (int off = 16; off > 0; off >>= 1) a = vi_max(a, shfl_vi(a, off));
  return a;
}

__global__ void __launch_bounds__(32 * kWarpsPerBlock) k_bvh_warp(const BuildTask* tasks, int ntasks, const double* V,
                                                                  const int32_t* T, const double* T9,
                                                                  const double* C3, uint32_t* prim, NodeD* nodes,
                                                                  RssD* rss, int32_t* left_out, double* Pbuf,
                                                                  int32_t* Bbuf, uint32_t* spanbuf) {
  __shared__ double sterm[kWarpsPerBlock][32][9];
  __shared__ int32_t sB[kWarpsPerBlock][32];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int ti = blockIdx.x * kWarpsPerBlock + w;
  if (ti >= ntasks) return;
  const BuildTask tk = tasks[ti];
  if (tk.count <= kSmallTask || tk.count > kBlockTask) return;
  const unsigned full = 0xffffffffu;
  const int n = tk.count, f = tk.first;
  const uint32_t* span = prim + f;
  // (1) the nine covariance chains, lane k < 9 owns sum k
  double acc = 0.0;
  for (int base = 0; base < n; base += 32) {
    const int m = min(32, n - base);
    if (lane < m) {
      const double* o = T9 + 9 * (long long)span[base + lane];
#pragma unroll
      for (int k = 0; k < 9; ++k) sterm[w][lane][k] = o[k];
    }
    __syncwarp();
    if (lane < 9) {
      int j = 0;
      for (; j + 8 <= m; j += 8) {
        double t[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) t[u] = sterm[w][j + u][lane];
#pragma unroll
        for (int u = 0; u < 8; ++u) acc += t[u];
      }
      for (; j < m; ++j) acc += sterm[w][j][lane];
    }
    __syncwarp();
  }
  double s[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) s[k] = __shfl_sync(full, acc, k);
  // (2) axes on lane 0, broadcast
  NodeD nd;
  if (lane == 0) axes_from_sums(s, n, nd.axis);
#pragma unroll
  for (int k = 0; k < 9; ++k) nd.axis[k] = __shfl_sync(full, nd.axis[k], 0);
  double ax[3][3];
  for (int k = 0; k < 3; ++k)
    for (int c = 0; c < 3; ++c) ax[k][c] = nd.axis[3 * c + k];
  // (3) projections of the 3n points (stored), extremes with first-index ties
  const int np = 3 * n;
  double* P = Pbuf + 9 * (long long)f;
  const double big = DBL_MAX;
  VI mn[3], mx[3];
  for (int k = 0; k < 3; ++k) {
    mn[k] = VI{big, INT_MAX};
    mx[k] = VI{-big, INT_MAX};
  }
  for (int e = lane; e < np; e += 32) {
    const double* p = V + 3 * (long long)T[3 * (long long)span[e / 3] + e % 3];
    double o[3];
    proj_point(ax, p, o);
    for (int k = 0; k < 3; ++k) {
      P[3 * e + k] = o[k];
      mn[k] = vi_min(mn[k], VI{o[k], e});
      mx[k] = vi_max(mx[k], VI{o[k], e});
    }
  }
  for (int k = 0; k < 3; ++k) {
    mn[k] = warp_min(mn[k]);
    mx[k] = warp_max(mx[k]);
  }
  __syncwarp();
  {
    const double mnv[3] = {mn[0].v, mn[1].v, mn[2].v}, mxv[3] = {mx[0].v, mx[1].v, mx[2].v};
    obb_from_extremes(mnv, mxv, nd);
  }
  // (4) RSS: z extremes are the OBB's (first among equals either way)
  const double minz = mn[2].v, maxz = mx[2].v;
  const double r = 0.5 * (maxz - minz);
  const double radsqr = r * r;
  const double cz = 0.5 * (maxz + minz);
  double ext[2][2];
  for (int c = 0; c < 2; ++c) {
    // imin / imax: the first index of the extreme value
    const int imin = mn[c].i, imax = mx[c].i;
    const double lo0 = P[3 * imin + c] + rss_cap(P[3 * imin + 2], cz, radsqr);
    const double hi0 = P[3 * imax + c] - rss_cap(P[3 * imax + 2], cz, radsqr);
    VI lo{lo0, -1}, hi{hi0, -1};
    for (int e = lane; e < np; e += 32) {
      const double pc = P[3 * e + c];
      if (pc < lo.v) lo = vi_min(lo, VI{pc + rss_cap(P[3 * e + 2], cz, radsqr), e});
      if (pc > hi.v) hi = vi_max(hi, VI{pc - rss_cap(P[3 * e + 2], cz, radsqr), e});
    }
    ext[c][0] = warp_min(lo).v;
    ext[c][1] = warp_max(hi).v;
  }
  double minx = ext[0][0], maxx = ext[0][1], miny = ext[1][0], maxy = ext[1][1];
  {
    // corners: only points outside the rectangle in x and in y can move it; in order
    const double x0 = minx, x1 = maxx, y0 = miny, y1 = maxy;
    for (int base = 0; base < np; base += 32) {
      const int e = base + lane;
      bool cand = false;
      if (e < np) {
        const double X = P[3 * e], Y = P[3 * e + 1];
        cand = (X > x1 || X < x0) && (Y > y1 || Y < y0);
      }
      // as in k_bvh_block: evaluate the remaining candidates against the current rectangle,
      // apply the first that moves it, repeat after it (the rectangle is the same in every lane)
      unsigned pending = __ballot_sync(full, cand);
      while (pending) {
        bool moves = false;
        if ((pending >> lane) & 1u) {
          double a0 = minx, a1 = maxx, a2 = miny, a3 = maxy;
          moves = rss_corner<false>(P[3 * e], P[3 * e + 1], P[3 * e + 2], cz, radsqr, a0, a1, a2, a3);
        }
        const unsigned mv = __ballot_sync(full, moves);
        if (!mv) break;
        const int b = __ffs(mv) - 1;
        const int ee = base + b;
        rss_corner<true>(P[3 * ee], P[3 * ee + 1], P[3 * ee + 2], cz, radsqr, minx, maxx, miny, maxy);
        pending &= ~((2u << b) - 1u);  // the candidates after b
      }
    }
  }
  if (lane == 0) {
    RssD rs;
    rss_write(ax, minx, maxx, miny, maxy, cz, r, nd.axis, rs);
    rss[tk.id] = rs;
  }
  // (5) mean split and the Lomuto partition (n > kSmallTask >= 1 here)
  const double split = ((s[0] * ax[0][0] + s[1] * ax[0][1]) + s[2] * ax[0][2]) / (3 * n);
  int32_t* B = Bbuf + 2 * (long long)f;  // the log, <= 2n entries
  uint32_t* out = spanbuf + f;
  const unsigned lt = (1u << lane) - 1u;
  int nR = 0, nRot = 0, nL = 0;  // running counts (warp-uniform)
  for (int base = 0; base < n; base += 32) {
    const int i = base + lane;
    bool isL = false, isR = false;
    uint32_t pv = 0;
    if (i < n) {
      pv = span[i];
      const double* c = C3 + 3 * (long long)pv;
      isL = !(dotd3(ax[0], c[0], c[1], c[2]) > split);
      isR = !isL;
    }
    const unsigned mR = __ballot_sync(full, isR);
    const int rb = nR + __popc(mR & lt);          // rights before i
    const bool rot = isL && rb > 0;               // a left met while the queue is non-empty
    const unsigned mRot = __ballot_sync(full, rot);
    const int ob = nRot + __popc(mRot & lt);      // rotations before i
    const unsigned mL = __ballot_sync(full, isL);
    if (isL) out[nL + __popc(mL & lt)] = pv;      // lefts keep their order
    if (isR) B[rb + ob] = (int32_t)pv;            // append
    if (rot) B[rb + ob] = -(ob + 1);              // copy of the entry at the rotation index
    nR += __popc(mR);
    nRot += __popc(mRot);
    nL += __popc(mL);
  }
  __syncwarp();
  // resolve the log front to back: an entry refers only to an earlier one
  const int lenB = nR + nRot;
  for (int base = 0; base < lenB; base += 32) {
    const int k = base + lane;
    int32_t v = (k < lenB) ? B[k] : 0;
    if (k < lenB && v < 0) {
      const int j = -v - 1;
      if (j < base) v = B[j];
    }
    sB[w][lane] = v;
    __syncwarp();
    // references inside this chunk resolve in at most 32 passes
    for (int pass = 0; pass < 32; ++pass) {
      const bool pending = (k < lenB) && (v < 0);
      if (!__any_sync(full, pending)) break;
      if (pending) {
        const int j = -v - 1;
        const int32_t t = sB[w][j - base];
        if (t >= 0) v = t;
      }
      __syncwarp();
      sB[w][lane] = v;
      __syncwarp();
    }
    if (k < lenB) B[k] = v;
    __syncwarp();
  }
  for (int t = lane; t < nR; t += 32) out[nL + t] = (uint32_t)B[nRot + t];
  __syncwarp();
  for (int t = lane; t < n; t += 32) prim[f + t] = out[t];
  int left = nL;
  if (left == 0 || left == n) left = n / 2;
  if (lane == 0) {
    nd.child = child_base(tk);
    nd.pad = 0;
    nodes[tk.id] = nd;
    left_out[ti] = left;
  }
}

// ---------------------------------------------------------------------------------
// The largest tasks: one block of kBT threads each, the same steps as k_bvh_warp
// ---------------------------------------------------------------------------------
constexpr int kBW = kBT / 32;

struct BlockScratch {
  double term[kChainChunk][9];
  double vv[kBW][8];
  int ii[kBW][8];
  int cnt[3][kBW];
  int32_t B[kBT];
  int32_t cand[kBT];
  double s9[9];
  double axis[9];
  double rect[4];
  int ncand;
};

// block-wide (value, index) reductions; every thread receives the result
__device__ VI block_min_vi(VI a, BlockScratch& sh, int slot) {
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  a = warp_min(a);
  if (lane == 0) {
    sh.vv[w][slot] = a.v;
    sh.ii[w][slot] = a.i;
  }
  __syncthreads();
  VI r{sh.vv[0][slot], sh.ii[0][slot]};
  for (int k = 1; k < kBW; ++k) r = vi_min(r, VI{sh.vv[k][slot], sh.ii[k][slot]});
  __syncthreads();
  return r;
}
__device__ VI block_max_vi(VI a, BlockScratch& sh, int slot) {
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  a = warp_max(a);
  if (lane == 0) {
    sh.vv[w][slot] = a.v;
    sh.ii[w][slot] = a.i;
  }
  __syncthreads();
  VI r{sh.vv[0][slot], sh.ii[0][slot]};
  for (int k = 1; k < kBW; ++k) r = vi_max(r, VI{sh.vv[k][slot], sh.ii[k][slot]});
  __syncthreads();
  return r;
}

// exclusive counts of three flags over the block (thread order) and their totals
__device__ void block_counts3(const bool f[3], int before[3], int total[3], BlockScratch& sh) {
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const unsigned lt = (1u << lane) - 1u;
  unsigned m[3];
  for (int c = 0; c < 3; ++c) {
    m[c] = __ballot_sync(0xffffffffu, f[c]);
    if (lane == 0) sh.cnt[c][w] = __popc(m[c]);
  }
  __syncthreads();
  for (int c = 0; c < 3; ++c) {
    int b = 0, t = 0;
    for (int k = 0; k < kBW; ++k) {
      if (k < w) b += sh.cnt[c][k];
      t += sh.cnt[c][k];
    }
    before[c] = b + __popc(m[c] & lt);
    total[c] = t;
  }
  __syncthreads();
}

__global__ void __launch_bounds__(kBT) k_bvh_block(const BuildTask* tasks, int ntasks, const double* V,
                                                   const int32_t* T, const double* T9, const double* C3,
                                                   uint32_t* prim, NodeD* nodes, RssD* rss, int32_t* left_out,
                                                   double* Pbuf, int32_t* Bbuf, uint32_t* spanbuf) {
  extern __shared__ __align__(16) unsigned char smem[];
  BlockScratch& sh = *reinterpret_cast<BlockScratch*>(smem);
  const int ti = blockIdx.x;
  if (ti >= ntasks) return;
  const BuildTask tk = tasks[ti];
  if (tk.count <= kBlockTask) return;
  const int tid = threadIdx.x;
  const int n = tk.count, f = tk.first;
  const uint32_t* span = prim + f;
  // (1) covariance chains: thread k < 9 owns sum k, all threads stage the terms
  double acc = 0.0;
  for (int base = 0; base < n; base += kChainChunk) {
    const int m = min(kChainChunk, n - base);
    for (int t = tid; t < m; t += kBT) {
      const double* o = T9 + 9 * (long long)span[base + t];
#pragma unroll
      for (int k = 0; k < 9; ++k) sh.term[t][k] = o[k];
    }
    __syncthreads();
    if (tid < 9) {
      // loads issued ahead of the dependent additions (no padding term: adding +0
      // would turn a -0 sum into +0)
      int j = 0;
      for (; j + 8 <= m; j += 8) {
        double t[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) t[u] = sh.term[j + u][tid];
#pragma unroll
        for (int u = 0; u < 8; ++u) acc += t[u];
      }
      for (; j < m; ++j) acc += sh.term[j][tid];
    }
    __syncthreads();
  }
  if (tid < 9) sh.s9[tid] = acc;
  __syncthreads();
  double s[9];
  for (int k = 0; k < 9; ++k) s[k] = sh.s9[k];
  NodeD nd;
  if (tid == 0) {
    axes_from_sums(s, n, nd.axis);
    for (int k = 0; k < 9; ++k) sh.axis[k] = nd.axis[k];
  }
  __syncthreads();
  for (int k = 0; k < 9; ++k) nd.axis[k] = sh.axis[k];
  double ax[3][3];
  for (int k = 0; k < 3; ++k)
    for (int c = 0; c < 3; ++c) ax[k][c] = nd.axis[3 * c + k];
  // (2) projections and their extremes
  const int np = 3 * n;
  double* P = Pbuf + 9 * (long long)f;
  const double big = DBL_MAX;
  VI mn[3], mx[3];
  for (int k = 0; k < 3; ++k) {
    mn[k] = VI{big, INT_MAX};
    mx[k] = VI{-big, INT_MAX};
  }
  for (int e = tid; e < np; e += kBT) {
    const double* p = V + 3 * (long long)T[3 * (long long)span[e / 3] + e % 3];
    double o[3];
    proj_point(ax, p, o);
    for (int k = 0; k < 3; ++k) {
      P[3 * e + k] = o[k];
      mn[k] = vi_min(mn[k], VI{o[k], e});
      mx[k] = vi_max(mx[k], VI{o[k], e});
    }
  }
  for (int k = 0; k < 3; ++k) {
    mn[k] = block_min_vi(mn[k], sh, k);
    mx[k] = block_max_vi(mx[k], sh, 3 + k);
  }
  {
    const double mnv[3] = {mn[0].v, mn[1].v, mn[2].v}, mxv[3] = {mx[0].v, mx[1].v, mx[2].v};
    obb_from_extremes(mnv, mxv, nd);
  }
  const double minz = mn[2].v, maxz = mx[2].v;
  const double r = 0.5 * (maxz - minz);
  const double radsqr = r * r;
  const double cz = 0.5 * (maxz + minz);
  double ext[2][2];
  for (int c = 0; c < 2; ++c) {
    const int imin = mn[c].i, imax = mx[c].i;
    const double lo0 = P[3 * imin + c] + rss_cap(P[3 * imin + 2], cz, radsqr);
    const double hi0 = P[3 * imax + c] - rss_cap(P[3 * imax + 2], cz, radsqr);
    VI lo{lo0, -1}, hi{hi0, -1};
    for (int e = tid; e < np; e += kBT) {
      const double pc = P[3 * e + c];
      if (pc < lo.v) lo = vi_min(lo, VI{pc + rss_cap(P[3 * e + 2], cz, radsqr), e});
      if (pc > hi.v) hi = vi_max(hi, VI{pc - rss_cap(P[3 * e + 2], cz, radsqr), e});
    }
    ext[c][0] = block_min_vi(lo, sh, 0).v;
    ext[c][1] = block_max_vi(hi, sh, 1).v;
  }
  // corners, in point order, over the points outside the rectangle in x and in y
  if (tid == 0) {
    sh.rect[0] = ext[0][0];
    sh.rect[1] = ext[0][1];
    sh.rect[2] = ext[1][0];
    sh.rect[3] = ext[1][1];
  }
  {
    const double x0 = ext[0][0], x1 = ext[0][1], y0 = ext[1][0], y1 = ext[1][1];
    for (int base = 0; base < np; base += kBT) {
      const int e = base + tid;
      bool fl[3] = {false, false, false};
      if (e < np) {
        const double X = P[3 * e], Y = P[3 * e + 1];
        fl[0] = (X > x1 || X < x0) && (Y > y1 || Y < y0);
      }
      int before[3], total[3];
      block_counts3(fl, before, total, sh);
      if (fl[0]) sh.cand[before[0]] = e;
      __syncthreads();
      // the candidates in order: every one is evaluated against the current rectangle at
      // once; the first that moves it is applied (by thread 0) and the ones after it are
      // evaluated again; the ones before it saw the rectangle the serial loop would show
      int from = 0;
      while (from < total[0]) {
        if (tid == 0) sh.ncand = INT_MAX;
        __syncthreads();
        const int q = from + tid;
        if (q < total[0]) {
          const int ee = sh.cand[q];
          double a0 = sh.rect[0], a1 = sh.rect[1], a2 = sh.rect[2], a3 = sh.rect[3];
          if (rss_corner<false>(P[3 * ee], P[3 * ee + 1], P[3 * ee + 2], cz, radsqr, a0, a1, a2, a3))
            atomicMin(&sh.ncand, q);
        }
        __syncthreads();
        const int first = sh.ncand;
        if (first == INT_MAX) break;
        if (tid == 0) {
          const int ee = sh.cand[first];
          double a0 = sh.rect[0], a1 = sh.rect[1], a2 = sh.rect[2], a3 = sh.rect[3];
          rss_corner<true>(P[3 * ee], P[3 * ee + 1], P[3 * ee + 2], cz, radsqr, a0, a1, a2, a3);
          sh.rect[0] = a0;
          sh.rect[1] = a1;
          sh.rect[2] = a2;
          sh.rect[3] = a3;
        }
        __syncthreads();
        from = first + 1;
      }
      __syncthreads();
    }
  }
  if (tid == 0) {
    RssD rs;
    rss_write(ax, sh.rect[0], sh.rect[1], sh.rect[2], sh.rect[3], cz, r, nd.axis, rs);
    rss[tk.id] = rs;
  }
  // (3) mean split and the Lomuto partition (as k_bvh_warp, block-wide counts)
  const double split = ((s[0] * ax[0][0] + s[1] * ax[0][1]) + s[2] * ax[0][2]) / (3 * n);
  int32_t* B = Bbuf + 2 * (long long)f;
  uint32_t* out = spanbuf + f;
  int nR = 0, nRot = 0, nL = 0;
  for (int base = 0; base < n; base += kBT) {
    const int i = base + tid;
    bool isL = false;
    uint32_t pv = 0;
    if (i < n) {
      pv = span[i];
      const double* c = C3 + 3 * (long long)pv;
      isL = !(dotd3(ax[0], c[0], c[1], c[2]) > split);
    }
    const bool isR = (i < n) && !isL;
    // rights before i first: a left rotates only when some right precedes it
    bool fl[3] = {isR, false, isL};
    int before[3], total[3];
    block_counts3(fl, before, total, sh);
    const int rb = nR + before[0];
    const bool rot = isL && rb > 0;
    bool fr[3] = {rot, false, false};
    int before2[3], total2[3];
    block_counts3(fr, before2, total2, sh);
    const int ob = nRot + before2[0];
    if (isL) out[nL + before[2]] = pv;
    if (isR) B[rb + ob] = (int32_t)pv;
    if (rot) B[rb + ob] = -(ob + 1);
    nR += total[0];
    nRot += total2[0];
    nL += total[2];
  }
  __syncthreads();
  const int lenB = nR + nRot;
  for (int base = 0; base < lenB; base += kBT) {
    const int k = base + tid;
    int32_t v = (k < lenB) ? B[k] : 0;
    if (k < lenB && v < 0) {
      const int j = -v - 1;
      if (j < base) v = B[j];
    }
    sh.B[tid] = v;
    __syncthreads();
    for (int pass = 0; pass < kBT; ++pass) {
      const bool pending = (k < lenB) && (v < 0);
      if (!__syncthreads_or(pending)) break;
      if (pending) {
        const int32_t t = sh.B[-v - 1 - base];
        if (t >= 0) v = t;
      }
      __syncthreads();
      sh.B[tid] = v;
      __syncthreads();
    }
    if (k < lenB) B[k] = v;
    __syncthreads();
  }
  for (int t = tid; t < nR; t += kBT) out[nL + t] = (uint32_t)B[nRot + t];
  __syncthreads();
  for (int t = tid; t < n; t += kBT) prim[f + t] = out[t];
  int left = nL;
  if (left == 0 || left == n) left = n / 2;
  if (tid == 0) {
    nd.child = child_base(tk);
    nd.pad = 0;
    nodes[tk.id] = nd;
    left_out[ti] = left;
  }
}

// next level: the two children of every internal task, in task order
__global__ void k_bvh_children(const BuildTask* tasks, int ntasks, const int32_t* left_out, const int64_t* rank,
                               BuildTask* next, int32_t* level_ids, int* maxcount) {
  const int ti = blockIdx.x * blockDim.x + threadIdx.x;
  if (ti >= ntasks) return;
  const BuildTask tk = tasks[ti];
  if (tk.count < 2) return;
  const int q = (int)rank[ti];
  const int L = left_out[ti];
  const int cb = child_base(tk);
  atomicMax(maxcount, max(L, tk.count - L));
  next[2 * q] = BuildTask{cb, tk.first, L, tk.pre + 1, tk.lb};
  next[2 * q + 1] = BuildTask{cb + 1, tk.first + L, tk.count - L, tk.pre + 2 * L, tk.lb + L};
  level_ids[q] = tk.id;
}

__global__ void k_bvh_internal_flags(const BuildTask* tasks, int ntasks, int32_t* flags) {
  const int ti = blockIdx.x * blockDim.x + threadIdx.x;
  if (ti < ntasks) flags[ti] = tasks[ti].count >= 2 ? 1 : 0;
}

__global__ void k_bvh_iota(uint32_t* prim, int nt) {
  const int stride = gridDim.x * blockDim.x;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nt; i += stride) prim[i] = (uint32_t)i;
}

__global__ void k_bvh_root(BuildTask* t, int nt) { *t = BuildTask{0, 0, nt, 0, 0}; }

// grid for a grid-stride kernel
unsigned grid_of(long long n, int block) {
  long long g = (n + block - 1) / block;
  return (unsigned)std::max<long long>(1, std::min<long long>(g, 152LL * 64));
}
// grid covering n threads (kernels with one thread per item)
unsigned blocks_for(long long n, int block) { return (unsigned)std::max<long long>(1, (n + block - 1) / block); }

}  // namespace

cudaError_t build_bvh_device(const double* V, const int32_t* T, int nt, NodeD* nodes, RssD* rss,
                             std::vector<int64_t>& level_off, int32_t* level_ids, int* max_depth, cudaStream_t s) {
  if (nt <= 0) return cudaErrorInvalidValue;
  const size_t n = (size_t)nt;
  void* buf[9] = {nullptr};
  const size_t bytes[9] = {72 * n, 24 * n, 4 * n, 72 * n, 8 * n, 4 * n, sizeof(BuildTask) * 2 * n, 4 * n + 16,
                           8 * (n + 1) + 8 * (2 * ((n + 4095) / 4096) + 4)};
  cudaError_t e = cudaSuccess;
  for (int k = 0; k < 9 && e == cudaSuccess; ++k) e = cudaMalloc(&buf[k], std::max<size_t>(bytes[k], 16));
  if (e == cudaSuccess) {
    double* T9 = (double*)buf[0];
    double* C3 = (double*)buf[1];
    uint32_t* prim = (uint32_t*)buf[2];
    double* P = (double*)buf[3];
    int32_t* B = (int32_t*)buf[4];
    uint32_t* spanbuf = (uint32_t*)buf[5];
    BuildTask* tasks = (BuildTask*)buf[6];
    BuildTask* next = tasks + n;
    int32_t* left_out = (int32_t*)buf[7];
    int64_t* rank = (int64_t*)buf[8];
    int64_t* scan_tmp = rank + (n + 1);
    int32_t* flags = (int32_t*)spanbuf;  // free between the partition and the next level
    int* maxcount = (int*)(left_out + n);  // largest task of the next level
    k_bvh_tri_terms<<<grid_of(nt, 128), 128, 0, s>>>(V, T, nt, T9, C3);
    k_bvh_iota<<<grid_of(nt, 256), 256, 0, s>>>(prim, nt);
    k_bvh_root<<<1, 1, 0, s>>>(tasks, nt);
    g_kernel_launches += 3;
    level_off.assign(1, 0);
    int ntasks = 1, depth = 0;
    int64_t level_max_count = nt;  // the largest task of the current level
    static bool attr_set = false;
    if (!attr_set) {
      e = cudaFuncSetAttribute(k_bvh_block, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(BlockScratch));
      attr_set = (e == cudaSuccess);
    }
    int64_t nlevel_ids = 0;
    while (ntasks > 0 && e == cudaSuccess) {
      k_bvh_small<<<blocks_for(ntasks, 128), 128, 0, s>>>(tasks, ntasks, V, T, T9, C3, prim, nodes, rss, left_out);
      k_bvh_warp<<<(unsigned)((ntasks + kWarpsPerBlock - 1) / kWarpsPerBlock), 32 * kWarpsPerBlock, 0, s>>>(
          tasks, ntasks, V, T, T9, C3, prim, nodes, rss, left_out, P, B, spanbuf);
      if (level_max_count > kBlockTask) {
        k_bvh_block<<<(unsigned)ntasks, kBT, sizeof(BlockScratch), s>>>(tasks, ntasks, V, T, T9, C3, prim, nodes, rss,
                                                                      left_out, P, B, spanbuf);
        ++g_kernel_launches;
      }
      k_bvh_internal_flags<<<blocks_for(ntasks, 256), 256, 0, s>>>(tasks, ntasks, flags);
      g_kernel_launches += 3;
      if ((e = launch_exclusive_scan(flags, ntasks, rank, scan_tmp, s)) != cudaSuccess) break;
      if ((e = cudaMemsetAsync(maxcount, 0, sizeof(int), s)) != cudaSuccess) break;
      k_bvh_children<<<blocks_for(ntasks, 128), 128, 0, s>>>(tasks, ntasks, left_out, rank, next,
                                                           level_ids + nlevel_ids, maxcount);
      ++g_kernel_launches;
      int64_t ninternal = 0;
      int hmax = 0;
      if ((e = cudaMemcpyAsync(&ninternal, rank + ntasks, 8, cudaMemcpyDeviceToHost, s)) != cudaSuccess) break;
      if ((e = cudaMemcpyAsync(&hmax, maxcount, sizeof(int), cudaMemcpyDeviceToHost, s)) != cudaSuccess) break;
      if ((e = cudaStreamSynchronize(s)) != cudaSuccess) break;
      level_max_count = hmax;
      if (ninternal > 0) {
        nlevel_ids += ninternal;
        level_off.push_back(nlevel_ids);
        std::swap(tasks, next);
        next = tasks == (BuildTask*)buf[6] ? tasks + n : (BuildTask*)buf[6];
        ++depth;
      }
      ntasks = (int)(2 * ninternal);
      if ((e = cudaGetLastError()) != cudaSuccess) break;
    }
    *max_depth = depth;
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  }
  for (int k = 0; k < 9; ++k)
    if (buf[k]) cudaFree(buf[k]);
  return e;
}

}  // namespace fclgpu
