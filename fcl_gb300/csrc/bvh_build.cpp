// Host construction of BVHModel<OBBRSS<double>> and packing of its device layouts.
//
// The tree must be bit-identical to FCL's, because every traversal decision on the
// device depends on it.  The build therefore follows FCL 0.7.0 operation by
// operation: top-down (geometry/bvh/BVH_model-inl.h:833-938), fit by
// BVFitter<OBBRSS> (geometry/bvh/detail/BV_fitter-inl.h:448-478) = covariance of
// the triangle vertices (math/geometry-inl.h:1335-1421), cyclic Jacobi eigen
// decomposition (eigen_old, :477-558), axes ordered by eigenvalue (axisFromEigen,
// :563-598), OBB extent (getExtentAndCenter_mesh) and RSS fit
// (getRadiusAndOriginAndRectangleSize, :709-990); MEAN split of the triangle
// centroids along the first axis (geometry/bvh/detail/BV_splitter-inl.h:422-436,
// 492-500, 540-546) with FCL's in-place partition and n/2 fallback; children
// allocated as the pair (num_bvs, num_bvs+1) in depth-first order.
//
// Arithmetic conventions (Eigen is not available to pin them): 3-term dot products
// and matrix products sum left to right, ((x0 + x1) + x2); no fused multiply-add
// (this file is compiled with -ffp-contract=off).
#include <algorithm>
#include <atomic>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <limits>
#include <mutex>
#include <thread>
#include <vector>

#include "bvh_build.h"

namespace fclgpu {

namespace {

struct D3 {
  double x, y, z;
};
inline D3 d3(double a, double b, double c) { return D3{a, b, c}; }
inline double dotd(const D3& a, const D3& b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
inline D3 crossd(const D3& a, const D3& b) {
  return d3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}

// Column k of a row-major 3x3.
inline D3 colk(const double* m, int k) { return d3(m[k], m[3 + k], m[6 + k]); }

class Builder {
 public:
  Builder(const double* verts, int64_t nv, const int32_t* tris, int64_t nt) : V_(verts), T_(tris), nt_((int)nt) {
    (void)nv;
  }

  // Node ids are FCL's: a node's children are the pair (num_bvs, num_bvs + 1) taken when
  // the node is split, in depth-first order, so a node split with `base` as num_bvs
  // gives its left subtree base + 2 and its right subtree base + 2 * (left primitives)
  // (a subtree of k primitives takes 2 (k - 1) ids).  Subtrees are therefore
  // independent: large meshes split their upper levels into tasks run on several host
  // threads, with the same ids, the same partitions and so the same tree.
  void run(HostBVH& out) {
    const int n_nodes = 2 * nt_ - 1;
    out.nodes.assign(n_nodes, NodeD());
    out.rss.assign(n_nodes, RssD());
    prim_.resize(nt_);
    for (int i = 0; i < nt_; ++i) prim_[i] = (uint32_t)i;
    const unsigned hw = std::thread::hardware_concurrency();
    const int workers = nt_ >= kParallelMin ? (int)std::min(16u, std::max(1u, hw)) : 1;
    if (workers <= 1) {
      std::vector<double> proj;
      out.max_depth = subtree(Task{0, 0, nt_, 0, 1}, out, proj);
      return;
    }
    // shared task stack: tasks of at least kTaskMin primitives are split here and
    // their children queued; smaller ones run as whole subtrees
    std::mutex mu;
    std::condition_variable cv;
    std::vector<Task> tasks{Task{0, 0, nt_, 0, 1}};
    int outstanding = 1, max_depth = 0;
    auto worker = [&]() {
      std::vector<double> proj;
      int local_depth = 0;
      for (;;) {
        Task tk;
        {
          std::unique_lock<std::mutex> lk(mu);
          cv.wait(lk, [&] { return !tasks.empty() || outstanding == 0; });
          if (tasks.empty()) break;
          tk = tasks.back();
          tasks.pop_back();
        }
        Task kids[2];
        int nkids = 0;
        if (tk.count >= kTaskMin) {
          local_depth = std::max(local_depth, node(tk, out, proj, kids, nkids));
        } else {
          local_depth = std::max(local_depth, subtree(tk, out, proj));
        }
        {
          std::lock_guard<std::mutex> lk(mu);
          for (int k = 0; k < nkids; ++k) tasks.push_back(kids[k]);
          outstanding += nkids - 1;
        }
        cv.notify_all();
      }
      std::lock_guard<std::mutex> lk(mu);
      max_depth = std::max(max_depth, local_depth);
    };
    std::vector<std::thread> pool;
    for (int t = 0; t < workers; ++t) pool.emplace_back(worker);
    for (auto& th : pool) th.join();
    out.max_depth = max_depth;
  }

 private:
  static constexpr int kParallelMin = 16384;  // meshes below this build on one thread
  static constexpr int kTaskMin = 4096;       // tasks this large are split into two tasks

  struct Task {
    int id, first, count, depth;
    int base;  // FCL's num_bvs when this node is split
  };

  // Fits node tk and, unless it is a leaf, splits its primitives (FCL's mean split with
  // its in-place partition) and returns its two children as tasks (kids, nkids).
  // Returns the node's depth.
  int node(const Task& tk, HostBVH& out, std::vector<double>& proj, Task* kids, int& nkids) {
    nkids = 0;
    NodeD& nd = out.nodes[tk.id];
    RssD& rs = out.rss[tk.id];
    uint32_t* span = prim_.data() + tk.first;
    fit(span, tk.count, nd, rs, proj);
    for (int k = 0; k < 9; ++k) rs.axis[k] = nd.axis[k];  // BVFitter<OBBRSS>: rss.axis = obb.axis
    if (tk.count == 1) {
      nd.child = -((int)span[0] + 1);
      return tk.depth;
    }
    const D3 axis0 = colk(nd.axis, 0);
    const double split = mean_split_value(span, tk.count, axis0);
    nd.child = tk.base;
    int left = 0;
    for (int i = 0; i < tk.count; ++i) {
      const int32_t* t = T_ + 3 * (int64_t)span[i];
      const double* p1 = V_ + 3 * (int64_t)t[0];
      const double* p2 = V_ + 3 * (int64_t)t[1];
      const double* p3 = V_ + 3 * (int64_t)t[2];
      D3 c = d3(((p1[0] + p2[0]) + p3[0]) / 3.0, ((p1[1] + p2[1]) + p3[1]) / 3.0,
                ((p1[2] + p2[2]) + p3[2]) / 3.0);
      if (!(dotd(axis0, c) > split)) {
        std::swap(span[i], span[left]);
        ++left;
      }
    }
    if (left == 0 || left == tk.count) left = tk.count / 2;
    // right first: a LIFO runs the left subtree first, as FCL's recursion does
    kids[0] = Task{nd.child + 1, tk.first + left, tk.count - left, tk.depth + 1, tk.base + 2 * left};
    kids[1] = Task{nd.child, tk.first, left, tk.depth + 1, tk.base + 2};
    nkids = 2;
    return tk.depth;
  }

  // The whole subtree of tk on this thread; returns its largest depth.
  int subtree(const Task& root, HostBVH& out, std::vector<double>& proj) {
    int max_depth = 0;
    std::vector<Task> todo{root};
    while (!todo.empty()) {
      const Task tk = todo.back();
      todo.pop_back();
      Task kids[2];
      int nkids = 0;
      max_depth = std::max(max_depth, node(tk, out, proj, kids, nkids));
      for (int k = 0; k < nkids; ++k) todo.push_back(kids[k]);
    }
    return max_depth;
  }

  const double* vtx(int32_t id) const { return V_ + 3 * (int64_t)id; }

  double mean_split_value(const uint32_t* span, int n, const D3& sv) const {
    double c0 = 0.0, c1 = 0.0, c2 = 0.0;
    for (int i = 0; i < n; ++i) {
      const int32_t* t = T_ + 3 * (int64_t)span[i];
      const double *p1 = vtx(t[0]), *p2 = vtx(t[1]), *p3 = vtx(t[2]);
      c0 += (p1[0] + p2[0] + p3[0]);
      c1 += (p1[1] + p2[1] + p3[1]);
      c2 += (p1[2] + p2[2] + p3[2]);
    }
    return (c0 * sv.x + c1 * sv.y + c2 * sv.z) / (3 * n);
  }

  void fit(const uint32_t* span, int n, NodeD& nd, RssD& rs, std::vector<double>& proj_) {
    // --- covariance of the 3n vertices
    double s1x = 0, s1y = 0, s1z = 0;
    double sxx = 0, syy = 0, szz = 0, sxy = 0, sxz = 0, syz = 0;
    for (int i = 0; i < n; ++i) {
      const int32_t* t = T_ + 3 * (int64_t)span[i];
      const double *a = vtx(t[0]), *b = vtx(t[1]), *c = vtx(t[2]);
      s1x += (a[0] + b[0]) + c[0];
      s1y += (a[1] + b[1]) + c[1];
      s1z += (a[2] + b[2]) + c[2];
      sxx += (a[0] * a[0] + b[0] * b[0] + c[0] * c[0]);
      syy += (a[1] * a[1] + b[1] * b[1] + c[1] * c[1]);
      szz += (a[2] * a[2] + b[2] * b[2] + c[2] * c[2]);
      sxy += (a[0] * a[1] + b[0] * b[1] + c[0] * c[1]);
      sxz += (a[0] * a[2] + b[0] * b[2] + c[0] * c[2]);
      syz += (a[1] * a[2] + b[1] * b[2] + c[1] * c[2]);
    }
    const int np = 3 * n;
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

    double evals[3] = {0, 0, 0};
    double evecs[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};  // evecs[k] = k-th eigenvector
    jacobi(C, evals, evecs);

    // --- axes: largest, middle, then their cross product
    int lo, mid, hi;
    if (evals[0] > evals[1]) { hi = 0; lo = 1; }
    else { lo = 0; hi = 1; }
    if (evals[2] < evals[lo]) { mid = lo; lo = 2; }
    else if (evals[2] > evals[hi]) { mid = hi; hi = 2; }
    else { mid = 2; }
    D3 a0 = d3(evecs[hi][0], evecs[hi][1], evecs[hi][2]);
    D3 a1 = d3(evecs[mid][0], evecs[mid][1], evecs[mid][2]);
    D3 a2 = crossd(a0, a1);
    const D3 ax[3] = {a0, a1, a2};
    for (int r = 0; r < 3; ++r) {
      nd.axis[3 * r + 0] = r == 0 ? a0.x : (r == 1 ? a0.y : a0.z);
      nd.axis[3 * r + 1] = r == 0 ? a1.x : (r == 1 ? a1.y : a1.z);
      nd.axis[3 * r + 2] = r == 0 ? a2.x : (r == 1 ? a2.y : a2.z);
    }

    // --- projections of every vertex occurrence (shared by the OBB and RSS fits)
    proj_.resize(3 * (size_t)np);
    double* P = proj_.data();
    for (int i = 0; i < n; ++i) {
      const int32_t* t = T_ + 3 * (int64_t)span[i];
      for (int j = 0; j < 3; ++j) {
        const double* p = vtx(t[j]);
        const D3 q = d3(p[0], p[1], p[2]);
        double* o = P + 3 * (3 * (size_t)i + j);
        o[0] = dotd(ax[0], q);
        o[1] = dotd(ax[1], q);
        o[2] = dotd(ax[2], q);
      }
    }

    // --- OBB: extent and centre (getExtentAndCenter_mesh)
    const double big = std::numeric_limits<double>::max();
    double mn[3] = {big, big, big}, mx[3] = {-big, -big, -big};
    for (int i = 0; i < np; ++i)
      for (int k = 0; k < 3; ++k) {
        const double v = P[3 * i + k];
        if (v > mx[k]) mx[k] = v;
        if (v < mn[k]) mn[k] = v;
      }
    const double o0 = (mx[0] + mn[0]) / 2, o1 = (mx[1] + mn[1]) / 2, o2 = (mx[2] + mn[2]) / 2;
    for (int r = 0; r < 3; ++r)
      nd.To[r] = (nd.axis[3 * r] * o0 + nd.axis[3 * r + 1] * o1) + nd.axis[3 * r + 2] * o2;
    nd.ext[0] = (mx[0] - mn[0]) / 2;
    nd.ext[1] = (mx[1] - mn[1]) / 2;
    nd.ext[2] = (mx[2] - mn[2]) / 2;

    rss_fit(P, np, ax, rs);
  }

  // Cyclic Jacobi rotation as in FCL's eigen_old; evecs[k] receives the k-th
  // eigenvector (column k of the accumulated rotation).
  static void jacobi(const double C[3][3], double evals[3], double evecs[3][3]) {
    double R[3][3];
    std::memcpy(R, C, sizeof(R));
    double v[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
    double b[3], d[3], z[3];
    for (int p = 0; p < 3; ++p) {
      b[p] = d[p] = R[p][p];
      z[p] = 0;
    }
    for (int sweep = 0; sweep < 50; ++sweep) {
      double sm = 0;
      for (int p = 0; p < 3; ++p)
        for (int q = p + 1; q < 3; ++q) sm += std::abs(R[p][q]);
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
          const double g = 100.0 * std::abs(R[p][q]);
          if (sweep > 3 && std::abs(d[p]) + g == std::abs(d[p]) && std::abs(d[q]) + g == std::abs(d[q])) {
            R[p][q] = 0.0;
          } else if (std::abs(R[p][q]) > tresh) {
            double h = d[q] - d[p];
            double t;
            if (std::abs(h) + g == std::abs(h)) {
              t = (R[p][q]) / h;
            } else {
              const double theta = 0.5 * h / (R[p][q]);
              t = 1.0 / (std::abs(theta) + std::sqrt(1.0 + theta * theta));
              if (theta < 0.0) t = -t;
            }
            const double c = 1.0 / std::sqrt(1 + t * t);
            const double s = t * c;
            const double tau = s / (1.0 + c);
            h = t * R[p][q];
            z[p] -= h;
            z[q] += h;
            d[p] -= h;
            d[q] += h;
            R[p][q] = 0.0;
            for (int j = 0; j < p; ++j) rot(R[j][p], R[j][q], s, tau);
            for (int j = p + 1; j < q; ++j) rot(R[p][j], R[j][q], s, tau);
            for (int j = q + 1; j < 3; ++j) rot(R[p][j], R[q][j], s, tau);
            for (int j = 0; j < 3; ++j) rot(v[j][p], v[j][q], s, tau);
          }
        }
      }
      for (int p = 0; p < 3; ++p) {
        b[p] += z[p];
        d[p] = b[p];
        z[p] = 0.0;
      }
    }
    // no convergence in 50 sweeps: FCL leaves its outputs unchanged; keep identity
  }
  static inline void rot(double& x, double& y, double s, double tau) {
    const double g = x, h = y;
    x = g - s * (h + g * tau);
    y = h + s * (g - h * tau);
  }

  // RSS of the projected points P (getRadiusAndOriginAndRectangleSize).
  static void rss_fit(const double* P, int np, const D3 ax[3], RssD& rs) {
    auto px = [&](int i) { return P[3 * i + 0]; };
    auto py = [&](int i) { return P[3 * i + 1]; };
    auto pz = [&](int i) { return P[3 * i + 2]; };
    double minz = pz(0), maxz = pz(0);
    for (int i = 1; i < np; ++i) {
      const double zv = pz(i);
      if (zv < minz) minz = zv;
      else if (zv > maxz) maxz = zv;
    }
    const double r = 0.5 * (maxz - minz);
    const double radsqr = r * r;
    const double cz = 0.5 * (maxz + minz);
    auto cap = [&](int i) { const double dz = pz(i) - cz; return std::sqrt(std::max<double>(radsqr - dz * dz, 0)); };

    // x extent of the rectangle
    int imin = 0, imax = 0;
    double vmin = px(0), vmax = px(0);
    for (int i = 1; i < np; ++i) {
      const double xv = px(i);
      if (xv < vmin) { imin = i; vmin = xv; }
      else if (xv > vmax) { imax = i; vmax = xv; }
    }
    double minx = px(imin) + cap(imin);
    double maxx = px(imax) - cap(imax);
    for (int i = 0; i < np; ++i)
      if (px(i) < minx) { const double x = px(i) + cap(i); if (x < minx) minx = x; }
    for (int i = 0; i < np; ++i)
      if (px(i) > maxx) { const double x = px(i) - cap(i); if (x > maxx) maxx = x; }

    // y extent
    imin = imax = 0;
    vmin = vmax = py(0);
    for (int i = 1; i < np; ++i) {
      const double yv = py(i);
      if (yv < vmin) { imin = i; vmin = yv; }
      else if (yv > vmax) { imax = i; vmax = yv; }
    }
    double miny = py(imin) + cap(imin);
    double maxy = py(imax) - cap(imax);
    for (int i = 0; i < np; ++i)
      if (py(i) < miny) { const double y = py(i) + cap(i); if (y < miny) miny = y; }
    for (int i = 0; i < np; ++i)
      if (py(i) > maxy) { const double y = py(i) - cap(i); if (y > maxy) maxy = y; }

    // corners
    const double a = std::sqrt(0.5);
    for (int i = 0; i < np; ++i) {
      const double X = px(i), Y = py(i), Z = pz(i);
      if (X > maxx) {
        if (Y > maxy) {
          const double dx = X - maxx, dy = Y - maxy;
          double u = dx * a + dy * a;
          const double t = (a * u - dx) * (a * u - dx) + (a * u - dy) * (a * u - dy) + (cz - Z) * (cz - Z);
          u = u - std::sqrt(std::max<double>(radsqr - t, 0));
          if (u > 0) { maxx += u * a; maxy += u * a; }
        } else if (Y < miny) {
          const double dx = X - maxx, dy = Y - miny;
          double u = dx * a - dy * a;
          const double t = (a * u - dx) * (a * u - dx) + (-a * u - dy) * (-a * u - dy) + (cz - Z) * (cz - Z);
          u = u - std::sqrt(std::max<double>(radsqr - t, 0));
          if (u > 0) { maxx += u * a; miny -= u * a; }
        }
      } else if (X < minx) {
        if (Y > maxy) {
          const double dx = X - minx, dy = Y - maxy;
          double u = dy * a - dx * a;
          const double t = (-a * u - dx) * (-a * u - dx) + (a * u - dy) * (a * u - dy) + (cz - Z) * (cz - Z);
          u = u - std::sqrt(std::max<double>(radsqr - t, 0));
          if (u > 0) { minx -= u * a; maxy += u * a; }
        } else if (Y < miny) {
          const double dx = X - minx, dy = Y - miny;
          double u = -dx * a - dy * a;
          const double t = (-a * u - dx) * (-a * u - dx) + (-a * u - dy) * (-a * u - dy) + (cz - Z) * (cz - Z);
          u = u - std::sqrt(std::max<double>(radsqr - t, 0));
          if (u > 0) { minx -= u * a; miny -= u * a; }
        }
      }
    }
    const double ox[3] = {ax[0].x * minx, ax[0].y * minx, ax[0].z * minx};
    const double oy[3] = {ax[1].x * miny, ax[1].y * miny, ax[1].z * miny};
    const double oz[3] = {ax[2].x * cz, ax[2].y * cz, ax[2].z * cz};
    for (int k = 0; k < 3; ++k) rs.To[k] = (ox[k] + oy[k]) + oz[k];
    rs.l[0] = maxx - minx;
    if (rs.l[0] < 0) rs.l[0] = 0;
    rs.l[1] = maxy - miny;
    if (rs.l[1] < 0) rs.l[1] = 0;
    rs.r = r;
  }

  const double* V_;
  const int32_t* T_;
  int nt_;
  std::vector<uint32_t> prim_;
};

inline float f32(double x) { return (float)x; }

}  // namespace

int build_obbrss(const double* verts, int64_t nv, const int32_t* tris, int64_t nt, HostBVH& out) {
  if (nt <= 0 || nv <= 0) return -1;
  Builder b(verts, nv, tris, nt);
  b.run(out);
  return 0;
}

void pack_fp32(const double* verts, const int32_t* tris, int64_t nt, const HostBVH& bvh, PackedF32& pk) {
  const size_t nn = bvh.nodes.size();
  pk.nodes32.resize(16 * nn);
  pk.size64.resize(nn);
  pk.rss32.resize(20 * nn);
  pk.cmax = 0.0;
  pk.rmax = 0.0;
  for (size_t i = 0; i < nn; ++i) {
    const NodeD& n = bvh.nodes[i];
    const RssD& r = bvh.rss[i];
    float* o = &pk.nodes32[16 * i];
    for (int k = 0; k < 3; ++k) {
      o[4 * k + 0] = f32(n.axis[0 + k]);
      o[4 * k + 1] = f32(n.axis[3 + k]);
      o[4 * k + 2] = f32(n.axis[6 + k]);
      o[4 * k + 3] = f32(n.To[k]);
    }
    o[12] = f32(n.ext[0]);
    o[13] = f32(n.ext[1]);
    o[14] = f32(n.ext[2]);
    std::memcpy(&o[15], &n.child, 4);
    pk.size64[i] = (n.ext[0] * n.ext[0] + n.ext[1] * n.ext[1]) + n.ext[2] * n.ext[2];
    float* q = &pk.rss32[20 * i];
    q[0] = f32(r.To[0]);
    q[1] = f32(r.To[1]);
    q[2] = f32(r.To[2]);
    q[3] = f32(r.r);
    q[4] = f32(r.l[0]);
    q[5] = f32(r.l[1]);
    q[6] = 0.f;
    q[7] = 0.f;
    for (int k = 0; k < 3; ++k) {
      q[8 + 4 * k + 0] = f32(r.axis[0 + k]);
      q[8 + 4 * k + 1] = f32(r.axis[3 + k]);
      q[8 + 4 * k + 2] = f32(r.axis[6 + k]);
      q[8 + 4 * k + 3] = 0.f;
    }
    pk.cmax = std::max(pk.cmax, std::sqrt((n.To[0] * n.To[0] + n.To[1] * n.To[1]) + n.To[2] * n.To[2]));
    pk.rmax = std::max(pk.rmax, std::sqrt((r.To[0] * r.To[0] + r.To[1] * r.To[1]) + r.To[2] * r.To[2]));
  }
  pk.tri32.resize(12 * (size_t)nt);
  for (int64_t t = 0; t < nt; ++t) {
    const double* p1 = verts + 3 * (int64_t)tris[3 * t + 0];
    const double* p2 = verts + 3 * (int64_t)tris[3 * t + 1];
    const double* p3 = verts + 3 * (int64_t)tris[3 * t + 2];
    float hi[3], lo[3], d2[3], d3v[3];
    for (int k = 0; k < 3; ++k) {
      hi[k] = f32(p1[k]);
      lo[k] = f32(p1[k] - (double)hi[k]);
      d2[k] = f32(p2[k] - p1[k]);
      d3v[k] = f32(p3[k] - p1[k]);
    }
    float* o = &pk.tri32[12 * t];
    o[0] = hi[0]; o[1] = hi[1]; o[2] = hi[2]; o[3] = lo[0];
    o[4] = lo[1]; o[5] = lo[2]; o[6] = d2[0]; o[7] = d2[1];
    o[8] = d2[2]; o[9] = d3v[0]; o[10] = d3v[1]; o[11] = d3v[2];
  }
}

}  // namespace fclgpu
