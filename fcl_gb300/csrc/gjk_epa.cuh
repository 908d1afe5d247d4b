// Device GJK/EPA for convex shape pairs (FCL's own solver, GST_INDEP), FP64.
//
// Follows convexity_based_algorithm/gjk-inl.h:81-298, epa-inl.h:54-399,
// minkowski_diff-inl.h:65-265 and math/detail/project-inl.h:183-306 operation by
// operation.  Pointers of the reference become small indices: simplex vertices live
// in one array (slots 0-3 = GJK's store, 4.. = EPA's store), faces in a fixed pool
// with the same intrusive hull/stock lists (same insertion order, so findBest breaks
// ties identically), and EPA's recursive horizon expansion runs on an explicit frame
// stack with the same short-circuit order.
#pragma once
#include "geom.cuh"

namespace fclgpu {

// GJKSolver_indep's parameters (narrowphase/detail/gjk_solver_indep.h; defaults
// gjk_solver_indep-inl.h:1039-1049): GJK and EPA tolerances and iteration caps.  The
// defaults are the solver's own; fcl::collide sets both tolerances to
// CollisionRequest::gjk_tolerance and fcl::distance the GJK tolerance to
// DistanceRequest::distance_tolerance (collision-inl.h:164-170, distance-inl.h:211-215).
struct SolverParams {
  double gjk_tolerance;
  double epa_tolerance;
  int32_t gjk_max_iterations;
  int32_t epa_max_iterations;
};
constexpr double kSolverDefaultTol = 2.0097183471152322e-14;  // std::pow(eps, 7/8) (math/constants.h:164-167)
#define FCLG_SOLVER_DEFAULTS {kSolverDefaultTol, kSolverDefaultTol, 128, 255}

#if defined(__CUDACC__)
// One copy per translation unit that launches solver kernels; each launch refreshes it
// from the process-wide values (upload_solver_params).
static __device__ SolverParams g_dev_solver_params = FCLG_SOLVER_DEFAULTS;
// Host: the values set by fclgpu_set_gjk_solver_params.
SolverParams current_solver_params();
static inline cudaError_t upload_solver_params(cudaStream_t s) {
  const SolverParams p = current_solver_params();
  return cudaMemcpyToSymbolAsync(g_dev_solver_params, &p, sizeof(p), 0, cudaMemcpyHostToDevice, s);
}
#endif

FCLG_HD SolverParams solver_params() {
#if defined(__CUDA_ARCH__)
  return g_dev_solver_params;
#else
  return SolverParams FCLG_SOLVER_DEFAULTS;  // host builds of the device code use the defaults
#endif
}

enum : int { SHAPE_BOX = 0, SHAPE_SPHERE = 1, SHAPE_CAPSULE = 2, SHAPE_CYLINDER = 3, SHAPE_CONE = 4, SHAPE_CONVEX = 5,
             SHAPE_TRIANGLE = 6 /* TriangleP: 9 doubles at verts + 3 * voff (mesh-shape leaves) */ };

struct DevShape {
  int type;
  int voff;  // convex: first vertex in the vertex pool
  int vcnt;  // convex: number of vertices
  int pad;
  double p[3];  // box: side; sphere: radius; capsule/cylinder/cone: radius, lz
};

struct ShapeRef {
  DevShape s;
  const double* verts;  // convex vertex pool (3 doubles per vertex)
};

typedef V3<double> D3v;

FCLG_HD unsigned long long dbits(double x) {
#if defined(__CUDA_ARCH__)
  return (unsigned long long)__double_as_longlong(x);
#else
  unsigned long long u;
  memcpy(&u, &x, 8);
  return u;
#endif
}

// FP32 copy of the convex vertex pool: for a Convex, DevShape.pad is the offset (in
// doubles) from the pool base to an array of float4 (x, y, z, 0), one per pool vertex;
// 0 means no copy.
FCLG_HD const float4* convex_v32(const ShapeRef& sh) {
  return sh.s.pad > 0 ? reinterpret_cast<const float4*>(sh.verts + sh.s.pad) + sh.s.voff : nullptr;
}

FCLG_HD D3v d3neg(const D3v& a) { return v3(-a.x, -a.y, -a.z); }
FCLG_HD D3v d3scale(const D3v& a, double s) { return v3(a.x * s, a.y * s, a.z * s); }
FCLG_HD double d3norm(const D3v& a) { return sqrt(sqnorm(a)); }
FCLG_HD D3v d3normalized(const D3v& a) {
  const double n = d3norm(a);
  return v3(a.x / n, a.y / n, a.z / n);
}
FCLG_HD double d3triple(const D3v& x, const D3v& y, const D3v& z) { return dot(x, cross(y, z)); }

// minkowski_diff-inl.h:65-206 (shape support in its own frame)
FCLG_HD D3v shape_support(const ShapeRef& sh, const D3v& dir) {
  const DevShape& s = sh.s;
  switch (s.type) {
    case SHAPE_BOX:
      return v3((dir.x > 0) ? (s.p[0] / 2) : (-s.p[0] / 2), (dir.y > 0) ? (s.p[1] / 2) : (-s.p[1] / 2),
                (dir.z > 0) ? (s.p[2] / 2) : (-s.p[2] / 2));
    case SHAPE_SPHERE:
      return d3scale(dir, s.p[0]);
    case SHAPE_CAPSULE: {
      const double half_h = s.p[1] * 0.5;
      const D3v v = d3scale(dir, s.p[0]);
      const D3v pos1 = v3(0.0, 0.0, half_h) + v;
      const D3v pos2 = v3(0.0, 0.0, -half_h) + v;
      if (dot(dir, pos1) > dot(dir, pos2)) return pos1;
      return pos2;
    }
    case SHAPE_CONE: {
      double zdist = dir.x * dir.x + dir.y * dir.y;
      double len = zdist + dir.z * dir.z;
      zdist = sqrt(zdist);
      len = sqrt(len);
      const double half_h = s.p[1] * 0.5;
      const double radius = s.p[0];
      const double sin_a = radius / sqrt(radius * radius + 4 * half_h * half_h);
      if (dir.z > len * sin_a) return v3(0.0, 0.0, half_h);
      if (zdist > 0) {
        const double rad = radius / zdist;
        return v3(rad * dir.x, rad * dir.y, -half_h);
      }
      return v3(0.0, 0.0, -half_h);
    }
    case SHAPE_CYLINDER: {
      const double zdist = sqrt(dir.x * dir.x + dir.y * dir.y);
      const double half_h = s.p[1] * 0.5;
      if (zdist == 0.0) return v3(0.0, 0.0, (dir.z > 0) ? half_h : -half_h);
      const double d = s.p[0] / zdist;
      return v3(d * dir.x, d * dir.y, (dir.z > 0) ? half_h : -half_h);
    }
    case SHAPE_CONVEX: {
      // the first vertex of maximal dir.v (strict >), as FCL's linear scan.  With the
      // FP32 copy, FP32 dot products with a rigorous bound E_i = 8u sum_k |dir_k v_k|
      // (u = 2^-24; covers the FP32 and the FP64 rounding) select the candidates,
      // df_i + E_i >= max_j (df_j - E_j); every vertex left out has an FP64 dot below
      // the maximum, so the FP64 scan over the candidates returns the same vertex.
      double maxdot = -1.7976931348623157e308;
      D3v bestv = v3(0.0, 0.0, 0.0);
      const double* V = sh.verts + 3 * (long long)s.voff;
      const float4* V32 = convex_v32(sh);
      if (V32) {
        const float dx = (float)dir.x, dy = (float)dir.y, dz = (float)dir.z;
        const float ax = fabsf(dx), ay = fabsf(dy), az = fabsf(dz);
        float mlo = -3.4e38f;
        for (int i = 0; i < s.vcnt; ++i) {
          const float4 p = V32[i];
          const float df = fmaf(dx, p.x, fmaf(dy, p.y, dz * p.z));
          const float E = fmaf(4.76837158e-07f, fmaf(ax, fabsf(p.x), fmaf(ay, fabsf(p.y), az * fabsf(p.z))), 1e-30f);
          mlo = fmaxf(mlo, df - E);
        }
        for (int i = 0; i < s.vcnt; ++i) {
          const float4 p = V32[i];
          const float df = fmaf(dx, p.x, fmaf(dy, p.y, dz * p.z));
          const float E = fmaf(4.76837158e-07f, fmaf(ax, fabsf(p.x), fmaf(ay, fabsf(p.y), az * fabsf(p.z))), 1e-30f);
          if (!(df + E >= mlo)) continue;
          const D3v vi = v3(V[3 * i], V[3 * i + 1], V[3 * i + 2]);
          const double d = dot(dir, vi);
          if (d > maxdot) {
            bestv = vi;
            maxdot = d;
          }
        }
        return bestv;
      }
      for (int i = 0; i < s.vcnt; ++i) {
        const D3v vi = v3(V[3 * i], V[3 * i + 1], V[3 * i + 2]);
        const double d = dot(dir, vi);
        if (d > maxdot) {
          bestv = vi;
          maxdot = d;
        }
      }
      return bestv;
    }
    case SHAPE_TRIANGLE: {  // TriangleP (minkowski_diff-inl.h:78-97)
      const double* V = sh.verts + 3 * (long long)s.voff;
      const D3v a = v3(V[0], V[1], V[2]), b = v3(V[3], V[4], V[5]), c = v3(V[6], V[7], V[8]);
      const double dota = dot(dir, a), dotb = dot(dir, b), dotc = dot(dir, c);
      if (dota > dotb) return (dotc > dota) ? c : a;
      return (dotc > dotb) ? c : b;
    }
  }
  return v3(0.0, 0.0, 0.0);
}

struct Minkowski {
  ShapeRef s0, s1;
  M3<double> toshape1;  // R2^T R1
  M3<double> R0;        // toshape0 = tf1^-1 tf2
  D3v t0;
  FCLG_HD D3v support0(const D3v& d) const { return shape_support(s0, d); }
  FCLG_HD D3v support1(const D3v& d) const { return mulv(R0, shape_support(s1, mulv(toshape1, d))) + t0; }
  FCLG_HD D3v support(const D3v& d) const { return support0(d) - support1(d3neg(d)); }
  FCLG_HD D3v support(const D3v& d, int index) const { return index ? support1(d) : support0(d); }
};

FCLG_HD void make_minkowski(const ShapeRef& a, const M3<double>& R1, const D3v& t1, const ShapeRef& b,
                            const M3<double>& R2, const D3v& t2, Minkowski& m) {
  m.s0 = a;
  m.s1 = b;
  m.toshape1 = mulT(R2, R1);
  M3<double> Ri;
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) Ri(r, c) = R1(c, r);
  const D3v ti = d3neg(mulv(Ri, t1));
  m.R0 = mul(Ri, R2);
  m.t0 = mulv(Ri, t2) + ti;
}

// ---- simplex projections (project-inl.h) ------------------------------------------
struct ProjRes {
  double par[4];
  double sqd;
  unsigned enc;
};
FCLG_HD void proj_init(ProjRes& r) {
  r.par[0] = r.par[1] = r.par[2] = r.par[3] = 0.0;
  r.sqd = -1;
  r.enc = 0;
}

FCLG_HD ProjRes project_line_origin(const D3v& a, const D3v& b) {
  ProjRes res;
  proj_init(res);
  const D3v d = b - a;
  const double l = sqnorm(d);
  if (l > 0) {
    const double t = -dot(a, d);
    res.par[1] = (t >= l) ? 1 : ((t <= 0) ? 0 : (t / l));
    res.par[0] = 1 - res.par[1];
    if (t >= l) {
      res.sqd = sqnorm(b);
      res.enc = 2;
    } else if (t <= 0) {
      res.sqd = sqnorm(a);
      res.enc = 1;
    } else {
      res.sqd = sqnorm(a + d3scale(d, res.par[1]));
      res.enc = 3;
    }
  }
  return res;
}

FCLG_HD ProjRes project_triangle_origin(const D3v& a, const D3v& b, const D3v& c) {
  ProjRes res;
  proj_init(res);
  const int nexti[3] = {1, 2, 0};
  const D3v vt[3] = {a, b, c};
  const D3v dl[3] = {a - b, b - c, c - a};
  const D3v n = cross(dl[0], dl[1]);
  const double l = sqnorm(n);
  if (l > 0) {
    double mindist = -1;
    for (int i = 0; i < 3; ++i) {
      if (dot(vt[i], cross(dl[i], n)) > 0) {
        const int j = nexti[i];
        const ProjRes rl = project_line_origin(vt[i], vt[j]);
        if (mindist < 0 || rl.sqd < mindist) {
          mindist = rl.sqd;
          res.enc = (unsigned)(((rl.enc & 1) ? 1 << i : 0) + ((rl.enc & 2) ? 1 << j : 0));
          res.par[i] = rl.par[0];
          res.par[j] = rl.par[1];
          res.par[nexti[j]] = 0;
        }
      }
    }
    if (mindist < 0) {
      const double d = dot(a, n);
      const double s = sqrt(l);
      const D3v o = d3scale(n, d / l);
      mindist = sqnorm(o);
      res.enc = 7;
      res.par[0] = d3norm(cross(dl[1], b - o)) / s;
      res.par[1] = d3norm(cross(dl[2], c - o)) / s;
      res.par[2] = 1 - res.par[0] - res.par[1];
    }
    res.sqd = mindist;
  }
  return res;
}

FCLG_HD ProjRes project_tetra_origin(const D3v& a, const D3v& b, const D3v& c, const D3v& d) {
  ProjRes res;
  proj_init(res);
  const int nexti[3] = {1, 2, 0};
  const D3v vt[4] = {a, b, c, d};
  const D3v dl[3] = {a - d, b - d, c - d};
  const double vl = d3triple(dl[0], dl[1], dl[2]);
  const bool ng = (vl * dot(a, cross(b - c, a - b))) <= 0;
  if (ng && fabs(vl) > 0) {
    double mindist = -1;
    for (int i = 0; i < 3; ++i) {
      const int j = nexti[i];
      const double s = vl * dot(d, cross(dl[i], dl[j]));
      if (s > 0) {
        const ProjRes rt = project_triangle_origin(vt[i], vt[j], d);
        if (mindist < 0 || rt.sqd < mindist) {
          mindist = rt.sqd;
          res.enc = (unsigned)((rt.enc & 1 ? 1 << i : 0) + (rt.enc & 2 ? 1 << j : 0) + (rt.enc & 4 ? 8 : 0));
          res.par[i] = rt.par[0];
          res.par[j] = rt.par[1];
          res.par[nexti[j]] = 0;
          res.par[3] = rt.par[2];
        }
      }
    }
    if (mindist < 0) {
      mindist = 0;
      res.enc = 15;
      res.par[0] = d3triple(c, b, d) / vl;
      res.par[1] = d3triple(a, c, d) / vl;
      res.par[2] = d3triple(b, a, d) / vl;
      res.par[3] = 1 - (res.par[0] + res.par[1] + res.par[2]);
    }
    res.sqd = mindist;
  } else if (!ng) {
    res = project_triangle_origin(a, b, c);
    res.par[3] = 0;
  }
  return res;
}

// ---- GJK -----------------------------------------------------------------------------
enum : int { GJK_VALID = 0, GJK_INSIDE = 1, GJK_FAILED = 2 };

constexpr int kEpaVerts = 64;
constexpr int kEpaFaces = 128;
constexpr int kSimplexSlots = 4 + kEpaVerts;

struct SimplexVert {
  D3v d, w;
};
struct Simplex {
  int c[4];
  double p[4];
  int rank;
};

struct GjkState {
  Minkowski shape;
  D3v ray;
  double distance;
  Simplex simplices[2];
  int free_v[4];
  int nfree;
  int current;
  int status;
  SimplexVert* V;  // vertex slots (>= 4 + EPA vertices)
  double tolerance;

  FCLG_HD void get_support(const D3v& d, SimplexVert& sv) const {
    sv.d = d3normalized(d);
    sv.w = shape.support(sv.d);
  }
  FCLG_HD void remove_vertex(Simplex& s) { free_v[nfree++] = s.c[--s.rank]; }
  FCLG_HD void append_vertex(Simplex& s, const D3v& v) {
    s.p[s.rank] = 0;
    s.c[s.rank] = free_v[--nfree];
    get_support(v, V[s.c[s.rank++]]);
  }

  // GJK::evaluate (gjk-inl.h:81-231) as begin / step / finish, so that a lane can run
  // one iteration at a time (the batch kernels refill a lane with the next pair as soon
  // as its GJK ends); evaluate() is the three in sequence.
  int iterations;
  double alpha;
  D3v lastw[4];
  int clastw;
  int max_iter;

  FCLG_HD void begin(const D3v& guess, int max_iterations) {
    iterations = 0;
    alpha = 0;
    clastw = 0;
    max_iter = max_iterations;
    free_v[0] = 0;
    free_v[1] = 1;
    free_v[2] = 2;
    free_v[3] = 3;
    nfree = 4;
    current = 0;
    status = GJK_VALID;
    distance = 0.0;
    simplices[0].rank = 0;
    ray = guess;
    append_vertex(simplices[0], (sqnorm(ray) > 0) ? d3neg(ray) : v3(1.0, 0.0, 0.0));
    simplices[0].p[0] = 1;
    ray = V[simplices[0].c[0]].w;
    lastw[0] = lastw[1] = lastw[2] = lastw[3] = ray;
  }
  // one pass of the do-while body; true when the loop ends
  FCLG_HD bool step() {
    const int next = 1 - current;
    Simplex& curr = simplices[current];
    Simplex& nxt = simplices[next];
    const double rl = d3norm(ray);
    if (rl < tolerance) {
      status = GJK_INSIDE;
      return true;
    }
    append_vertex(curr, d3neg(ray));
    const D3v w = V[curr.c[curr.rank - 1]].w;
    bool found = false;
    for (int i = 0; i < 4; ++i) {
      if (sqnorm(w - lastw[i]) < tolerance) {
        found = true;
        break;
      }
    }
    if (found) {
      remove_vertex(simplices[current]);
      return true;
    } else {
      lastw[clastw = (clastw + 1) & 3] = w;
    }
    const double omega = dot(ray, w) / rl;
    alpha = fmax(alpha, omega);
    if ((rl - alpha) - tolerance * rl <= 0) {
      remove_vertex(simplices[current]);
      return true;
    }
    ProjRes pr;
    proj_init(pr);
    switch (curr.rank) {
      case 2: pr = project_line_origin(V[curr.c[0]].w, V[curr.c[1]].w); break;
      case 3: pr = project_triangle_origin(V[curr.c[0]].w, V[curr.c[1]].w, V[curr.c[2]].w); break;
      case 4: pr = project_tetra_origin(V[curr.c[0]].w, V[curr.c[1]].w, V[curr.c[2]].w, V[curr.c[3]].w); break;
    }
    if (pr.sqd >= 0) {
      nxt.rank = 0;
      ray = v3(0.0, 0.0, 0.0);
      current = next;
      for (int i = 0; i < curr.rank; ++i) {
        if (pr.enc & (1u << i)) {
          nxt.c[nxt.rank] = curr.c[i];
          nxt.p[nxt.rank++] = pr.par[i];
          ray = ray + d3scale(V[curr.c[i]].w, pr.par[i]);
        } else {
          free_v[nfree++] = curr.c[i];
        }
      }
      if (pr.enc == 15) status = GJK_INSIDE;
    } else {
      remove_vertex(simplices[current]);
      return true;
    }
    status = ((++iterations) < max_iter) ? status : GJK_FAILED;
    return status != GJK_VALID;
  }
  FCLG_HD int finish() {
    switch (status) {
      case GJK_VALID: distance = d3norm(ray); break;
      case GJK_INSIDE: distance = 0; break;
      default: break;
    }
    return status;
  }
  FCLG_HD int evaluate(const D3v& guess, int max_iterations) {
    begin(guess, max_iterations);
    while (!step()) {
    }
    return finish();
  }

  // encloseOrigin (gjk-inl.h:235-298), unrolled by rank
  FCLG_HD bool enclose4(Simplex& s) {
    return fabs(d3triple(V[s.c[0]].w - V[s.c[3]].w, V[s.c[1]].w - V[s.c[3]].w, V[s.c[2]].w - V[s.c[3]].w)) > 0;
  }
  FCLG_HD bool enclose3(Simplex& s) {
    const D3v n = cross(V[s.c[1]].w - V[s.c[0]].w, V[s.c[2]].w - V[s.c[0]].w);
    if (sqnorm(n) > 0) {
      append_vertex(s, n);
      if (enclose4(s)) return true;
      remove_vertex(s);
      append_vertex(s, d3neg(n));
      if (enclose4(s)) return true;
      remove_vertex(s);
    }
    return false;
  }
  FCLG_HD bool enclose2(Simplex& s) {
    const D3v d = V[s.c[1]].w - V[s.c[0]].w;
    for (int i = 0; i < 3; ++i) {
      D3v axis = v3(0.0, 0.0, 0.0);
      if (i == 0) axis.x = 1;
      if (i == 1) axis.y = 1;
      if (i == 2) axis.z = 1;
      const D3v p = cross(d, axis);
      if (sqnorm(p) > 0) {
        append_vertex(s, p);
        if (enclose3(s)) return true;
        remove_vertex(s);
        append_vertex(s, d3neg(p));
        if (enclose3(s)) return true;
        remove_vertex(s);
      }
    }
    return false;
  }
  FCLG_HD bool enclose1(Simplex& s) {
    for (int i = 0; i < 3; ++i) {
      D3v axis = v3(0.0, 0.0, 0.0);
      if (i == 0) axis.x = 1;
      if (i == 1) axis.y = 1;
      if (i == 2) axis.z = 1;
      append_vertex(s, axis);
      if (enclose2(s)) return true;
      remove_vertex(s);
      append_vertex(s, d3neg(axis));
      if (enclose2(s)) return true;
      remove_vertex(s);
    }
    return false;
  }
  FCLG_HD bool enclose_origin() {
    Simplex& s = simplices[current];
    switch (s.rank) {
      case 1: return enclose1(s);
      case 2: return enclose2(s);
      case 3: return enclose3(s);
      case 4: return enclose4(s);
    }
    return false;
  }
};

// ---- EPA -------------------------------------------------------------------------------
enum : int {
  EPA_VALID = 0, EPA_TOUCHING, EPA_DEGENERATED, EPA_NONCONVEX, EPA_INVALIDHULL, EPA_OUTOFFACES, EPA_OUTOFVERTICES,
  EPA_ACCURACYREACHED, EPA_FALLBACK, EPA_FAILED
};

struct EpaFace {
  D3v n;
  double d;
  unsigned long long sqd;  // bits of d * d (>= 0): findBest compares them as integers
  int pass;
  short c[3];   // vertex slots
  short f[3];   // adjacent faces
  short l[2];   // list links (-1 = null)
  unsigned char e[3];
};

struct EpaList {
  int root;
  int count;
};

struct EpaState {
  EpaFace F[kEpaFaces];
  EpaList hull, stock;
  int nextsv;
  int status;
  D3v normal;
  double depth;
  int res_rank;
  int res_c[3];
  double res_p[3];
  double tolerance;

  FCLG_HD void list_append(EpaList& L, int face) {
    F[face].l[0] = -1;
    F[face].l[1] = (short)L.root;
    if (L.root >= 0) F[L.root].l[0] = (short)face;
    L.root = face;
    ++L.count;
  }
  FCLG_HD void list_remove(EpaList& L, int face) {
    if (F[face].l[1] >= 0) F[F[face].l[1]].l[0] = F[face].l[0];
    if (F[face].l[0] >= 0) F[F[face].l[0]].l[1] = F[face].l[1];
    if (face == L.root) L.root = F[face].l[1];
    --L.count;
  }
  FCLG_HD void bind(int fa, int ea, int fb, int eb) {
    F[fa].e[ea] = (unsigned char)eb;
    F[fa].f[ea] = (short)fb;
    F[fb].e[eb] = (unsigned char)ea;
    F[fb].f[eb] = (short)fa;
  }
  FCLG_HD void init() {
    hull.root = stock.root = -1;
    hull.count = stock.count = 0;
    status = EPA_FAILED;
    normal = v3(0.0, 0.0, 0.0);
    depth = 0;
    nextsv = 0;
    for (int i = 0; i < kEpaFaces; ++i) list_append(stock, kEpaFaces - i - 1);
  }
  FCLG_HD bool edge_dist(int face, const SimplexVert& a, const SimplexVert& b, double& dist) const {
    const D3v ba = b.w - a.w;
    const D3v n_ab = cross(ba, F[face].n);
    const double a_dot_nab = dot(a.w, n_ab);
    if (a_dot_nab < 0) {
      const double a_dot_ba = dot(a.w, ba);
      const double b_dot_ba = dot(b.w, ba);
      if (a_dot_ba > 0)
        dist = d3norm(a.w);
      else if (b_dot_ba < 0)
        dist = d3norm(b.w);
      else {
        const double a_dot_b = dot(a.w, b.w);
        dist = sqrt(fmax(sqnorm(a.w) * sqnorm(b.w) - a_dot_b * a_dot_b, 0.0));
      }
      return true;
    }
    return false;
  }
  FCLG_HD int new_face(const SimplexVert* V, int a, int b, int c, bool forced) {
    if (stock.root >= 0) {
      const int face = stock.root;
      list_remove(stock, face);
      list_append(hull, face);
      EpaFace& fc = F[face];
      fc.pass = 0;
      fc.c[0] = (short)a;
      fc.c[1] = (short)b;
      fc.c[2] = (short)c;
      fc.n = cross(V[b].w - V[a].w, V[c].w - V[a].w);
      const double l = d3norm(fc.n);
      if (l > tolerance) {
        if (!(edge_dist(face, V[a], V[b], fc.d) || edge_dist(face, V[b], V[c], fc.d) ||
              edge_dist(face, V[c], V[a], fc.d))) {
          fc.d = dot(V[a].w, fc.n) / l;
        }
        fc.n = v3(fc.n.x / l, fc.n.y / l, fc.n.z / l);
        fc.sqd = dbits(fc.d * fc.d);
        if (forced || fc.d >= -tolerance)
          return face;
        else
          status = EPA_NONCONVEX;
      } else {
        status = EPA_DEGENERATED;
      }
      list_remove(hull, face);
      list_append(stock, face);
      return -1;
    }
    status = (stock.root >= 0) ? EPA_OUTOFVERTICES : EPA_OUTOFFACES;
    return -1;
  }
  // findBest (epa-inl.h): the first face in hull order with the smallest d * d.  The
  // squares are non-negative doubles, whose order is the order of their bit patterns,
  // so the scan compares integers; a NaN square at the root wins as in FCL (no later
  // face compares less than NaN), and later NaN squares never win (their bits exceed
  // every finite square's).
  FCLG_HD int find_best() const {
    int minf = hull.root;
    unsigned long long mind = F[minf].sqd;
    if (mind > 0x7FF0000000000000ull) return minf;
    for (int f = F[minf].l[1]; f >= 0; f = F[f].l[1]) {
      const unsigned long long sqd = F[f].sqd;
      if (sqd < mind) {
        minf = f;
        mind = sqd;
      }
    }
    return minf;
  }

  struct Horizon {
    int cf, ff, nf;
  };

  // expand(pass, w, f, e, horizon) of epa-inl.h:348-399 on an explicit frame stack.
  FCLG_HD bool expand(const SimplexVert* V, int pass, int w, int f0, int e0, Horizon& hz, bool& overflow) {
    const int nexti[3] = {1, 2, 0};
    const int previ[3] = {2, 0, 1};
    struct Frame {
      short f;
      unsigned char e, state;
    };
    Frame st[kEpaFaces];
    int sp = 0;
    st[sp++] = Frame{(short)f0, (unsigned char)e0, 0};
    bool ret = false;
    while (sp > 0) {
      Frame& fr = st[sp - 1];
      const int f = fr.f;
      if (fr.state == 0) {
        if (F[f].pass == pass) {
          ret = false;
          --sp;
          continue;
        }
        const int e1 = nexti[fr.e];
        if (dot(F[f].n, V[w].w) - F[f].d < -tolerance) {
          const int nf = new_face(V, F[f].c[e1], F[f].c[fr.e], w, false);
          if (nf >= 0) {
            bind(nf, 0, f, fr.e);
            if (hz.cf >= 0)
              bind(nf, 2, hz.cf, 1);
            else
              hz.ff = nf;
            hz.cf = nf;
            ++hz.nf;
            ret = true;
          } else {
            ret = false;
          }
          --sp;
          continue;
        }
        F[f].pass = pass;
        fr.state = 1;
        if (sp >= kEpaFaces) {
          overflow = true;
          return false;
        }
        const int cf = F[f].f[e1], ce = F[f].e[e1];
        st[sp++] = Frame{(short)cf, (unsigned char)ce, 0};
        continue;
      }
      if (fr.state == 1) {
        if (!ret) {
          --sp;  // ret stays false
          continue;
        }
        const int e2 = previ[fr.e];
        fr.state = 2;
        if (sp >= kEpaFaces) {
          overflow = true;
          return false;
        }
        const int cf = F[f].f[e2], ce = F[f].e[e2];
        st[sp++] = Frame{(short)cf, (unsigned char)ce, 0};
        continue;
      }
      // state 2: second child returned ret
      if (ret) {
        list_remove(hull, f);
        list_append(stock, f);
      }
      --sp;
    }
    return ret;
  }

  // EPA::evaluate (epa-inl.h:224-344) as begin / step / finish, so that a lane can run
  // one expansion at a time; evaluate() is the three in sequence.  V holds the GJK
  // simplex slots 0-3 and EPA's support vertices at 4..4+kEpaVerts-1.
  GjkState* gk;
  int best, pass, iterations, max_iter;
  EpaFace outer;

  // true when the expansion loop has to run; false when the result is already final
  // (the FallBack case)
  FCLG_HD bool begin(GjkState& gjk, const D3v& guess, int max_iterations) {
    gk = &gjk;
    max_iter = max_iterations;
    SimplexVert* V = gjk.V;
    Simplex& simplex = gjk.simplices[gjk.current];
    if ((simplex.rank > 1) && gjk.enclose_origin()) {
      while (hull.root >= 0) {
        const int f = hull.root;
        list_remove(hull, f);
        list_append(stock, f);
      }
      status = EPA_VALID;
      nextsv = 0;
      if (dot(V[simplex.c[0]].w - V[simplex.c[3]].w,
              cross(V[simplex.c[1]].w - V[simplex.c[3]].w, V[simplex.c[2]].w - V[simplex.c[3]].w)) < 0) {
        const int tmp = simplex.c[0];
        simplex.c[0] = simplex.c[1];
        simplex.c[1] = tmp;
        const double tv = simplex.p[0];
        simplex.p[0] = simplex.p[1];
        simplex.p[1] = tv;
      }
      const int t0 = new_face(V, simplex.c[0], simplex.c[1], simplex.c[2], true);
      const int t1 = new_face(V, simplex.c[1], simplex.c[0], simplex.c[3], true);
      const int t2 = new_face(V, simplex.c[2], simplex.c[1], simplex.c[3], true);
      const int t3 = new_face(V, simplex.c[0], simplex.c[2], simplex.c[3], true);
      if (hull.count == 4) {
        best = find_best();
        outer = F[best];
        pass = 0;
        bind(t0, 0, t1, 0);
        bind(t0, 1, t2, 0);
        bind(t0, 2, t3, 0);
        bind(t1, 1, t3, 2);
        bind(t1, 2, t2, 1);
        bind(t2, 2, t3, 1);
        status = EPA_VALID;
        iterations = 0;
        if (max_iter > 0) return true;
        finish();
        return false;
      }
    }
    status = EPA_FALLBACK;
    normal = d3neg(guess);
    const double nl = d3norm(normal);
    if (nl > 0)
      normal = v3(normal.x / nl, normal.y / nl, normal.z / nl);
    else
      normal = v3(1.0, 0.0, 0.0);
    depth = 0;
    res_rank = 1;
    res_c[0] = simplex.c[0];
    res_p[0] = 1;
    return false;
  }
  // one pass of the expansion loop; true when the loop ends (then finish() has run)
  FCLG_HD bool step() {
    SimplexVert* V = gk->V;
    bool done = false;
    if (nextsv < kEpaVerts) {
      Horizon hz{-1, -1, 0};
      const int w = 4 + nextsv++;
      bool valid = true;
      F[best].pass = ++pass;
      gk->get_support(F[best].n, V[w]);
      const double wdist = dot(F[best].n, V[w].w) - F[best].d;
      if (wdist > tolerance) {
        bool overflow = false;
        for (int j = 0; (j < 3) && valid; ++j) valid &= expand(V, pass, w, F[best].f[j], F[best].e[j], hz, overflow);
        if (overflow) valid = false;
        if (valid && hz.nf >= 3) {
          bind(hz.ff, 2, hz.cf, 1);
          list_remove(hull, best);
          list_append(stock, best);
          best = find_best();
          outer = F[best];
        } else {
          status = EPA_INVALIDHULL;
          done = true;
        }
      } else {
        status = EPA_ACCURACYREACHED;
        done = true;
      }
    } else {
      status = EPA_OUTOFVERTICES;
      done = true;
    }
    if (!done && ++iterations >= max_iter) done = true;
    if (done) finish();
    return done;
  }
  FCLG_HD void finish() {
    const SimplexVert* V = gk->V;
    const D3v projection = d3scale(outer.n, outer.d);
    normal = outer.n;
    depth = outer.d;
    res_rank = 3;
    res_c[0] = outer.c[0];
    res_c[1] = outer.c[1];
    res_c[2] = outer.c[2];
    res_p[0] = d3norm(cross(V[outer.c[1]].w - projection, V[outer.c[2]].w - projection));
    res_p[1] = d3norm(cross(V[outer.c[2]].w - projection, V[outer.c[0]].w - projection));
    res_p[2] = d3norm(cross(V[outer.c[0]].w - projection, V[outer.c[1]].w - projection));
    const double sum = res_p[0] + res_p[1] + res_p[2];
    res_p[0] /= sum;
    res_p[1] /= sum;
    res_p[2] /= sum;
  }
  FCLG_HD int evaluate(GjkState& gjk, const D3v& guess, int max_iterations) {
    if (begin(gjk, guess, max_iterations))
      while (!step()) {
      }
    return status;
  }
};

}  // namespace fclgpu
