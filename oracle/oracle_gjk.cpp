// FP64 CPU oracle: FCL 0.7.0's own GJK/EPA (GST_INDEP) and closed-form pairs.
// TEST INFRASTRUCTURE ONLY.  Structure (pointer-linked simplex vertices, intrusive
// face lists, stock order) follows the reference so tie-breaks are identical.
#include "oracle_gjk.h"

#include <algorithm>
#include <cmath>
#include <limits>

namespace oracle {

namespace {

inline double triple(const V3& x, const V3& y, const V3& z) { return dot(x, cross(y, z)); }
inline V3 normalized(const V3& v) {
  double n = norm(v);
  return mk(v[0] / n, v[1] / n, v[2] / n);
}
const double kTol = 2.0097183471152322e-14;  // std::pow(eps, 7/8) = 2^-45.5 (math/constants.h:164-167)

// GJKSolver_indep's parameters as the solver used by fcl::collide / fcl::distance holds
// them (gjk_solver_indep-inl.h:1039-1049 defaults; collision-inl.h:164-170 and
// distance-inl.h:211-215 set the tolerances from the request).
struct SolverParamsO {
  double gjk_tolerance = kTol, epa_tolerance = kTol;
  size_t gjk_max_iterations = 128, epa_max_iterations = 255;
};
SolverParamsO g_solver_params;

// narrowphase/detail/convexity_based_algorithm/minkowski_diff-inl.h:65-206
V3 get_support(const Shape& s, const V3& dir) {
  switch (s.type) {
    case SH_BOX:
      return mk((dir[0] > 0) ? (s.p[0] / 2) : (-s.p[0] / 2), (dir[1] > 0) ? (s.p[1] / 2) : (-s.p[1] / 2),
                (dir[2] > 0) ? (s.p[2] / 2) : (-s.p[2] / 2));
    case SH_SPHERE:
      return scale(dir, s.p[0]);
    case SH_CAPSULE: {
      double half_h = s.p[1] * 0.5;
      V3 pos1 = mk(0, 0, half_h), pos2 = mk(0, 0, -half_h);
      V3 v = scale(dir, s.p[0]);
      pos1 = add(pos1, v);
      pos2 = add(pos2, v);
      if (dot(dir, pos1) > dot(dir, pos2)) return pos1;
      return pos2;
    }
    case SH_CONE: {
      double zdist = dir[0] * dir[0] + dir[1] * dir[1];
      double len = zdist + dir[2] * dir[2];
      zdist = std::sqrt(zdist);
      len = std::sqrt(len);
      double half_h = s.p[1] * 0.5;
      double radius = s.p[0];
      double sin_a = radius / std::sqrt(radius * radius + 4 * half_h * half_h);
      if (dir[2] > len * sin_a) return mk(0, 0, half_h);
      if (zdist > 0) {
        double rad = radius / zdist;
        return mk(rad * dir[0], rad * dir[1], -half_h);
      }
      return mk(0, 0, -half_h);
    }
    case SH_CYLINDER: {
      double zdist = std::sqrt(dir[0] * dir[0] + dir[1] * dir[1]);
      double half_h = s.p[1] * 0.5;
      if (zdist == 0.0) return mk(0, 0, (dir[2] > 0) ? half_h : -half_h);
      double d = s.p[0] / zdist;
      return mk(d * dir[0], d * dir[1], (dir[2] > 0) ? half_h : -half_h);
    }
    case SH_CONVEX: {
      double maxdot = -std::numeric_limits<double>::max();
      V3 bestv = mk(0, 0, 0);
      for (int i = 0; i < s.nverts; ++i) {
        double d = dot(dir, s.verts[i]);
        if (d > maxdot) {
          bestv = s.verts[i];
          maxdot = d;
        }
      }
      return bestv;
    }
    case SH_TRIANGLE: {  // TriangleP (minkowski_diff-inl.h:78-97)
      const double dota = dot(dir, s.verts[0]);
      const double dotb = dot(dir, s.verts[1]);
      const double dotc = dot(dir, s.verts[2]);
      if (dota > dotb) return (dotc > dota) ? s.verts[2] : s.verts[0];
      return (dotc > dotb) ? s.verts[2] : s.verts[1];
    }
  }
  return mk(0, 0, 0);
}

struct Minkowski {
  const Shape* s0;
  const Shape* s1;
  M3 toshape1;  // R2^T R1
  Tf toshape0;  // tf1^-1 tf2
  V3 support0(const V3& d) const { return get_support(*s0, d); }
  V3 support1(const V3& d) const { return apply(toshape0, get_support(*s1, mulv(toshape1, d))); }
  V3 support(const V3& d) const { return sub(support0(d), support1(neg(d))); }
  V3 support(const V3& d, int index) const { return index ? support1(d) : support0(d); }
};

Minkowski make_minkowski(const Shape& s1, const Tf& tf1, const Shape& s2, const Tf& tf2) {
  Minkowski m;
  m.s0 = &s1;
  m.s1 = &s2;
  m.toshape1 = mulT(tf2.R, tf1.R);
  // tf1.inverse(Isometry) * tf2
  M3 Ri = transpose(tf1.R);
  V3 ti = neg(mulv(Ri, tf1.t));
  m.toshape0.R = mul(Ri, tf2.R);
  m.toshape0.t = add(mulv(Ri, tf2.t), ti);
  return m;
}

}  // namespace

// math/detail/project-inl.h:183-200
ProjectResult project_line(const V3& a, const V3& b) {
  ProjectResult res;
  const V3 d = sub(b, a);
  const double l = sqnorm(d);
  if (l > 0) {
    const double t = -dot(a, d);
    res.parameterization[1] = (t >= l) ? 1 : ((t <= 0) ? 0 : (t / l));
    res.parameterization[0] = 1 - res.parameterization[1];
    if (t >= l) {
      res.sqr_distance = sqnorm(b);
      res.encode = 2;
    } else if (t <= 0) {
      res.sqr_distance = sqnorm(a);
      res.encode = 1;
    } else {
      res.sqr_distance = sqnorm(add(a, scale(d, res.parameterization[1])));
      res.encode = 3;
    }
  }
  return res;
}

// project-inl.h:203-249
ProjectResult project_triangle(const V3& a, const V3& b, const V3& c) {
  ProjectResult res;
  static const size_t nexti[3] = {1, 2, 0};
  const V3* vt[] = {&a, &b, &c};
  const V3 dl[] = {sub(a, b), sub(b, c), sub(c, a)};
  const V3 n = cross(dl[0], dl[1]);
  const double l = sqnorm(n);
  if (l > 0) {
    double mindist = -1;
    for (size_t i = 0; i < 3; ++i) {
      if (dot(*vt[i], cross(dl[i], n)) > 0) {
        size_t j = nexti[i];
        ProjectResult res_line = project_line(*vt[i], *vt[j]);
        if (mindist < 0 || res_line.sqr_distance < mindist) {
          mindist = res_line.sqr_distance;
          res.encode = (unsigned)(((res_line.encode & 1) ? 1 << i : 0) + ((res_line.encode & 2) ? 1 << j : 0));
          res.parameterization[i] = res_line.parameterization[0];
          res.parameterization[j] = res_line.parameterization[1];
          res.parameterization[nexti[j]] = 0;
        }
      }
    }
    if (mindist < 0) {
      double d = dot(a, n);
      double s = std::sqrt(l);
      V3 o_to_project = scale(n, d / l);
      mindist = sqnorm(o_to_project);
      res.encode = 7;
      res.parameterization[0] = norm(cross(dl[1], sub(b, o_to_project))) / s;
      res.parameterization[1] = norm(cross(dl[2], sub(c, o_to_project))) / s;
      res.parameterization[2] = 1 - res.parameterization[0] - res.parameterization[1];
    }
    res.sqr_distance = mindist;
  }
  return res;
}

// project-inl.h:252-306
ProjectResult project_tetra(const V3& a, const V3& b, const V3& c, const V3& d) {
  ProjectResult res;
  static const size_t nexti[] = {1, 2, 0};
  const V3* vt[] = {&a, &b, &c, &d};
  const V3 dl[3] = {sub(a, d), sub(b, d), sub(c, d)};
  double vl = triple(dl[0], dl[1], dl[2]);
  bool ng = (vl * dot(a, cross(sub(b, c), sub(a, b)))) <= 0;
  if (ng && std::abs(vl) > 0) {
    double mindist = -1;
    for (size_t i = 0; i < 3; ++i) {
      size_t j = nexti[i];
      double s = vl * dot(d, cross(dl[i], dl[j]));
      if (s > 0) {
        ProjectResult res_triangle = project_triangle(*vt[i], *vt[j], d);
        if (mindist < 0 || res_triangle.sqr_distance < mindist) {
          mindist = res_triangle.sqr_distance;
          res.encode = (unsigned)((res_triangle.encode & 1 ? 1 << i : 0) + (res_triangle.encode & 2 ? 1 << j : 0) +
                                  (res_triangle.encode & 4 ? 8 : 0));
          res.parameterization[i] = res_triangle.parameterization[0];
          res.parameterization[j] = res_triangle.parameterization[1];
          res.parameterization[nexti[j]] = 0;
          res.parameterization[3] = res_triangle.parameterization[2];
        }
      }
    }
    if (mindist < 0) {
      mindist = 0;
      res.encode = 15;
      res.parameterization[0] = triple(c, b, d) / vl;
      res.parameterization[1] = triple(a, c, d) / vl;
      res.parameterization[2] = triple(b, a, d) / vl;
      res.parameterization[3] = 1 - (res.parameterization[0] + res.parameterization[1] + res.parameterization[2]);
    }
    res.sqr_distance = mindist;
  } else if (!ng) {
    res = project_triangle(a, b, c);
    res.parameterization[3] = 0;
  }
  return res;
}

namespace {

// ---------------------------------------------------------------------------------
// GJK (convexity_based_algorithm/gjk-inl.h:81-298)
// ---------------------------------------------------------------------------------
struct SimplexV {
  V3 d, w;
};
struct Simplex {
  SimplexV* c[4];
  double p[4];
  size_t rank = 0;
};

enum GStatus { G_Valid = 0, G_Inside = 1, G_Failed = 2 };

struct GJK {
  Minkowski shape;
  V3 ray;
  double distance;
  Simplex simplices[2];
  SimplexV store_v[4];
  SimplexV* free_v[4];
  size_t nfree;
  size_t current;
  Simplex* simplex;
  int status;
  size_t max_iterations = g_solver_params.gjk_max_iterations;
  double tolerance = g_solver_params.gjk_tolerance;

  void get_support(const V3& d, SimplexV& sv) const {
    sv.d = normalized(d);
    sv.w = shape.support(sv.d);
  }
  void remove_vertex(Simplex& s) { free_v[nfree++] = s.c[--s.rank]; }
  void append_vertex(Simplex& s, const V3& v) {
    s.p[s.rank] = 0;
    s.c[s.rank] = free_v[--nfree];
    get_support(v, *s.c[s.rank++]);
  }

  int evaluate(const Minkowski& shape_, const V3& guess) {
    size_t iterations = 0;
    double alpha = 0;
    V3 lastw[4];
    size_t clastw = 0;
    free_v[0] = &store_v[0];
    free_v[1] = &store_v[1];
    free_v[2] = &store_v[2];
    free_v[3] = &store_v[3];
    nfree = 4;
    current = 0;
    status = G_Valid;
    shape = shape_;
    distance = 0.0;
    simplices[0].rank = 0;
    ray = guess;
    append_vertex(simplices[0], (sqnorm(ray) > 0) ? neg(ray) : mk(1, 0, 0));
    simplices[0].p[0] = 1;
    ray = simplices[0].c[0]->w;
    lastw[0] = lastw[1] = lastw[2] = lastw[3] = ray;
    do {
      size_t next = 1 - current;
      Simplex& curr = simplices[current];
      Simplex& nxt = simplices[next];
      double rl = norm(ray);
      if (rl < tolerance) {
        status = G_Inside;
        break;
      }
      append_vertex(curr, neg(ray));
      V3& w = curr.c[curr.rank - 1]->w;
      bool found = false;
      for (size_t i = 0; i < 4; ++i) {
        if (sqnorm(sub(w, lastw[i])) < tolerance) {
          found = true;
          break;
        }
      }
      if (found) {
        remove_vertex(simplices[current]);
        break;
      } else {
        lastw[clastw = (clastw + 1) & 3] = w;
      }
      double omega = dot(ray, w) / rl;
      alpha = std::max(alpha, omega);
      if ((rl - alpha) - tolerance * rl <= 0) {
        remove_vertex(simplices[current]);
        break;
      }
      ProjectResult pr;
      switch (curr.rank) {
        case 2: pr = project_line(curr.c[0]->w, curr.c[1]->w); break;
        case 3: pr = project_triangle(curr.c[0]->w, curr.c[1]->w, curr.c[2]->w); break;
        case 4: pr = project_tetra(curr.c[0]->w, curr.c[1]->w, curr.c[2]->w, curr.c[3]->w); break;
      }
      if (pr.sqr_distance >= 0) {
        nxt.rank = 0;
        ray = mk(0, 0, 0);
        current = next;
        for (size_t i = 0; i < curr.rank; ++i) {
          if (pr.encode & (1 << i)) {
            nxt.c[nxt.rank] = curr.c[i];
            nxt.p[nxt.rank++] = pr.parameterization[i];
            ray = add(ray, scale(curr.c[i]->w, pr.parameterization[i]));
          } else {
            free_v[nfree++] = curr.c[i];
          }
        }
        if (pr.encode == 15) status = G_Inside;
      } else {
        remove_vertex(simplices[current]);
        break;
      }
      status = ((++iterations) < max_iterations) ? status : G_Failed;
    } while (status == G_Valid);
    simplex = &simplices[current];
    switch (status) {
      case G_Valid: distance = norm(ray); break;
      case G_Inside: distance = 0; break;
      default: break;
    }
    return status;
  }

  bool enclose_origin() {
    switch (simplex->rank) {
      case 1:
        for (size_t i = 0; i < 3; ++i) {
          V3 axis = mk(0, 0, 0);
          axis[i] = 1;
          append_vertex(*simplex, axis);
          if (enclose_origin()) return true;
          remove_vertex(*simplex);
          append_vertex(*simplex, neg(axis));
          if (enclose_origin()) return true;
          remove_vertex(*simplex);
        }
        break;
      case 2: {
        V3 d = sub(simplex->c[1]->w, simplex->c[0]->w);
        for (size_t i = 0; i < 3; ++i) {
          V3 axis = mk(0, 0, 0);
          axis[i] = 1;
          V3 p = cross(d, axis);
          if (sqnorm(p) > 0) {
            append_vertex(*simplex, p);
            if (enclose_origin()) return true;
            remove_vertex(*simplex);
            append_vertex(*simplex, neg(p));
            if (enclose_origin()) return true;
            remove_vertex(*simplex);
          }
        }
      } break;
      case 3: {
        V3 n = cross(sub(simplex->c[1]->w, simplex->c[0]->w), sub(simplex->c[2]->w, simplex->c[0]->w));
        if (sqnorm(n) > 0) {
          append_vertex(*simplex, n);
          if (enclose_origin()) return true;
          remove_vertex(*simplex);
          append_vertex(*simplex, neg(n));
          if (enclose_origin()) return true;
          remove_vertex(*simplex);
        }
      } break;
      case 4:
        if (std::abs(triple(sub(simplex->c[0]->w, simplex->c[3]->w), sub(simplex->c[1]->w, simplex->c[3]->w),
                            sub(simplex->c[2]->w, simplex->c[3]->w))) > 0)
          return true;
        break;
    }
    return false;
  }
};

// ---------------------------------------------------------------------------------
// EPA (convexity_based_algorithm/epa-inl.h:54-399)
// ---------------------------------------------------------------------------------
enum EStatus {
  E_Valid = 0, E_Touching, E_Degenerated, E_NonConvex, E_InvalidHull, E_OutOfFaces, E_OutOfVertices,
  E_AccuracyReached, E_FallBack, E_Failed
};

struct SimplexF {
  V3 n;
  double d;
  SimplexV* c[3];
  SimplexF* f[3];
  SimplexF* l[2];
  size_t e[3];
  size_t pass;
};
struct SimplexList {
  SimplexF* root = nullptr;
  size_t count = 0;
  void append(SimplexF* face) {
    face->l[0] = nullptr;
    face->l[1] = root;
    if (root) root->l[0] = face;
    root = face;
    ++count;
  }
  void remove(SimplexF* face) {
    if (face->l[1]) face->l[1]->l[0] = face->l[0];
    if (face->l[0]) face->l[0]->l[1] = face->l[1];
    if (face == root) root = face->l[1];
    --count;
  }
};
struct SimplexHorizon {
  SimplexF* cf = nullptr;
  SimplexF* ff = nullptr;
  size_t nf = 0;
};

struct EPA {
  size_t max_face_num = 128, max_vertex_num = 64, max_iterations = g_solver_params.epa_max_iterations;
  double tolerance = g_solver_params.epa_tolerance;
  int status;
  Simplex result;
  V3 normal;
  double depth;
  std::vector<SimplexV> sv_store;
  std::vector<SimplexF> fc_store;
  size_t nextsv;
  SimplexList hull, stock;

  EPA() {
    sv_store.resize(max_vertex_num);
    fc_store.resize(max_face_num);
    status = E_Failed;
    normal = mk(0, 0, 0);
    depth = 0;
    nextsv = 0;
    for (size_t i = 0; i < max_face_num; ++i) stock.append(&fc_store[max_face_num - i - 1]);
  }

  static void bind(SimplexF* fa, size_t ea, SimplexF* fb, size_t eb) {
    fa->e[ea] = eb;
    fa->f[ea] = fb;
    fb->e[eb] = ea;
    fb->f[eb] = fa;
  }

  bool get_edge_dist(SimplexF* face, SimplexV* a, SimplexV* b, double& dist) {
    V3 ba = sub(b->w, a->w);
    V3 n_ab = cross(ba, face->n);
    double a_dot_nab = dot(a->w, n_ab);
    if (a_dot_nab < 0) {
      double a_dot_ba = dot(a->w, ba);
      double b_dot_ba = dot(b->w, ba);
      if (a_dot_ba > 0)
        dist = norm(a->w);
      else if (b_dot_ba < 0)
        dist = norm(b->w);
      else {
        double a_dot_b = dot(a->w, b->w);
        dist = std::sqrt(std::max(sqnorm(a->w) * sqnorm(b->w) - a_dot_b * a_dot_b, 0.0));
      }
      return true;
    }
    return false;
  }

  SimplexF* new_face(SimplexV* a, SimplexV* b, SimplexV* c, bool forced) {
    if (stock.root) {
      SimplexF* face = stock.root;
      stock.remove(face);
      hull.append(face);
      face->pass = 0;
      face->c[0] = a;
      face->c[1] = b;
      face->c[2] = c;
      face->n = cross(sub(b->w, a->w), sub(c->w, a->w));
      double l = norm(face->n);
      if (l > tolerance) {
        if (!(get_edge_dist(face, a, b, face->d) || get_edge_dist(face, b, c, face->d) ||
              get_edge_dist(face, c, a, face->d))) {
          face->d = dot(a->w, face->n) / l;
        }
        face->n = mk(face->n[0] / l, face->n[1] / l, face->n[2] / l);
        if (forced || face->d >= -tolerance)
          return face;
        else
          status = E_NonConvex;
      } else
        status = E_Degenerated;
      hull.remove(face);
      stock.append(face);
      return nullptr;
    }
    status = stock.root ? E_OutOfVertices : E_OutOfFaces;
    return nullptr;
  }

  SimplexF* find_best() {
    SimplexF* minf = hull.root;
    double mind = minf->d * minf->d;
    for (SimplexF* f = minf->l[1]; f; f = f->l[1]) {
      double sqd = f->d * f->d;
      if (sqd < mind) {
        minf = f;
        mind = sqd;
      }
    }
    return minf;
  }

  bool expand(size_t pass, SimplexV* w, SimplexF* f, size_t e, SimplexHorizon& horizon) {
    static const size_t nexti[] = {1, 2, 0};
    static const size_t previ[] = {2, 0, 1};
    if (f->pass != pass) {
      const size_t e1 = nexti[e];
      if (dot(f->n, w->w) - f->d < -tolerance) {
        SimplexF* nf = new_face(f->c[e1], f->c[e], w, false);
        if (nf) {
          bind(nf, 0, f, e);
          if (horizon.cf)
            bind(nf, 2, horizon.cf, 1);
          else
            horizon.ff = nf;
          horizon.cf = nf;
          ++horizon.nf;
          return true;
        }
      } else {
        const size_t e2 = previ[e];
        f->pass = pass;
        if (expand(pass, w, f->f[e1], f->e[e1], horizon) && expand(pass, w, f->f[e2], f->e[e2], horizon)) {
          hull.remove(f);
          stock.append(f);
          return true;
        }
      }
    }
    return false;
  }

  int evaluate(GJK& gjk, const V3& guess) {
    Simplex& simplex = *gjk.simplex;
    if ((simplex.rank > 1) && gjk.enclose_origin()) {
      while (hull.root) {
        SimplexF* f = hull.root;
        hull.remove(f);
        stock.append(f);
      }
      status = E_Valid;
      nextsv = 0;
      if (dot(sub(simplex.c[0]->w, simplex.c[3]->w),
              cross(sub(simplex.c[1]->w, simplex.c[3]->w), sub(simplex.c[2]->w, simplex.c[3]->w))) < 0) {
        SimplexV* tmp = simplex.c[0];
        simplex.c[0] = simplex.c[1];
        simplex.c[1] = tmp;
        double tmpv = simplex.p[0];
        simplex.p[0] = simplex.p[1];
        simplex.p[1] = tmpv;
      }
      SimplexF* tetrahedron[] = {new_face(simplex.c[0], simplex.c[1], simplex.c[2], true),
                                 new_face(simplex.c[1], simplex.c[0], simplex.c[3], true),
                                 new_face(simplex.c[2], simplex.c[1], simplex.c[3], true),
                                 new_face(simplex.c[0], simplex.c[2], simplex.c[3], true)};
      if (hull.count == 4) {
        SimplexF* best = find_best();
        SimplexF outer = *best;
        size_t pass = 0;
        size_t iterations = 0;
        bind(tetrahedron[0], 0, tetrahedron[1], 0);
        bind(tetrahedron[0], 1, tetrahedron[2], 0);
        bind(tetrahedron[0], 2, tetrahedron[3], 0);
        bind(tetrahedron[1], 1, tetrahedron[3], 2);
        bind(tetrahedron[1], 2, tetrahedron[2], 1);
        bind(tetrahedron[2], 2, tetrahedron[3], 1);
        status = E_Valid;
        for (; iterations < max_iterations; ++iterations) {
          if (nextsv < max_vertex_num) {
            SimplexHorizon horizon;
            SimplexV* w = &sv_store[nextsv++];
            bool valid = true;
            best->pass = ++pass;
            gjk.get_support(best->n, *w);
            double wdist = dot(best->n, w->w) - best->d;
            if (wdist > tolerance) {
              for (size_t j = 0; (j < 3) && valid; ++j) valid &= expand(pass, w, best->f[j], best->e[j], horizon);
              if (valid && horizon.nf >= 3) {
                bind(horizon.ff, 2, horizon.cf, 1);
                hull.remove(best);
                stock.append(best);
                best = find_best();
                outer = *best;
              } else {
                status = E_InvalidHull;
                break;
              }
            } else {
              status = E_AccuracyReached;
              break;
            }
          } else {
            status = E_OutOfVertices;
            break;
          }
        }
        V3 projection = scale(outer.n, outer.d);
        normal = outer.n;
        depth = outer.d;
        result.rank = 3;
        result.c[0] = outer.c[0];
        result.c[1] = outer.c[1];
        result.c[2] = outer.c[2];
        result.p[0] = norm(cross(sub(outer.c[1]->w, projection), sub(outer.c[2]->w, projection)));
        result.p[1] = norm(cross(sub(outer.c[2]->w, projection), sub(outer.c[0]->w, projection)));
        result.p[2] = norm(cross(sub(outer.c[0]->w, projection), sub(outer.c[1]->w, projection)));
        double sum = result.p[0] + result.p[1] + result.p[2];
        result.p[0] /= sum;
        result.p[1] /= sum;
        result.p[2] /= sum;
        return status;
      }
    }
    status = E_FallBack;
    normal = neg(guess);
    double nl = norm(normal);
    if (nl > 0)
      normal = mk(normal[0] / nl, normal[1] / nl, normal[2] / nl);
    else
      normal = mk(1, 0, 0);
    depth = 0;
    result.rank = 1;
    result.c[0] = simplex.c[0];
    result.p[0] = 1;
    return status;
  }
};

// ---------------------------------------------------------------------------------
// Closed-form pairs (primitive_shape_algorithm/*-inl.h)
// ---------------------------------------------------------------------------------
// Point p of frame B expressed in frame A: X_AB = X_FA^-1 X_FB (Isometry inverse).
inline V3 inv_apply(const Tf& X, const V3& p) {
  M3 Ri = transpose(X.R);
  V3 ti = neg(mulv(Ri, X.t));
  return add(mulv(Ri, p), ti);
}
// translation of X_FA.inverse() * X_FB
inline V3 rel_translation(const Tf& XA, const Tf& XB) { return inv_apply(XA, XB.t); }

// ---- box-box (box_box-inl.h) -------------------------------------------------------
// box_box-inl.h:60-80
void bb_line_closest(const V3& pa, const V3& ua, const V3& pb, const V3& ub, double* alpha, double* beta) {
  const V3 p = sub(pb, pa);
  const double uaub = dot(ua, ub);
  const double q1 = dot(ua, p);
  const double q2 = -dot(ub, p);
  double d = 1 - uaub * uaub;
  if (d <= (double)(0.0001f)) {
    *alpha = 0;
    *beta = 0;
  } else {
    d = 1 / d;
    *alpha = (q1 + uaub * q2) * d;
    *beta = (uaub * q1 + q2) * d;
  }
}

// box_box-inl.h:84-164: Sutherland-Hodgman clip of the quad p[8] by |x| < h0 then
// |y| < h1, stopping once 8 points exist
int bb_clip(const double h[2], const double p[8], double ret[16]) {
  std::vector<double> cur(p, p + 8), nxt;
  int nq = 4;
  for (int dir = 0; dir <= 1; ++dir) {
    for (int sign = -1; sign <= 1; sign += 2) {
      nxt.clear();
      int nr = 0;
      for (int i = 0; i < nq; ++i) {
        const double* a = &cur[2 * i];
        const double* b = &cur[2 * ((i + 1) % nq)];
        const bool ina = sign * a[dir] < h[dir], inb = sign * b[dir] < h[dir];
        if (ina) {
          nxt.push_back(a[0]);
          nxt.push_back(a[1]);
          if (++nr == 8) {
            std::copy(nxt.begin(), nxt.end(), ret);
            return 8;
          }
        }
        if (ina != inb) {
          double pt[2];
          pt[1 - dir] = a[1 - dir] + (b[1 - dir] - a[1 - dir]) / (b[dir] - a[dir]) * (sign * h[dir] - a[dir]);
          pt[dir] = sign * h[dir];
          nxt.push_back(pt[0]);
          nxt.push_back(pt[1]);
          if (++nr == 8) {
            std::copy(nxt.begin(), nxt.end(), ret);
            return 8;
          }
        }
      }
      cur = nxt;
      nq = nr;
    }
  }
  std::copy(cur.begin(), cur.end(), ret);
  return nq;
}

// box_box-inl.h:168-240: keep m of the n polygon points, i0 first, then the free point
// whose angle about the centroid is nearest A[i0] + j 2 pi / m
void bb_cull(int n, const double p[], int m, int i0, int iret[]) {
  double a, cx, cy, q;
  if (n == 1) {
    cx = p[0];
    cy = p[1];
  } else if (n == 2) {
    cx = 0.5 * (p[0] + p[2]);
    cy = 0.5 * (p[1] + p[3]);
  } else {
    a = cx = cy = 0;
    for (int i = 0; i < n - 1; ++i) {
      q = p[i * 2] * p[i * 2 + 3] - p[i * 2 + 2] * p[i * 2 + 1];
      a += q;
      cx += q * (p[i * 2] + p[i * 2 + 2]);
      cy += q * (p[i * 2 + 1] + p[i * 2 + 3]);
    }
    q = p[n * 2 - 2] * p[1] - p[0] * p[n * 2 - 1];
    if (std::abs(a + q) > std::numeric_limits<double>::epsilon())
      a = 1 / (3 * (a + q));
    else
      a = 1e18f;
    cx = a * (cx + q * (p[n * 2 - 2] + p[0]));
    cy = a * (cy + q * (p[n * 2 - 1] + p[1]));
  }
  double A[8];
  for (int i = 0; i < n; ++i) A[i] = std::atan2(p[i * 2 + 1] - cy, p[i * 2] - cx);
  int avail[8];
  for (int i = 0; i < n; ++i) avail[i] = 1;
  avail[i0] = 0;
  iret[0] = i0;
  const double pi = 3.141592653589793238462643383279502884197169399;
  for (int j = 1; j < m; ++j) {
    a = j * (2 * pi / m) + A[i0];
    if (a > pi) a -= 2 * pi;
    double maxdiff = 1e9;
    iret[j] = i0;
    for (int i = 0; i < n; ++i) {
      if (!avail[i]) continue;
      double diff = std::abs(A[i] - a);
      if (diff > pi) diff = 2 * pi - diff;
      if (diff < maxdiff) {
        maxdiff = diff;
        iret[j] = i;
      }
    }
    avail[iret[j]] = 0;
  }
}

struct BbContact {
  V3 normal, pos;
  double depth;
};

// box_box-inl.h:244-834 (boxBox2) with maxc contacts; returns return_code
int box_box2(const double* side1, const Tf& tf1, const double* side2, const Tf& tf2, int maxc,
             std::vector<BbContact>& out) {
  const M3 &R1 = tf1.R, &R2 = tf2.R;
  const V3 &T1 = tf1.t, &T2 = tf2.t;
  const V3 p = sub(T2, T1);
  const V3 pp = mulTv(R1, p);
  const V3 A = scale(mk(side1[0], side1[1], side1[2]), 0.5);
  const V3 B = scale(mk(side2[0], side2[1], side2[2]), 0.5);
  const M3 R = mulT(R1, R2);
  M3 Q;
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) Q(r, c) = std::abs(R(r, c));

  double s = -std::numeric_limits<double>::max();
  int invert_normal = 0, code = 0;
  const M3* normalR = nullptr;
  int best_col = -1;
  V3 normalC = mk(0, 0, 0);
  auto face = [&](double tmp, double s2, const M3* Rn, int colid, int c) {
    if (s2 > 0) return false;
    if (s2 > s) {
      s = s2;
      best_col = colid;
      normalR = Rn;
      invert_normal = tmp < 0;
      code = c;
    }
    return true;
  };
  for (int i = 0; i < 3; ++i)
    if (!face(pp[i], std::abs(pp[i]) - (dot(row(Q, i), B) + A[i]), &R1, i, 1 + i)) return 0;
  for (int j = 0; j < 3; ++j) {
    const double tmp = dot(col(R2, j), p);
    if (!face(tmp, std::abs(tmp) - (dot(col(Q, j), A) + B[j]), &R2, j, 4 + j)) return 0;
  }
  const double eps = std::numeric_limits<double>::epsilon();
  {
    const double mA = std::max(std::max(A[0], A[1]), A[2]), mB = std::max(std::max(B[0], B[1]), B[2]);
    const double sf = std::max(std::max(mA, mB), 1.0) * 10.0 * eps;
    for (int r = 0; r < 3; ++r)
      for (int c = 0; c < 3; ++c) Q(r, c) += sf;
  }
  // the nine edge axes in the reference's order (u1 x v1 .. u3 x v3), each as the
  // projection tmp, the radius sum and the unnormalised axis n (box-1 frame)
  struct Edge {
    double tmp, rad;
    V3 n;
  };
  const Edge edges[9] = {
      {pp[2] * R(1, 0) - pp[1] * R(2, 0), A[1] * Q(2, 0) + A[2] * Q(1, 0) + B[1] * Q(0, 2) + B[2] * Q(0, 1),
       mk(0, -R(2, 0), R(1, 0))},
      {pp[2] * R(1, 1) - pp[1] * R(2, 1), A[1] * Q(2, 1) + A[2] * Q(1, 1) + B[0] * Q(0, 2) + B[2] * Q(0, 0),
       mk(0, -R(2, 1), R(1, 1))},
      {pp[2] * R(1, 2) - pp[1] * R(2, 2), A[1] * Q(2, 2) + A[2] * Q(1, 2) + B[0] * Q(0, 1) + B[1] * Q(0, 0),
       mk(0, -R(2, 2), R(1, 2))},
      {pp[0] * R(2, 0) - pp[2] * R(0, 0), A[0] * Q(2, 0) + A[2] * Q(0, 0) + B[1] * Q(1, 2) + B[2] * Q(1, 1),
       mk(R(2, 0), 0, -R(0, 0))},
      {pp[0] * R(2, 1) - pp[2] * R(0, 1), A[0] * Q(2, 1) + A[2] * Q(0, 1) + B[0] * Q(1, 2) + B[2] * Q(1, 0),
       mk(R(2, 1), 0, -R(0, 1))},
      {pp[0] * R(2, 2) - pp[2] * R(0, 2), A[0] * Q(2, 2) + A[2] * Q(0, 2) + B[0] * Q(1, 1) + B[1] * Q(1, 0),
       mk(R(2, 2), 0, -R(0, 2))},
      {pp[1] * R(0, 0) - pp[0] * R(1, 0), A[0] * Q(1, 0) + A[1] * Q(0, 0) + B[1] * Q(2, 2) + B[2] * Q(2, 1),
       mk(-R(1, 0), R(0, 0), 0)},
      {pp[1] * R(0, 1) - pp[0] * R(1, 1), A[0] * Q(1, 1) + A[1] * Q(0, 1) + B[0] * Q(2, 2) + B[2] * Q(2, 0),
       mk(-R(1, 1), R(0, 1), 0)},
      {pp[1] * R(0, 2) - pp[0] * R(1, 2), A[0] * Q(1, 2) + A[1] * Q(0, 2) + B[0] * Q(2, 1) + B[1] * Q(2, 0),
       mk(-R(1, 2), R(0, 2), 0)},
  };
  // the reference evaluates each edge axis only after the previous ones passed; the
  // table above computes all nine first, which changes no value
  for (int e = 0; e < 9; ++e) {
    double s2 = std::abs(edges[e].tmp) - edges[e].rad;
    if (s2 > 0) return 0;
    const double l = norm(edges[e].n);
    if (l > eps) {
      s2 /= l;
      if (s2 * 1.05 > s) {
        s = s2;
        best_col = -1;
        normalC = mk(edges[e].n[0] / l, edges[e].n[1] / l, edges[e].n[2] / l);
        invert_normal = edges[e].tmp < 0;
        code = 7 + e;
      }
    }
  }
  if (!code) return 0;
  V3 normal = best_col != -1 ? col(*normalR, best_col) : mulv(R1, normalC);
  if (invert_normal) normal = neg(normal);
  const double depth = -s;

  if (code > 6) {
    V3 pa = T1;
    for (int j = 0; j < 3; ++j) pa = add(pa, scale(col(R1, j), A[j] * (dot(col(R1, j), normal) > 0 ? 1 : -1)));
    V3 pb = T2;
    for (int j = 0; j < 3; ++j) pb = add(pb, scale(col(R2, j), B[j] * (dot(col(R2, j), normal) > 0 ? -1 : 1)));
    double alpha, beta;
    const V3 ua = col(R1, (code - 7) / 3), ub = col(R2, (code - 7) % 3);
    bb_line_closest(pa, ua, pb, ub, &alpha, &beta);
    pa = add(pa, scale(ua, alpha));
    pb = add(pb, scale(ub, beta));
    out.push_back({normal, scale(add(pa, pb), 0.5), depth});
    return code;
  }

  const bool r1 = code <= 3;
  const M3& Ra = r1 ? R1 : R2;
  const M3& Rb = r1 ? R2 : R1;
  const V3& pa = r1 ? T1 : T2;
  const V3& pb = r1 ? T2 : T1;
  const V3& Sa = r1 ? A : B;
  const V3& Sb = r1 ? B : A;
  const V3 normal2 = r1 ? normal : neg(normal);
  const V3 nr = mulTv(Rb, normal2);
  const V3 anr = mk(std::abs(nr[0]), std::abs(nr[1]), std::abs(nr[2]));
  int lanr, a1, a2;
  if (anr[1] > anr[0]) {
    if (anr[1] > anr[2]) {
      a1 = 0, lanr = 1, a2 = 2;
    } else {
      a1 = 0, a2 = 1, lanr = 2;
    }
  } else {
    if (anr[0] > anr[2]) {
      lanr = 0, a1 = 1, a2 = 2;
    } else {
      a1 = 0, a2 = 1, lanr = 2;
    }
  }
  const V3 center = nr[lanr] < 0 ? add(sub(pb, pa), scale(col(Rb, lanr), Sb[lanr]))
                                 : sub(sub(pb, pa), scale(col(Rb, lanr), Sb[lanr]));
  const int codeN = r1 ? code - 1 : code - 4;
  const int code1 = codeN == 0 ? 1 : 0;
  const int code2 = codeN == 2 ? 1 : 2;
  const double c1 = dot(col(Ra, code1), center), c2 = dot(col(Ra, code2), center);
  double m11 = dot(col(Rb, a1), col(Ra, code1)), m12 = dot(col(Rb, a2), col(Ra, code1));
  double m21 = dot(col(Rb, a1), col(Ra, code2)), m22 = dot(col(Rb, a2), col(Ra, code2));
  const double k1 = m11 * Sb[a1], k2 = m21 * Sb[a1], k3 = m12 * Sb[a2], k4 = m22 * Sb[a2];
  const double quad[8] = {c1 - k1 - k3, c2 - k2 - k4, c1 - k1 + k3, c2 - k2 + k4,
                          c1 + k1 + k3, c2 + k2 + k4, c1 + k1 - k3, c2 + k2 - k4};
  const double rect[2] = {Sa[code1], Sa[code2]};
  double ret[16];
  const int n_int = bb_clip(rect, quad, ret);
  if (n_int < 1) return code;
  V3 points[8];
  double dep[8];
  const double det1 = 1.f / (m11 * m22 - m12 * m21);
  m11 *= det1;
  m12 *= det1;
  m21 *= det1;
  m22 *= det1;
  int cnum = 0;
  for (int j = 0; j < n_int; ++j) {
    const double e1 = m22 * (ret[j * 2] - c1) - m12 * (ret[j * 2 + 1] - c2);
    const double e2 = -m21 * (ret[j * 2] - c1) + m11 * (ret[j * 2 + 1] - c2);
    points[cnum] = add(add(center, scale(col(Rb, a1), e1)), scale(col(Rb, a2), e2));
    dep[cnum] = Sa[codeN] - dot(normal2, points[cnum]);
    if (dep[cnum] >= 0) {
      ret[cnum * 2] = ret[j * 2];
      ret[cnum * 2 + 1] = ret[j * 2 + 1];
      cnum++;
    }
  }
  if (cnum < 1) return code;
  if (maxc > cnum) maxc = cnum;
  if (maxc < 1) maxc = 1;
  int iret[8] = {0, 1, 2, 3, 4, 5, 6, 7};
  if (cnum > maxc) {
    int i1 = 0;
    double maxdepth = dep[0];
    for (int i = 1; i < cnum; ++i)
      if (dep[i] > maxdepth) {
        maxdepth = dep[i];
        i1 = i;
      }
    bb_cull(cnum, ret, maxc, i1, iret);
    cnum = maxc;
  }
  for (int j = 0; j < cnum; ++j) {
    const int i = iret[j];
    const V3 half = scale(normal, dep[i] / 2);
    out.push_back({normal, r1 ? add(add(points[i], pa), half) : sub(add(points[i], pa), half), dep[i]});
  }
  return code;
}

// boxBoxIntersect (box_box-inl.h:858-876) as collide() sees it: with contacts, the
// traversal node keeps num_max_contacts = 1 of them, the deepest, by a size-1
// std::partial_sort (shape_collision_traversal_node-inl.h:78-100), which keeps the
// first maximum in order; the pair counts as colliding only if a contact was added.
// Without contacts the answer is return_code != 0.
bool box_box_intersect(const Shape& s1, const Tf& tf1, const Shape& s2, const Tf& tf2, bool enable_contact,
                       ShapeResult& r) {
  std::vector<BbContact> cs;
  const int rc = box_box2(s1.p, tf1, s2.p, tf2, 4, cs);
  if (!enable_contact) return rc != 0;
  if (cs.empty()) return false;
  size_t best = 0;
  for (size_t i = 1; i < cs.size(); ++i)
    if (cs[best].depth < cs[i].depth) best = i;
  r.normal = cs[best].normal;
  r.point = cs[best].pos;
  r.depth = cs[best].depth;
  return true;
}

// sphere_sphere-inl.h:67-87
bool sphere_sphere_intersect(const Shape& s1, const Tf& tf1, const Shape& s2, const Tf& tf2, ShapeResult& r) {
  V3 diff = sub(tf2.t, tf1.t);
  double len = norm(diff);
  if (len > s1.p[0] + s2.p[0]) return false;
  r.normal = len > 0 ? mk(diff[0] / len, diff[1] / len, diff[2] / len) : diff;
  V3 t = scale(diff, s1.p[0]);
  double den = s1.p[0] + s2.p[0];
  r.point = add(tf1.t, mk(t[0] / den, t[1] / den, t[2] / den));
  r.depth = s1.p[0] + s2.p[0] - len;
  return true;
}
// sphere_sphere-inl.h:90-108
bool sphere_sphere_distance(const Shape& s1, const Tf& tf1, const Shape& s2, const Tf& tf2, double* dist, V3* p1,
                            V3* p2) {
  V3 o1 = tf1.t, o2 = tf2.t;
  V3 diff = sub(o1, o2);
  double len = norm(diff);
  if (len > s1.p[0] + s2.p[0]) {
    *dist = len - (s1.p[0] + s2.p[0]);
    *p1 = sub(o1, scale(diff, s1.p[0] / len));
    *p2 = add(o2, scale(diff, s2.p[0] / len));
    return true;
  }
  *dist = -1;
  return false;
}

// sphere_capsule-inl.h:71-88
void segment_closest(const V3& p, const V3& s1, const V3& s2, V3& sp) {
  V3 v = sub(s2, s1);
  V3 w = sub(p, s1);
  double c1 = dot(w, v);
  double c2 = dot(v, v);
  if (c1 <= 0)
    sp = s1;
  else if (c2 <= c1)
    sp = s2;
  else {
    double b = c1 / c2;
    sp = add(s1, scale(v, b));
  }
}
// sphere_capsule-inl.h:91-122
bool sphere_capsule_intersect(const Shape& s1, const Tf& tf1, const Shape& s2, const Tf& tf2, ShapeResult& r) {
  const V3 pos1 = mk(0., 0., 0.5 * s2.p[1]);
  const V3 pos2 = mk(0., 0., -0.5 * s2.p[1]);
  const V3 s_c = inv_apply(tf2, tf1.t);
  V3 segment_point;
  segment_closest(s_c, pos1, pos2, segment_point);
  V3 diff = sub(s_c, segment_point);
  const double distance = norm(diff) - s1.p[0] - s2.p[0];
  if (distance > 0) return false;
  const V3 local_normal = neg(normalized(diff));
  r.normal = mulv(tf2.R, local_normal);
  r.point = apply(tf2, add(segment_point, scale(local_normal, distance)));
  r.depth = -distance;
  return true;
}
// sphere_capsule-inl.h:125-166
bool sphere_capsule_distance(const Shape& s1, const Tf& tf1, const Shape& s2, const Tf& tf2, double* dist, V3* p1,
                             V3* p2) {
  V3 pos1 = mk(0., 0., 0.5 * s2.p[1]);
  V3 pos2 = mk(0., 0., -0.5 * s2.p[1]);
  V3 s_c = inv_apply(tf2, tf1.t);
  V3 segment_point;
  segment_closest(s_c, pos1, pos2, segment_point);
  V3 diff = sub(s_c, segment_point);
  double distance = norm(diff) - s1.p[0] - s2.p[0];
  if (distance <= 0) {
    *dist = -1;
    return false;
  }
  *dist = distance;
  diff = normalized(diff);
  *p1 = apply(tf2, sub(s_c, scale(diff, s1.p[0])));
  *p2 = apply(tf2, add(segment_point, scale(diff, s2.p[0])));
  return true;
}

// sphere_box-inl.h (nearestPointInBox, sphereBoxIntersect, sphereBoxDistance)
bool nearest_in_box(const double side[3], const V3& p, V3& n) {
  const V3 half = mk(side[0] / 2, side[1] / 2, side[2] / 2);
  bool clamped = false;
  for (int i = 0; i < 3; ++i) {
    n[i] = p[i];
    if (p[i] < -half[i]) {
      clamped = true;
      n[i] = -half[i];
    }
    if (p[i] > half[i]) {
      clamped = true;
      n[i] = half[i];
    }
  }
  return clamped;
}
bool sphere_box_intersect(const Shape& sph, const Tf& X_FS, const Shape& box, const Tf& X_FB, ShapeResult& res) {
  const double r = sph.p[0];
  const V3 p_BC = rel_translation(X_FB, X_FS);
  V3 p_BN;
  bool N_is_not_C = nearest_in_box(box.p, p_BC, p_BN);
  V3 p_CN_B = sub(p_BN, p_BC);
  double squared_distance = sqnorm(p_CN_B);
  if (squared_distance > r * r) return false;
  double depth = 0;
  V3 n_SB_B, p_BP;
  const double eps = 16 * std::numeric_limits<double>::epsilon();
  if (N_is_not_C && squared_distance > eps * eps) {
    double distance = std::sqrt(squared_distance);
    n_SB_B = mk(p_CN_B[0] / distance, p_CN_B[1] / distance, p_CN_B[2] / distance);
    depth = r - distance;
    p_BP = add(p_BN, scale(n_SB_B, depth * 0.5));
  } else {
    V3 half = mk(box.p[0] / 2, box.p[1] / 2, box.p[2] / 2);
    double min_distance = std::numeric_limits<double>::infinity();
    int min_axis = -1;
    for (int i = 0; i < 3; ++i) {
      double dist = p_BC[i] >= 0 ? half[i] - p_BC[i] : p_BC[i] + half[i];
      if (dist + eps < min_distance) {
        min_distance = dist;
        min_axis = i;
      }
    }
    n_SB_B = mk(0, 0, 0);
    n_SB_B[min_axis] = p_BC[min_axis] >= 0 ? -1 : 1;
    depth = min_distance + r;
    p_BP = add(p_BC, scale(n_SB_B, (r - min_distance) / 2));
  }
  res.normal = mulv(X_FB.R, n_SB_B);
  res.point = apply(X_FB, p_BP);
  res.depth = depth;
  return true;
}
bool sphere_box_distance(const Shape& sph, const Tf& X_FS, const Shape& box, const Tf& X_FB, double* distance,
                         V3* p_FSb, V3* p_FBs) {
  const V3 p_BC = rel_translation(X_FB, X_FS);
  const double r = sph.p[0];
  V3 p_BN;
  bool N_is_not_C = nearest_in_box(box.p, p_BC, p_BN);
  if (N_is_not_C) {
    V3 p_NC_B = sub(p_BC, p_BN);
    double squared_distance = sqnorm(p_NC_B);
    if (squared_distance > r * r) {
      double d = std::sqrt(squared_distance);
      *distance = d - r;
      *p_FBs = apply(X_FB, p_BN);
      const V3 u = mk(p_NC_B[0] / d, p_NC_B[1] / d, p_NC_B[2] / d);
      const V3 p_BSb = add(scale(u, d - r), p_BN);
      *p_FSb = apply(X_FB, p_BSb);
      return true;
    }
  }
  *distance = -1;
  return false;
}

// sphere_cylinder-inl.h (nearestPointInCylinder, sphereCylinderIntersect/Distance)
bool nearest_in_cylinder(double height, double radius, const V3& p_CQ, V3& p_CN) {
  p_CN = p_CQ;
  bool clamped = false;
  const double half_height = height / 2;
  if (p_CQ[2] > half_height) {
    clamped = true;
    p_CN[2] = half_height;
  } else if (p_CQ[2] < -half_height) {
    clamped = true;
    p_CN[2] = -half_height;
  }
  double rx = p_CQ[0], ry = p_CQ[1];
  double squared_distance = rx * rx + ry * ry;
  if (squared_distance > radius * radius) {
    clamped = true;
    const double k = radius / std::sqrt(squared_distance);
    rx *= k;
    ry *= k;
    p_CN[0] = rx;
    p_CN[1] = ry;
  }
  return clamped;
}
bool sphere_cylinder_intersect(const Shape& sph, const Tf& X_FS, const Shape& cyl, const Tf& X_FC,
                               ShapeResult& res) {
  const double r_s = sph.p[0];
  const V3 p_CS = rel_translation(X_FC, X_FS);
  V3 p_CN;
  bool S_is_outside = nearest_in_cylinder(cyl.p[1], cyl.p[0], p_CS, p_CN);
  const V3 p_SN_C = sub(p_CN, p_CS);
  const double p_SN_squared_dist = sqnorm(p_SN_C);
  if (p_SN_squared_dist > r_s * r_s) return false;
  double depth = 0;
  V3 n_SC_C, p_CP;
  const double eps = 16 * std::numeric_limits<double>::epsilon();
  if (S_is_outside && p_SN_squared_dist > eps * eps) {
    const double d_NS = std::sqrt(p_SN_squared_dist);
    n_SC_C = mk(p_SN_C[0] / d_NS, p_SN_C[1] / d_NS, p_SN_C[2] / d_NS);
    depth = r_s - d_NS;
    p_CP = add(p_CN, scale(n_SC_C, depth * 0.5));
  } else {
    const double h = cyl.p[1];
    const double face_distance = p_CS[2] >= 0 ? h / 2 - p_CS[2] : p_CS[2] + h / 2;
    const double nx = p_CS[0], ny = p_CS[1];
    const double d_CS_xy = std::sqrt(nx * nx + ny * ny);
    const double barrel_distance = cyl.p[0] - d_CS_xy;
    if (barrel_distance < face_distance - eps) {
      if (d_CS_xy > eps) {
        n_SC_C = mk(-nx / d_CS_xy, -ny / d_CS_xy, 0);
        depth = r_s + barrel_distance;
        p_CP = add(p_CS, scale(n_SC_C, (r_s - barrel_distance) / 2));
      } else {
        n_SC_C = mk(-1, 0, 0);
        depth = r_s + cyl.p[0];
        p_CP = add(p_CS, scale(n_SC_C, (r_s - barrel_distance) / 2));
      }
    } else {
      n_SC_C = mk(0, 0, 0);
      n_SC_C[2] = p_CS[2] >= 0 ? -1 : 1;
      depth = face_distance + r_s;
      p_CP = add(p_CS, scale(n_SC_C, (r_s - face_distance) / 2));
    }
  }
  res.normal = mulv(X_FC.R, n_SC_C);
  res.point = apply(X_FC, p_CP);
  res.depth = depth;
  return true;
}
bool sphere_cylinder_distance(const Shape& sph, const Tf& X_FS, const Shape& cyl, const Tf& X_FC, double* distance,
                              V3* p_FSc, V3* p_FCs) {
  const V3 p_CS = rel_translation(X_FC, X_FS);
  const double r_s = sph.p[0];
  V3 p_CN;
  bool S_is_outside = nearest_in_cylinder(cyl.p[1], cyl.p[0], p_CS, p_CN);
  if (S_is_outside) {
    const V3 p_NS_C = sub(p_CS, p_CN);
    const double p_NS_squared_dist = sqnorm(p_NS_C);
    if (p_NS_squared_dist > r_s * r_s) {
      double d = std::sqrt(p_NS_squared_dist);
      *distance = d - r_s;
      *p_FCs = apply(X_FC, p_CN);
      const V3 t = scale(p_NS_C, r_s);
      const V3 p_CSc = sub(p_CS, mk(t[0] / d, t[1] / d, t[2] / d));
      *p_FSc = apply(X_FC, p_CSc);
      return true;
    }
  }
  *distance = -1;
  return false;
}

// capsule_capsule-inl.h:81-244
double clampd(double n, double lo, double hi) {
  if (n < lo) return lo;
  if (n > hi) return hi;
  return n;
}
double closest_seg_seg(const V3& p_FP1, const V3& p_FQ1, const V3& p_FP2, const V3& p_FQ2, double* s, double* t,
                       V3* p_FC1, V3* p_FC2) {
  const double kEps = kTol;
  const double kEpsSquared = kEps * kEps;
  V3 p_P1Q1 = sub(p_FQ1, p_FP1);
  V3 p_P2Q2 = sub(p_FQ2, p_FP2);
  V3 p_P2P1 = sub(p_FP1, p_FP2);
  double a = dot(p_P1Q1, p_P1Q1);
  double e = dot(p_P2Q2, p_P2Q2);
  double f = dot(p_P2Q2, p_P2P1);
  if (a <= kEpsSquared && e <= kEpsSquared) {
    *s = *t = 0.0;
    *p_FC1 = p_FP1;
    *p_FC2 = p_FP2;
    return sqnorm(sub(*p_FC1, *p_FC2));
  }
  if (a <= kEpsSquared) {
    *s = 0.0;
    *t = clampd(f / e, 0.0, 1.0);
  } else {
    const double c = dot(p_P1Q1, p_P2P1);
    if (e <= kEpsSquared) {
      *t = 0.0;
      *s = clampd(-c / a, 0.0, 1.0);
    } else {
      const double b = dot(p_P1Q1, p_P2Q2);
      const double denom = std::max(0.0, a * e - b * b);
      if (denom > kEpsSquared)
        *s = clampd((b * f - c * e) / denom, 0.0, 1.0);
      else
        *s = 0.0;
      *t = (b * (*s) + f) / e;
      if (*t < 0.0) {
        *t = 0.0;
        *s = clampd(-c / a, 0.0, 1.0);
      } else if (*t > 1.0) {
        *t = 1.0;
        *s = clampd((b - c) / a, 0.0, 1.0);
      }
    }
  }
  *p_FC1 = add(p_FP1, scale(p_P1Q1, *s));
  *p_FC2 = add(p_FP2, scale(p_P2Q2, *t));
  return sqnorm(sub(*p_FC1, *p_FC2));
}
bool capsule_capsule_distance(const Shape& s1, const Tf& X1, const Shape& s2, const Tf& X2, double* dist, V3* pw1,
                              V3* pw2) {
  const V3 o1 = X1.t, o2 = X2.t;
  const V3 arm1 = scale(col(X1.R, 2), s1.p[1] / 2);
  const V3 arm2 = scale(col(X2.R, 2), s2.p[1] / 2);
  // half_length * Cz_F (scalar times vector)
  const V3 a1 = add(o1, arm1), b1 = sub(o1, arm1);
  const V3 a2 = add(o2, arm2), b2 = sub(o2, arm2);
  double s, t;
  V3 n1, n2;
  const double sq = closest_seg_seg(a1, b1, a2, b2, &s, &t, &n1, &n2);
  const double segment_dist = std::sqrt(sq);
  *dist = segment_dist - s1.p[0] - s2.p[0];
  V3 vhat;
  const double eps = kTol;
  if (segment_dist > eps) {
    V3 dd = sub(n2, n1);
    vhat = mk(dd[0] / segment_dist, dd[1] / segment_dist, dd[2] / segment_dist);
  } else {
    const V3 z1 = col(X1.R, 2), z2 = col(X2.R, 2);
    if (std::abs(dot(z1, z2)) < 1 - eps)
      vhat = normalized(cross(z1, z2));
    else
      vhat = col(X1.R, 0);
  }
  *pw1 = add(n1, scale(vhat, s1.p[0]));
  *pw2 = sub(n2, scale(vhat, s2.p[0]));
  return true;
}

}  // namespace

// ShapeIntersectIndepImpl (gjk_solver_indep-inl.h:111-166), GJK guess (1,0,0)
bool gjk_intersect(const Shape& s1, const Tf& tf1, const Shape& s2, const Tf& tf2, V3* normal, V3* point,
                   double* depth, int* gjk_status, int* epa_status) {
  V3 guess = mk(1, 0, 0);
  Minkowski shape = make_minkowski(s1, tf1, s2, tf2);
  GJK gjk;
  int gs = gjk.evaluate(shape, neg(guess));
  if (gjk_status) *gjk_status = gs;
  if (epa_status) *epa_status = -1;
  if (gs == G_Inside) {
    EPA epa;
    int es = epa.evaluate(gjk, neg(guess));
    if (epa_status) *epa_status = es;
    if (es != E_Failed) {
      V3 w0 = mk(0, 0, 0);
      for (size_t i = 0; i < epa.result.rank; ++i)
        w0 = add(w0, scale(shape.support(epa.result.c[i]->d, 0), epa.result.p[i]));
      *normal = epa.normal;
      *point = apply(tf1, sub(w0, scale(epa.normal, epa.depth * 0.5)));
      *depth = -epa.depth;
      return true;
    }
    return false;
  }
  return false;
}

// ShapeDistanceIndepImpl (gjk_solver_indep-inl.h:593-645)
bool gjk_distance(const Shape& s1, const Tf& tf1, const Shape& s2, const Tf& tf2, double* dist, V3* p1, V3* p2,
                  int* gjk_status) {
  V3 guess = mk(1, 0, 0);
  Minkowski shape = make_minkowski(s1, tf1, s2, tf2);
  GJK gjk;
  int gs = gjk.evaluate(shape, neg(guess));
  if (gjk_status) *gjk_status = gs;
  if (gs == G_Valid) {
    V3 w0 = mk(0, 0, 0), w1 = mk(0, 0, 0);
    for (size_t i = 0; i < gjk.simplex->rank; ++i) {
      double p = gjk.simplex->p[i];
      w0 = add(w0, scale(shape.support(gjk.simplex->c[i]->d, 0), p));
      w1 = add(w1, scale(shape.support(neg(gjk.simplex->c[i]->d), 1), p));
    }
    *dist = norm(sub(w0, w1));
    *p1 = apply(tf1, w0);
    *p2 = apply(tf1, w1);
    return true;
  }
  *dist = -1;
  return false;
}

// Dispatch of GJKSolver_indep (gjk_solver_indep-inl.h:242-262 intersect, 710-860
// distance) restricted to Box/Sphere/Capsule/Cylinder/Cone/Convex.
bool shape_intersect(const Shape& s1, const Tf& tf1, const Shape& s2, const Tf& tf2, ShapeResult& r,
                     bool enable_contact) {
  const int a = s1.type, b = s2.type;
  bool hit;
  if (a == SH_BOX && b == SH_BOX) {
    hit = box_box_intersect(s1, tf1, s2, tf2, enable_contact, r);
  } else if (a == SH_SPHERE && b == SH_SPHERE) {
    hit = sphere_sphere_intersect(s1, tf1, s2, tf2, r);
  } else if (a == SH_SPHERE && b == SH_CAPSULE) {
    hit = sphere_capsule_intersect(s1, tf1, s2, tf2, r);
  } else if (a == SH_CAPSULE && b == SH_SPHERE) {
    hit = sphere_capsule_intersect(s2, tf2, s1, tf1, r);
    if (hit) r.normal = neg(r.normal);
  } else if (a == SH_SPHERE && b == SH_BOX) {
    hit = sphere_box_intersect(s1, tf1, s2, tf2, r);
  } else if (a == SH_BOX && b == SH_SPHERE) {
    hit = sphere_box_intersect(s2, tf2, s1, tf1, r);
    if (hit) r.normal = neg(r.normal);
  } else if (a == SH_SPHERE && b == SH_CYLINDER) {
    hit = sphere_cylinder_intersect(s1, tf1, s2, tf2, r);
  } else if (a == SH_CYLINDER && b == SH_SPHERE) {
    hit = sphere_cylinder_intersect(s2, tf2, s1, tf1, r);
    if (hit) r.normal = neg(r.normal);
  } else {
    // GST_INDEP stores ContactPoint::penetration_depth = -epa.depth (the sign FCL
    // 0.7.0 reports for this solver); it is returned as is
    hit = gjk_intersect(s1, tf1, s2, tf2, &r.normal, &r.point, &r.depth, &r.gjk_status, &r.epa_status);
  }
  return hit;
}

void shape_distance(const Shape& s1, const Tf& tf1, const Shape& s2, const Tf& tf2, ShapeResult& r) {
  const int a = s1.type, b = s2.type;
  if (a == SH_SPHERE && b == SH_SPHERE) {
    sphere_sphere_distance(s1, tf1, s2, tf2, &r.distance, &r.p1, &r.p2);
  } else if (a == SH_SPHERE && b == SH_CAPSULE) {
    sphere_capsule_distance(s1, tf1, s2, tf2, &r.distance, &r.p1, &r.p2);
  } else if (a == SH_CAPSULE && b == SH_SPHERE) {
    sphere_capsule_distance(s2, tf2, s1, tf1, &r.distance, &r.p2, &r.p1);
  } else if (a == SH_SPHERE && b == SH_BOX) {
    sphere_box_distance(s1, tf1, s2, tf2, &r.distance, &r.p1, &r.p2);
  } else if (a == SH_BOX && b == SH_SPHERE) {
    sphere_box_distance(s2, tf2, s1, tf1, &r.distance, &r.p2, &r.p1);
  } else if (a == SH_SPHERE && b == SH_CYLINDER) {
    sphere_cylinder_distance(s1, tf1, s2, tf2, &r.distance, &r.p1, &r.p2);
  } else if (a == SH_CYLINDER && b == SH_SPHERE) {
    sphere_cylinder_distance(s2, tf2, s1, tf1, &r.distance, &r.p2, &r.p1);
  } else if (a == SH_CAPSULE && b == SH_CAPSULE) {
    capsule_capsule_distance(s1, tf1, s2, tf2, &r.distance, &r.p1, &r.p2);
  } else {
    gjk_distance(s1, tf1, s2, tf2, &r.distance, &r.p1, &r.p2, &r.gjk_status);
  }
}

void shape_pair(const Shape& s1, const Tf& tf1, const Shape& s2, const Tf& tf2, ShapeResult& r) {
  r.collide = false;
  r.normal = r.point = r.p1 = r.p2 = mk(0, 0, 0);
  r.depth = 0;
  r.distance = -1;
  r.gjk_status = r.epa_status = -1;
  r.collide = shape_intersect(s1, tf1, s2, tf2, r);
  if (!r.collide) shape_distance(s1, tf1, s2, tf2, r);
}

void set_solver_params(double gjk_tolerance, double epa_tolerance, size_t gjk_max_iterations,
                       size_t epa_max_iterations) {
  g_solver_params.gjk_tolerance = gjk_tolerance;
  g_solver_params.epa_tolerance = epa_tolerance;
  g_solver_params.gjk_max_iterations = gjk_max_iterations;
  g_solver_params.epa_max_iterations = epa_max_iterations;
}

}  // namespace oracle
