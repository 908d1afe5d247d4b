// Per-query OBBRSS collide traversal, shared by the GPU kernel and by the test-only
// host build that checks the kernel logic against the oracle without a GPU.
//
// The visit order is FCL's collisionRecurse (traversal_recurse-inl.h:82-129) with an
// explicit stack: test the pair; at a leaf pair run the triangle test and append a
// contact; otherwise descend into the larger node (firstOverSecond,
// bvh_collision_traversal_node-inl.h:77-89) and push the sibling.  The traversal
// ends as soon as num_max_contacts contacts exist (canStop between siblings,
// collision_request-inl.h:76-82: once it holds, FCL performs no further test).
#pragma once
#include "filter32.cuh"
#include "geom.cuh"
#include "kernels.h"

#if defined(__CUDA_ARCH__)
#define FCLG_LDG(p) __ldg(p)
#define FCLG_F2I(x) __float_as_int(x)
#else
#include <cstring>
#define FCLG_LDG(p) (*(p))
static inline int fclg_f2i_host(float x) {
  int i;
  std::memcpy(&i, &x, 4);
  return i;
}
#define FCLG_F2I(x) fclg_f2i_host(x)
#endif

namespace fclgpu {

struct QueryStats {
  long long nbv, nleaf, nrecheck;
  unsigned int status;
};

FCLG_HD void load_nodeD(const NodeD* p, NodeD& n) {
#if defined(__CUDA_ARCH__)
  const double2* s = reinterpret_cast<const double2*>(p);
  double2* d = reinterpret_cast<double2*>(&n);
#pragma unroll
  for (int i = 0; i < 8; ++i) d[i] = __ldg(s + i);
#else
  n = *p;
#endif
}

// Relative transform of query qi (tf1 = I when absent).
FCLG_HD void query_transform_collide(const double* tf1, const double* tf2, long long qi, M3<double>& R,
                                     V3<double>& T, double* ta) {
  double tb[12];
  if (tf1) {
    for (int i = 0; i < 12; ++i) ta[i] = FCLG_LDG(tf1 + 12 * qi + i);
  } else {
    for (int i = 0; i < 12; ++i) ta[i] = (i == 0 || i == 5 || i == 10) ? 1.0 : 0.0;
  }
  for (int i = 0; i < 12; ++i) tb[i] = FCLG_LDG(tf2 + 12 * qi + i);
  rel_collide(ta, tb, R, T);
}

// Exact FP64 leaf test (intersect-inl.h:597-617) on triangle ids p1, p2.
#if defined(__CUDACC__)
static __device__ __host__ __noinline__
#else
inline
#endif
bool leaf_collide64(const DevMesh& A, const DevMesh& B, int p1, int p2, const M3<double>& R, const V3<double>& T) {
  const int* ta = A.tris + 3 * (long long)p1;
  const int* tb = B.tris + 3 * (long long)p2;
  V3<double> P[3], Q[3];
  for (int k = 0; k < 3; ++k) {
    const double* pa = A.verts64 + 3 * (long long)FCLG_LDG(ta + k);
    const double* pb = B.verts64 + 3 * (long long)FCLG_LDG(tb + k);
    P[k] = v3(FCLG_LDG(pa), FCLG_LDG(pa + 1), FCLG_LDG(pa + 2));
    Q[k] = v3(FCLG_LDG(pb), FCLG_LDG(pb + 1), FCLG_LDG(pb + 2));
  }
  return tri_intersect<double>(P[0], P[1], P[2], Q[0], Q[1], Q[2], R, T);
}

#if defined(__CUDACC__)
static __device__ __host__ __noinline__
#else
inline
#endif
bool bv_overlap64(const DevMesh& A, const DevMesh& B, int b1, int b2, const M3<double>& R, const V3<double>& T) {
  NodeD na, nb;
  load_nodeD(A.nodes64 + b1, na);
  load_nodeD(B.nodes64 + b2, nb);
  return obb_overlap64(R, T, na, nb);
}

// Per-item traversal with a test budget, used by the work-splitting batch.
//
// An item is a query plus a starting BV pair.  The item runs FCL's DFS from that pair
// until it is exhausted or `budget` BV tests have been spent.  In the second case the
// unfinished frontier -- the current pair, then the stacked siblings from the top of
// the stack down -- is exactly the rest of the item's DFS order, split into
// contiguous pieces; the caller writes it out as new items in that order.  The
// item's own contacts are a prefix of its DFS-order output, so the batch output is
// rebuilt as: own contacts, then the children's outputs in order.
// Sink interface: push(item, rank, b1, b2) appends a contact; dump(item, qi, cur,
// stk, sp) writes the frontier (cur, stk[sp-1], ..., stk[0]) as child items of `item`.
template <int PREC, int STACK, class Sink>
FCLG_HD int collide_item(const CollideLaunch& L, long long qi, int sb1, int sb2, long long item, long long budget,
                         int maxc, Sink& sink, QueryStats& st) {
  const int pi = L.pair_of_query ? FCLG_LDG(L.pair_of_query + qi) : 0;
  const int2 mp = L.pairs[pi];
  const DevMesh A = L.meshes[mp.x];
  const DevMesh B = L.meshes[mp.y];
  M3<double> R;
  V3<double> T;
  double ta[12];
  query_transform_collide(L.tf1, L.tf2, qi, R, T, ta);
  QueryF32 qf;
  if (PREC == 1) make_query_f32(R, T, A.cmax, B.cmax, A.vmax, B.vmax, qf);
  int ncont = 0;
  st.nbv = st.nleaf = st.nrecheck = 0;
  st.status = 0;
  if (maxc <= 0) return 0;
  int2 stk[STACK];
  int sp = 0;
  int b1 = sb1, b2 = sb2;
  for (;;) {
    if (st.nbv >= budget) {
      sink.dump(item, qi, make_int2(b1, b2), stk, sp);
      break;
    }
    int c1, c2;
    bool overlap;
    if (PREC == 0) {
      NodeD na, nb;
      load_nodeD(A.nodes64 + b1, na);
      load_nodeD(B.nodes64 + b2, nb);
      c1 = na.child;
      c2 = nb.child;
      overlap = obb_overlap64(R, T, na, nb);
    } else {
      const float4* pa = reinterpret_cast<const float4*>(A.nodes32) + 4 * (long long)b1;
      const float4* pb = reinterpret_cast<const float4*>(B.nodes32) + 4 * (long long)b2;
      const float4 a0 = FCLG_LDG(pa), a1 = FCLG_LDG(pa + 1), a2 = FCLG_LDG(pa + 2), ea = FCLG_LDG(pa + 3);
      const float4 x0 = FCLG_LDG(pb), x1 = FCLG_LDG(pb + 1), x2 = FCLG_LDG(pb + 2), eb = FCLG_LDG(pb + 3);
      c1 = FCLG_F2I(ea.w);
      c2 = FCLG_F2I(eb.w);
      int r = obb_overlap_f32(qf, a0, a1, a2, ea, x0, x1, x2, eb);
      if (r == F_UNSURE) {
        ++st.nrecheck;
        r = bv_overlap64(A, B, b1, b2, R, T) ? F_TRUE : F_FALSE;
      }
      overlap = (r == F_TRUE);
    }
    ++st.nbv;
    if (overlap) {
      const bool l1 = c1 < 0, l2 = c2 < 0;
      if (l1 && l2) {
        ++st.nleaf;
        const int p1 = -(c1 + 1), p2 = -(c2 + 1);
        bool hit;
        if (PREC == 0) {
          hit = leaf_collide64(A, B, p1, p2, R, T);
        } else {
          const float4* ta4 = reinterpret_cast<const float4*>(A.tri32) + 3 * (long long)p1;
          const float4* tb4 = reinterpret_cast<const float4*>(B.tri32) + 3 * (long long)p2;
          int r = tri_intersect_f32(qf, FCLG_LDG(ta4), FCLG_LDG(ta4 + 1), FCLG_LDG(ta4 + 2), FCLG_LDG(tb4),
                                    FCLG_LDG(tb4 + 1), FCLG_LDG(tb4 + 2));
          if (r == F_UNSURE) {
            ++st.nrecheck;
            r = leaf_collide64(A, B, p1, p2, R, T) ? F_TRUE : F_FALSE;
          }
          hit = (r == F_TRUE);
        }
        if (hit) {
          sink.push((int)item, ncont, p1, p2);
          ++ncont;
          if (ncont >= maxc) break;
        }
      } else {
        bool first_over_second;
        if (l2)
          first_over_second = true;
        else if (l1)
          first_over_second = false;
        else
          first_over_second = size_key(A, b1) > size_key(B, b2);
        if (sp >= STACK || (L.stack_limit > 0 && sp >= L.stack_limit)) {
          st.status |= DEV_ERR_STACK;
          break;
        }
        if (first_over_second) {
          stk[sp++] = make_int2(c1 + 1, b2);
          b1 = c1;
        } else {
          stk[sp++] = make_int2(b1, c2 + 1);
          b2 = c2;
        }
        continue;
      }
    }
    if (sp == 0) break;
    const int2 e = stk[--sp];
    b1 = e.x;
    b2 = e.y;
  }
  return ncont;
}

// Runs query qi; contacts go to sink.push(qi, rank, b1, b2).  Returns the number of
// contacts.
template <int PREC, int STACK, class Sink>
FCLG_HD int collide_query(const CollideLaunch& L, long long qi, Sink& sink, QueryStats& st) {
  const int pi = L.pair_of_query ? FCLG_LDG(L.pair_of_query + qi) : 0;
  const int2 mp = L.pairs[pi];
  const DevMesh A = L.meshes[mp.x];
  const DevMesh B = L.meshes[mp.y];
  M3<double> R;
  V3<double> T;
  double ta[12];
  query_transform_collide(L.tf1, L.tf2, qi, R, T, ta);
  QueryF32 qf;
  if (PREC == 1) make_query_f32(R, T, A.cmax, B.cmax, A.vmax, B.vmax, qf);

  const int maxc = L.num_max_contacts;
  int ncont = 0;
  st.nbv = st.nleaf = st.nrecheck = 0;
  st.status = 0;
  if (maxc <= 0) return 0;
  int2 stk[STACK];
  int sp = 0;
  int b1 = 0, b2 = 0;
  for (;;) {
    int c1, c2;
    bool overlap;
    if (PREC == 0) {
      NodeD na, nb;
      load_nodeD(A.nodes64 + b1, na);
      load_nodeD(B.nodes64 + b2, nb);
      c1 = na.child;
      c2 = nb.child;
      overlap = obb_overlap64(R, T, na, nb);
    } else {
      const float4* pa = reinterpret_cast<const float4*>(A.nodes32) + 4 * (long long)b1;
      const float4* pb = reinterpret_cast<const float4*>(B.nodes32) + 4 * (long long)b2;
      const float4 a0 = FCLG_LDG(pa), a1 = FCLG_LDG(pa + 1), a2 = FCLG_LDG(pa + 2), ea = FCLG_LDG(pa + 3);
      const float4 x0 = FCLG_LDG(pb), x1 = FCLG_LDG(pb + 1), x2 = FCLG_LDG(pb + 2), eb = FCLG_LDG(pb + 3);
      c1 = FCLG_F2I(ea.w);
      c2 = FCLG_F2I(eb.w);
      int r = obb_overlap_f32(qf, a0, a1, a2, ea, x0, x1, x2, eb);
      if (r == F_UNSURE) {
        ++st.nrecheck;
        r = bv_overlap64(A, B, b1, b2, R, T) ? F_TRUE : F_FALSE;
      }
      overlap = (r == F_TRUE);
    }
    ++st.nbv;
    if (overlap) {
      const bool l1 = c1 < 0, l2 = c2 < 0;
      if (l1 && l2) {
        ++st.nleaf;
        const int p1 = -(c1 + 1), p2 = -(c2 + 1);
        bool hit;
        if (PREC == 0) {
          hit = leaf_collide64(A, B, p1, p2, R, T);
        } else {
          const float4* ta4 = reinterpret_cast<const float4*>(A.tri32) + 3 * (long long)p1;
          const float4* tb4 = reinterpret_cast<const float4*>(B.tri32) + 3 * (long long)p2;
          int r = tri_intersect_f32(qf, FCLG_LDG(ta4), FCLG_LDG(ta4 + 1), FCLG_LDG(ta4 + 2), FCLG_LDG(tb4),
                                    FCLG_LDG(tb4 + 1), FCLG_LDG(tb4 + 2));
          if (r == F_UNSURE) {
            ++st.nrecheck;
            r = leaf_collide64(A, B, p1, p2, R, T) ? F_TRUE : F_FALSE;
          }
          hit = (r == F_TRUE);
        }
        if (hit) {
          sink.push((int)qi, ncont, p1, p2);
          ++ncont;
          if (ncont >= maxc) break;
        }
      } else {
        bool first_over_second;
        if (l2)
          first_over_second = true;
        else if (l1)
          first_over_second = false;
        else
          first_over_second = size_key(A, b1) > size_key(B, b2);
        if (sp >= STACK || (L.stack_limit > 0 && sp >= L.stack_limit)) {
          st.status |= DEV_ERR_STACK;
          break;
        }
        if (first_over_second) {
          stk[sp++] = make_int2(c1 + 1, b2);
          b1 = c1;
        } else {
          stk[sp++] = make_int2(b1, c2 + 1);
          b2 = c2;
        }
        continue;
      }
    }
    if (sp == 0) break;
    const int2 e = stk[--sp];
    b1 = e.x;
    b2 = e.y;
  }
  return ncont;
}

}  // namespace fclgpu
