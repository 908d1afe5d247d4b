// Front-list (temporal coherence) collide of BVHModel<OBBRSS> pairs: FCL's
// collide(node, front_list) (collision_node-inl.h:72-82) with a BVHFrontList
// (geometry/bvh/detail/BVH_front.h).  One thread per query.
//
// An empty front runs collisionRecurse from the roots with the list
// (traversal_recurse-inl.h:82-129): no early stop, and every leaf pair (before its
// BV test) and every disjoint BV pair is appended to the front in visit order.
//
// A non-empty front runs propagateBVHFrontListCollisionRecurse
// (traversal_recurse-inl.h:463-521).  FCL iterates its std::list while the recursion
// appends to the same list, so the entries appended there are visited later in the same
// loop.  Only the original entries generate appended entries, so the loop is two passes:
//   pass 1, the original entries in order: a leaf pair becomes invalid and runs
//     collisionRecurse into the `append` list (append it, BV test, leaf test); a non-leaf
//     pair whose BVs overlap becomes invalid and recurses into both children, appending
//     to the main list (sequence E); a disjoint pair stays;
//   pass 2, the sequence E in order: its leaf pairs become invalid and run
//     collisionRecurse into `append` again (so a leaf reached this way is tested twice,
//     as in FCL); its disjoint pairs pass their BV test again and stay.
// The new front is the kept original entries, then the kept entries of E, then
// `append`.  E is not stored: pass 2 regenerates it by repeating pass 1's recursions
// with the BV tests only (no statistics, no leaf tests), which visits the same pairs.
//
// Contacts are added while fewer than num_max_contacts exist
// (mesh_collision_traversal_node-inl.h:549-578); the traversal itself does not stop.
// Statistics count FCL's BVTesting and leafTesting calls.
//
// Two launches: COUNT computes per query the contact count and the three front
// segment lengths; the host scans them; FILL writes contacts, front and statistics.
#include <algorithm>

#include "collide_traverse.cuh"
#include "kernels.h"

namespace fclgpu {

namespace {

template <int PREC>
struct FrontQuery {
  DevMesh A, B;
  M3<double> R;
  V3<double> T;
  QueryF32 qf;
  long long nbv, nleaf;

  // BVTesting's overlap decision (exact in both forms); children ids out
  __device__ bool overlap(int b1, int b2, int& c1, int& c2) const {
    if (PREC == 0) {
      NodeD na, nb;
      load_nodeD(A.nodes64 + b1, na);
      load_nodeD(B.nodes64 + b2, nb);
      c1 = na.child;
      c2 = nb.child;
      return obb_overlap64(R, T, na, nb);
    }
    const float4* pa = reinterpret_cast<const float4*>(A.nodes32) + 4 * (long long)b1;
    const float4* pb = reinterpret_cast<const float4*>(B.nodes32) + 4 * (long long)b2;
    const float4 a0 = __ldg(pa), a1 = __ldg(pa + 1), a2 = __ldg(pa + 2), ea = __ldg(pa + 3);
    const float4 x0 = __ldg(pb), x1 = __ldg(pb + 1), x2 = __ldg(pb + 2), eb = __ldg(pb + 3);
    c1 = __float_as_int(ea.w);
    c2 = __float_as_int(eb.w);
    int r = obb_overlap_f32(qf, a0, a1, a2, ea, x0, x1, x2, eb);
    if (r == F_UNSURE) r = bv_overlap64(A, B, b1, b2, R, T) ? F_TRUE : F_FALSE;
    return r == F_TRUE;
  }
  __device__ bool leaf_hit(int p1, int p2) const {
    if (PREC == 0) return leaf_collide64(A, B, p1, p2, R, T);
    const float4* ta4 = reinterpret_cast<const float4*>(A.tri32) + 3 * (long long)p1;
    const float4* tb4 = reinterpret_cast<const float4*>(B.tri32) + 3 * (long long)p2;
    int r = tri_intersect_f32(qf, __ldg(ta4), __ldg(ta4 + 1), __ldg(ta4 + 2), __ldg(tb4), __ldg(tb4 + 1),
                              __ldg(tb4 + 2));
    if (r == F_UNSURE) r = leaf_collide64(A, B, p1, p2, R, T) ? F_TRUE : F_FALSE;
    return r == F_TRUE;
  }
  __device__ void children(int b1, int b2, int& c1, int& c2) const {
    if (PREC == 0) {
      c1 = A.nodes64[b1].child;
      c2 = B.nodes64[b2].child;
    } else {
      c1 = __float_as_int(__ldg(reinterpret_cast<const float4*>(A.nodes32) + 4 * (long long)b1 + 3).w);
      c2 = __float_as_int(__ldg(reinterpret_cast<const float4*>(B.nodes32) + 4 * (long long)b2 + 3).w);
    }
  }
  __device__ bool first_over_second(int b1, int b2, int c1, int c2) const {
    const bool l1 = c1 < 0, l2 = c2 < 0;
    if (l2) return true;
    if (l1) return false;
    return size_key(A, b1) > size_key(B, b2);
  }
};

// Output cursors of one query
template <bool FILL>
struct FrontOut {
  int maxc;
  int ncont;
  int nkeep, nkeep2, nappend;
  int2* contacts;  // FILL: this query's contact slots
  int2* keep;      // FILL: this query's front, first segment
  int2* keep2;
  int2* append;
  __device__ void contact(int p1, int p2) {
    if (ncont < maxc) {
      if (FILL) contacts[ncont] = make_int2(p1, p2);
      ++ncont;
    }
  }
  __device__ void put_keep(int b1, int b2) {
    if (FILL) keep[nkeep] = make_int2(b1, b2);
    ++nkeep;
  }
  __device__ void put_keep2(int b1, int b2) {
    if (FILL) keep2[nkeep2] = make_int2(b1, b2);
    ++nkeep2;
  }
  __device__ void put_append(int b1, int b2) {
    if (FILL) append[nappend] = make_int2(b1, b2);
    ++nappend;
  }
};

// collisionRecurse(node, sb1, sb2, list) without early stop.  MODE 0: a recursion
// whose emitted entries go to `emit` with full tests; MODE 1: the regeneration of
// pass 2 (BV tests only, leaf pairs emitted untested).  Returns false on stack overflow.
template <int PREC, int STACK, int MODE, class Emit, bool FILL>
__device__ bool recurse(FrontQuery<PREC>& q, FrontOut<FILL>& o, int sb1, int sb2, Emit emit) {
  int2 stk[STACK];
  int sp = 0;
  stk[sp++] = make_int2(sb1, sb2);
  while (sp > 0) {
    const int2 e = stk[--sp];
    const int b1 = e.x, b2 = e.y;
    int c1, c2;
    q.children(b1, b2, c1, c2);
    const bool l1 = c1 < 0, l2 = c2 < 0;
    if (l1 && l2) {
      emit(b1, b2);  // updateFrontList before the BV test
      if (MODE == 1) continue;
      ++q.nbv;
      if (!q.overlap(b1, b2, c1, c2)) continue;
      ++q.nleaf;
      if (q.leaf_hit(-(c1 + 1), -(c2 + 1))) o.contact(-(c1 + 1), -(c2 + 1));
      continue;
    }
    if (MODE == 0) ++q.nbv;
    if (!q.overlap(b1, b2, c1, c2)) {
      emit(b1, b2);
      continue;
    }
    if (sp + 2 > STACK) return false;
    // the first child's subtree is finished before the second's starts
    if (q.first_over_second(b1, b2, c1, c2)) {
      stk[sp++] = make_int2(c1 + 1, b2);
      stk[sp++] = make_int2(c1, b2);
    } else {
      stk[sp++] = make_int2(b1, c2 + 1);
      stk[sp++] = make_int2(b1, c2);
    }
  }
  return true;
}

template <int PREC, int STACK, bool FILL>
__global__ void __launch_bounds__(128) k_collide_front(const FrontLaunch L) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= L.n) return;
  const int pi = L.pair_of_query ? __ldg(L.pair_of_query + i) : 0;
  if (pi < 0 || pi >= L.num_pairs) {
    atomicOr(L.status, DEV_ERR_PAIR);
    if (!FILL) {
      L.ncont[i] = 0;
      L.nseg[3 * i] = L.nseg[3 * i + 1] = L.nseg[3 * i + 2] = 0;
    }
    return;
  }
  FrontQuery<PREC> q;
  const int2 mp = L.pairs[pi];
  q.A = L.meshes[mp.x];
  q.B = L.meshes[mp.y];
  double ta[12];
  query_transform_collide(L.tf1, L.tf2, i, q.R, q.T, ta);
  if (PREC == 1) make_query_f32(q.R, q.T, q.A.cmax, q.B.cmax, q.A.vmax, q.B.vmax, q.qf);
  q.nbv = q.nleaf = 0;
  FrontOut<FILL> o;
  o.maxc = L.num_max_contacts;
  o.ncont = o.nkeep = o.nkeep2 = o.nappend = 0;
  if (FILL) {
    o.contacts = reinterpret_cast<int2*>(L.contacts) + L.cont_off[i];
    const long long f0 = L.front_out_off[i];
    o.keep = reinterpret_cast<int2*>(L.front_out) + f0;
    o.keep2 = o.keep + L.nseg[3 * i];
    o.append = o.keep2 + L.nseg[3 * i + 1];
  }
  const long long in0 = L.front_in_off ? L.front_in_off[i] : 0;
  const long long in1 = L.front_in_off ? L.front_in_off[i + 1] : 0;
  const int2* fin = reinterpret_cast<const int2*>(L.front_in);
  bool ok = true;
  if (in1 <= in0) {
    // empty front: collisionRecurse from the roots; the whole list is emitted in order
    ok = recurse<PREC, STACK, 0>(q, o, 0, 0, [&](int b1, int b2) { o.put_keep(b1, b2); });
  } else {
    // pass 1 over the original entries
    for (long long k = in0; k < in1 && ok; ++k) {
      const int2 e = fin[k];
      int c1, c2;
      q.children(e.x, e.y, c1, c2);
      if (c1 < 0 && c2 < 0) {
        ok = recurse<PREC, STACK, 0>(q, o, e.x, e.y, [&](int b1, int b2) { o.put_append(b1, b2); });
        continue;
      }
      ++q.nbv;
      if (!q.overlap(e.x, e.y, c1, c2)) {
        o.put_keep(e.x, e.y);
        continue;
      }
      const bool fos = q.first_over_second(e.x, e.y, c1, c2);
      const int2 s0 = fos ? make_int2(c1, e.y) : make_int2(e.x, c2);
      const int2 s1 = fos ? make_int2(c1 + 1, e.y) : make_int2(e.x, c2 + 1);
      auto to_main = [&](int, int) {};  // sequence E: regenerated in pass 2
      ok = recurse<PREC, STACK, 0>(q, o, s0.x, s0.y, to_main) && recurse<PREC, STACK, 0>(q, o, s1.x, s1.y, to_main);
    }
    // pass 2 over E, regenerated entry by entry
    auto visit = [&](int b1, int b2) {
      int c1, c2;
      q.children(b1, b2, c1, c2);
      if (c1 < 0 && c2 < 0) {
        o.put_append(b1, b2);
        ++q.nbv;
        if (q.overlap(b1, b2, c1, c2)) {
          ++q.nleaf;
          if (q.leaf_hit(-(c1 + 1), -(c2 + 1))) o.contact(-(c1 + 1), -(c2 + 1));
        }
      } else {
        ++q.nbv;  // disjoint when emitted, disjoint again at the same pose
        o.put_keep2(b1, b2);
      }
    };
    for (long long k = in0; k < in1 && ok; ++k) {
      const int2 e = fin[k];
      int c1, c2;
      q.children(e.x, e.y, c1, c2);
      if (c1 < 0 && c2 < 0) continue;
      if (!q.overlap(e.x, e.y, c1, c2)) continue;
      const bool fos = q.first_over_second(e.x, e.y, c1, c2);
      const int2 s0 = fos ? make_int2(c1, e.y) : make_int2(e.x, c2);
      const int2 s1 = fos ? make_int2(c1 + 1, e.y) : make_int2(e.x, c2 + 1);
      ok = recurse<PREC, STACK, 1>(q, o, s0.x, s0.y, visit) && recurse<PREC, STACK, 1>(q, o, s1.x, s1.y, visit);
    }
  }
  if (!ok) {
    atomicOr(L.status, DEV_ERR_STACK);
    if (FILL) return;
    o.ncont = o.nkeep = o.nkeep2 = o.nappend = 0;
  }
  if (!FILL) {
    L.ncont[i] = o.ncont;
    L.nseg[3 * i] = o.nkeep;
    L.nseg[3 * i + 1] = o.nkeep2;
    L.nseg[3 * i + 2] = o.nappend;
  } else {
    if (L.nbv) L.nbv[i] = q.nbv;
    if (L.nleaf) L.nleaf[i] = q.nleaf;
  }
}

// per query: front length = the three segments
__global__ void k_front_lengths(const int32_t* nseg, long long n, int32_t* len) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) len[i] = nseg[3 * i] + nseg[3 * i + 1] + nseg[3 * i + 2];
}

template <bool FILL>
cudaError_t launch_front_t(const FrontLaunch& L, int precision, int stack_entries, cudaStream_t s) {
  const unsigned grid = (unsigned)((L.n + 127) / 128);
  if (precision == 0) {
    if (stack_entries <= 64)
      k_collide_front<0, 64, FILL><<<grid, 128, 0, s>>>(L);
    else
      k_collide_front<0, 256, FILL><<<grid, 128, 0, s>>>(L);
  } else {
    if (stack_entries <= 64)
      k_collide_front<1, 64, FILL><<<grid, 128, 0, s>>>(L);
    else
      k_collide_front<1, 256, FILL><<<grid, 128, 0, s>>>(L);
  }
  ++g_kernel_launches;
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_collide_front(const FrontLaunch& L, int precision, int stack_entries, bool fill, cudaStream_t s) {
  if (L.n <= 0) return cudaSuccess;
  return fill ? launch_front_t<true>(L, precision, stack_entries, s)
              : launch_front_t<false>(L, precision, stack_entries, s);
}

cudaError_t launch_front_lengths(const int32_t* nseg, int64_t n, int32_t* len, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_front_lengths<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(nseg, n, len);
  ++g_kernel_launches;
  return cudaGetLastError();
}

}  // namespace fclgpu
