// Box-box intersection with contact: the closed form GJKSolver_indep registers for a
// Box pair (gjk_solver_indep-inl.h:250, primitive_shape_algorithm/box_box-inl.h), i.e.
// the separating-axis test of the 15 box axes followed by contact generation on the
// axis of least penetration (the "dBoxBox" scheme of the Open Dynamics Engine).
//
// Same decisions as the reference, in the reference's order, because the answer
// depends on them: the face axes of box 1 then box 2 keep the first strictly deeper
// axis, the 9 edge-edge axes are preferred only when 1.05 x their depth still beats it
// (box_box-inl.h:247-250), and the edge axes see the |R| matrix padded by
// 10 eps max(1, half sides) (:380-394).  Edge-edge contact: the closest points of the
// two edges (lineClosestApproach, :60-80).  Face contact: the incident face is clipped
// against the reference face (intersectRectQuad2, :84-164) and the points with
// non-negative depth are kept.
//
// Contact choice: with num_max_contacts = 1, FCL keeps the deepest of the (at most 4,
// culled by cullPoints2) contact points; the point cullPoints2 always keeps first is
// the first point of maximal depth, and std::partial_sort with a size-1 head keeps the
// first maximum it meets, so the answer is the first clipped point of maximal depth,
// which is what box_box_intersect returns without running the cull.
#pragma once
#include "gjk_epa.cuh"

namespace fclgpu {

struct BoxBoxOut {
  int code;  // 0: separated; 1-3: face of box 1, 4-6: face of box 2, 7-15: edge pair
  int num_points;  // contact points the reference would generate before culling
  D3v normal;      // world frame, from box 1 toward box 2
  double depth;    // of the chosen point
  D3v point;       // chosen contact point, world frame
};

// Polygon clipping of the incident quad (4 points, 2D) against the rectangle
// |x| < h[0], |y| < h[1]: each of the four half-planes in the order x < h, x > -h
// (dir 0, sign -1 then +1), then the same for y; at most 8 points are kept
// (box_box-inl.h:84-164).
FCLG_HD int clip_quad_rect(const double h[2], const double quad[8], double out[16]) {
  double bufA[16], bufB[16];
  const double* q = quad;
  int nq = 4;
  double* r = bufA;
  for (int dir = 0; dir <= 1; ++dir) {
    for (int sign = -1; sign <= 1; sign += 2) {
      int nr = 0;
      for (int i = 0; i < nq; ++i) {
        const double* pq = q + 2 * i;
        const double* nx = (i + 1 < nq) ? pq + 2 : q;
        const bool in_p = sign * pq[dir] < h[dir];
        if (in_p) {
          r[2 * nr] = pq[0];
          r[2 * nr + 1] = pq[1];
          if (++nr == 8) goto full;
        }
        if (in_p != (sign * nx[dir] < h[dir])) {
          r[2 * nr + 1 - dir] = pq[1 - dir] + (nx[1 - dir] - pq[1 - dir]) / (nx[dir] - pq[dir]) * (sign * h[dir] - pq[dir]);
          r[2 * nr + dir] = sign * h[dir];
          if (++nr == 8) goto full;
        }
      }
      q = r;
      nq = nr;
      r = (r == bufA) ? bufB : bufA;
      continue;
    full:
      for (int k = 0; k < 16; ++k) out[k] = r[k];
      return 8;
    }
  }
  for (int k = 0; k < 2 * nq; ++k) out[k] = q[k];
  return nq;
}

// Closest approach of two lines pa + s ua and pb + t ub (unit directions); near
// parallel lines (1 - (ua.ub)^2 <= 1e-4) give s = t = 0.
FCLG_HD void line_closest_approach(const D3v& pa, const D3v& ua, const D3v& pb, const D3v& ub, double& s,
                                   double& t) {
  const D3v p = pb - pa;
  const double uaub = dot(ua, ub);
  const double q1 = dot(ua, p);
  const double q2 = -dot(ub, p);
  double d = 1 - uaub * uaub;
  if (d <= (double)0.0001f) {
    s = t = 0;
    return;
  }
  d = 1 / d;
  s = (q1 + uaub * q2) * d;
  t = (uaub * q1 + q2) * d;
}

FCLG_HD D3v mcol(const M3<double>& M, int j) { return v3(M(0, j), M(1, j), M(2, j)); }

// side1/side2: full side lengths; (R1, T1), (R2, T2): the boxes' poses.
FCLG_HD void box_box_contact(const double* side1, const M3<double>& R1, const D3v& T1, const double* side2,
                             const M3<double>& R2, const D3v& T2, BoxBoxOut& o) {
  o.code = 0;
  o.num_points = 0;
  const D3v p = T2 - T1;
  const D3v pp = mulTv(R1, p);
  const double ppa[3] = {pp.x, pp.y, pp.z};
  const double A[3] = {side1[0] * 0.5, side1[1] * 0.5, side1[2] * 0.5};
  const double B[3] = {side2[0] * 0.5, side2[1] * 0.5, side2[2] * 0.5};
  const M3<double> R = mulT(R1, R2);
  M3<double> Q;
  for (int k = 0; k < 9; ++k) Q.m[k] = fabs(R.m[k]);

  double s = -1.7976931348623157e308;
  int code = 0, invert = 0, best_face = -1;  // best_face: column of R1 (code 1-3) or R2 (4-6)
  D3v normalC = v3(0.0, 0.0, 0.0);

  // face axes of box 1: u_i
  for (int i = 0; i < 3; ++i) {
    const double tmp = ppa[i];
    const double s2 = fabs(tmp) - ((((Q(i, 0) * B[0] + Q(i, 1) * B[1]) + Q(i, 2) * B[2])) + A[i]);
    if (s2 > 0) return;
    if (s2 > s) {
      s = s2;
      best_face = i;
      invert = tmp < 0;
      code = 1 + i;
    }
  }
  // face axes of box 2: v_j
  for (int j = 0; j < 3; ++j) {
    const double tmp = dot(mcol(R2, j), p);
    const double s2 = fabs(tmp) - ((((Q(0, j) * A[0] + Q(1, j) * A[1]) + Q(2, j) * A[2])) + B[j]);
    if (s2 > 0) return;
    if (s2 > s) {
      s = s2;
      best_face = j;
      invert = tmp < 0;
      code = 4 + j;
    }
  }

  const double eps = 2.220446049250313e-16;
  {
    const double amax = fmax(fmax(A[0], A[1]), A[2]);
    const double bmax = fmax(fmax(B[0], B[1]), B[2]);
    const double pad = fmax(fmax(amax, bmax), 1.0) * 10.0 * eps;
    for (int k = 0; k < 9; ++k) Q.m[k] += pad;
  }

  // edge axes u_i x v_j; (c1, c2) = the cyclic successors of i, (k1, k2) = the other
  // two indices of j in ascending order
  for (int i = 0; i < 3; ++i) {
    const int c1 = (i + 1) % 3, c2 = (i + 2) % 3;
    for (int j = 0; j < 3; ++j) {
      const int k1 = j == 0 ? 1 : 0, k2 = j == 2 ? 1 : 2;
      const double tmp = ppa[c2] * R(c1, j) - ppa[c1] * R(c2, j);
      const double s2raw =
          fabs(tmp) - (((A[c1] * Q(c2, j) + A[c2] * Q(c1, j)) + B[k1] * Q(i, k2)) + B[k2] * Q(i, k1));
      if (s2raw > 0) return;
      double n[3];
      n[i] = 0;
      n[c1] = -R(c2, j);
      n[c2] = R(c1, j);
      const double l = sqrt((n[0] * n[0] + n[1] * n[1]) + n[2] * n[2]);
      if (l > eps) {
        const double s2 = s2raw / l;
        if (s2 * 1.05 > s) {
          s = s2;
          best_face = -1;
          normalC = v3(n[0] / l, n[1] / l, n[2] / l);
          invert = tmp < 0;
          code = 7 + 3 * i + j;
        }
      }
    }
  }
  if (!code) return;

  D3v normal;
  if (best_face >= 0)
    normal = mcol(code <= 3 ? R1 : R2, best_face);
  else
    normal = mulv(R1, normalC);
  if (invert) normal = d3neg(normal);
  o.code = code;
  o.normal = normal;
  const double depth = -s;

  if (code > 6) {
    // edge of box 1 against edge of box 2
    D3v pa = T1;
    for (int j = 0; j < 3; ++j) {
      const double sg = dot(mcol(R1, j), normal) > 0 ? 1.0 : -1.0;
      pa = pa + d3scale(mcol(R1, j), A[j] * sg);
    }
    D3v pb = T2;
    for (int j = 0; j < 3; ++j) {
      const double sg = dot(mcol(R2, j), normal) > 0 ? -1.0 : 1.0;
      pb = pb + d3scale(mcol(R2, j), B[j] * sg);
    }
    const D3v ua = mcol(R1, (code - 7) / 3), ub = mcol(R2, (code - 7) % 3);
    double al, be;
    line_closest_approach(pa, ua, pb, ub, al, be);
    pa = pa + d3scale(ua, al);
    pb = pb + d3scale(ub, be);
    o.point = d3scale(pa + pb, 0.5);
    o.depth = depth;
    o.num_points = 1;
    return;
  }

  // face contact: reference face on box a, incident face on box b
  const bool ref1 = code <= 3;
  const M3<double>& Ra = ref1 ? R1 : R2;
  const M3<double>& Rb = ref1 ? R2 : R1;
  const D3v& Pa = ref1 ? T1 : T2;
  const D3v& Pb = ref1 ? T2 : T1;
  const double* Sa = ref1 ? A : B;
  const double* Sb = ref1 ? B : A;
  const D3v normal2 = ref1 ? normal : d3neg(normal);
  const D3v nr = mulTv(Rb, normal2);
  const double anr[3] = {fabs(nr.x), fabs(nr.y), fabs(nr.z)};
  const double nra[3] = {nr.x, nr.y, nr.z};
  int lanr, a1, a2;
  if (anr[1] > anr[0]) {
    if (anr[1] > anr[2]) {
      a1 = 0; lanr = 1; a2 = 2;
    } else {
      a1 = 0; a2 = 1; lanr = 2;
    }
  } else {
    if (anr[0] > anr[2]) {
      lanr = 0; a1 = 1; a2 = 2;
    } else {
      a1 = 0; a2 = 1; lanr = 2;
    }
  }
  const D3v off = d3scale(mcol(Rb, lanr), Sb[lanr]);
  const D3v center = nra[lanr] < 0 ? (Pb - Pa) + off : (Pb - Pa) - off;
  const int codeN = ref1 ? code - 1 : code - 4;
  const int code1 = codeN == 0 ? 1 : 0, code2 = codeN == 2 ? 1 : 2;

  const D3v ra1 = mcol(Ra, code1), ra2 = mcol(Ra, code2);
  const D3v rb1 = mcol(Rb, a1), rb2 = mcol(Rb, a2);
  const double c1 = dot(ra1, center), c2 = dot(ra2, center);
  double m11 = dot(rb1, ra1), m12 = dot(rb2, ra1), m21 = dot(rb1, ra2), m22 = dot(rb2, ra2);
  const double k1 = m11 * Sb[a1], k2 = m21 * Sb[a1], k3 = m12 * Sb[a2], k4 = m22 * Sb[a2];
  const double quad[8] = {c1 - k1 - k3, c2 - k2 - k4, c1 - k1 + k3, c2 - k2 + k4,
                          c1 + k1 + k3, c2 + k2 + k4, c1 + k1 - k3, c2 + k2 - k4};
  const double rect[2] = {Sa[code1], Sa[code2]};
  double ret[16];
  const int nint = clip_quad_rect(rect, quad, ret);
  if (nint < 1) return;  // code stays set: FCL reports the pair colliding without contacts

  const double det1 = 1.0 / (m11 * m22 - m12 * m21);
  m11 *= det1;
  m12 *= det1;
  m21 *= det1;
  m22 *= det1;
  int cnum = 0;
  double best = 0;
  D3v best_pt = v3(0.0, 0.0, 0.0);
  for (int j = 0; j < nint; ++j) {
    const double e1 = m22 * (ret[2 * j] - c1) - m12 * (ret[2 * j + 1] - c2);
    const double e2 = -m21 * (ret[2 * j] - c1) + m11 * (ret[2 * j + 1] - c2);
    const D3v pt = (center + d3scale(rb1, e1)) + d3scale(rb2, e2);
    const double dep = Sa[codeN] - dot(normal2, pt);
    if (dep >= 0) {
      if (cnum == 0 || dep > best) {
        best = dep;
        best_pt = pt;
      }
      ++cnum;
    }
  }
  o.num_points = cnum;
  if (cnum < 1) return;
  const D3v half = d3scale(normal, best / 2);
  o.point = ref1 ? (best_pt + Pa) + half : (best_pt + Pa) - half;
  o.depth = best;
}

}  // namespace fclgpu
