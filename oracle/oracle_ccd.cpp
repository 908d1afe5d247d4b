// Continuous collision of mesh pairs for the oracle (test infrastructure only):
// continuousCollideNaive (narrowphase/continuous_collision-inl.h:134-171) with
// TranslationMotion (math/motion/translation_motion-inl.h: the start rotation is held as
// a quaternion and turned back into a matrix at each step; translation start + range t).
#include <algorithm>
#include <cmath>
#include <vector>

#include "oracle_mesh.h"

namespace oracle {

void quat_from_matrix(const M3& m, double q[4]);  // oracle_refit.cpp (Eigen's Quaternion(Matrix3))
M3 matrix_from_quat(const double q[4]);           // oracle_refit.cpp (toRotationMatrix)

namespace {

// TranslationMotion(tf_beg, tf_end).integrate(dt) + getCurrentTransform
Tf translation_motion_at(const Tf& beg, const Tf& end, double dt) {
  if (dt > 1) dt = 1;
  double q[4];
  quat_from_matrix(beg.R, q);
  Tf f;
  f.R = matrix_from_quat(q);
  const V3 range = sub(end.t, beg.t);
  f.t = add(beg.t, scale(range, dt));
  return f;
}

}  // namespace

bool continuous_collide_naive(const Mesh& m1, const Tf& a0, const Tf& a1, const Mesh& m2, const Tf& b0,
                              const Tf& b1, size_t num_max_iterations, double toc_err, double& toc, Tf& ca,
                              Tf& cb) {
  size_t n_iter = std::min(num_max_iterations, (size_t)std::ceil(1 / toc_err));
  for (size_t i = 0; i < n_iter; ++i) {
    double t = i / (double)(n_iter - 1);
    Tf ta = translation_motion_at(a0, a1, t);
    Tf tb = translation_motion_at(b0, b1, t);
    std::vector<int> c;
    if (collide_mesh(m1, ta, m2, tb, 1, c, nullptr)) {
      toc = t;
      ca = ta;
      cb = tb;
      return true;
    }
  }
  toc = 1.0;
  return false;
}

}  // namespace oracle

extern "C" {
// TranslationMotion at n times (test access to the oracle's motion)
void orc_translation_motion(int64_t n, const double* beg, const double* end, const double* t, double* out) {
  using namespace oracle;
  for (int64_t i = 0; i < n; ++i) {
    Tf a, b;
    for (int r = 0; r < 3; ++r) {
      for (int c = 0; c < 3; ++c) {
        a.R(r, c) = beg[12 * i + 4 * r + c];
        b.R(r, c) = end[12 * i + 4 * r + c];
      }
      a.t[r] = beg[12 * i + 4 * r + 3];
      b.t[r] = end[12 * i + 4 * r + 3];
    }
    Tf f = translation_motion_at(a, b, t[i]);
    for (int r = 0; r < 3; ++r) {
      for (int c = 0; c < 3; ++c) out[12 * i + 4 * r + c] = f.R(r, c);
      out[12 * i + 4 * r + 3] = f.t[r];
    }
  }
}
}
