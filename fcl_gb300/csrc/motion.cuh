// Motions of continuous collision (math/motion/), FP64 in the reference's operation
// order, shared by the device kernels and the test-only host build.
#pragma once
#include "refit.cuh"

namespace fclgpu {

// TranslationMotion(tf_beg, tf_end).integrate(t) + getCurrentTransform
FCLG_HD void translation_motion_at(const double* beg, const double* end, double t, double* out) {
  if (t > 1) t = 1;
  double R[9], q[4], Rq[9];
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) R[3 * r + c] = beg[4 * r + c];
  quat_from_matrix(R, q);
  matrix_from_quat(q, Rq);
  for (int r = 0; r < 3; ++r) {
    for (int c = 0; c < 3; ++c) out[4 * r + c] = Rq[3 * r + c];
    const double start = beg[4 * r + 3];
    const double range = end[4 * r + 3] - start;
    out[4 * r + 3] = start + range * t;
  }
}

}  // namespace fclgpu
