// Launch interface of the convex shape-pair batch.
#pragma once
#include "gjk_epa.cuh"
#include "kernels.h"

namespace fclgpu {

struct ShapeLaunch {
  const DevShape* shapes;
  const double* verts;   // convex vertex pool
  const int32_t* ia;
  const int32_t* ib;
  const double* tf1;
  const double* tf2;
  int64_t n;
  BatchCounters* ctr;
  int32_t* hit;
  double* normal;
  double* point;
  double* depth;
  double* dist;
  double* p1;
  double* p2;
  int32_t* status;
  int32_t* order;                   // n: pair indices bucketed by (type, type)
  int32_t* epa_list;                // n: pairs whose GJK ended Inside
  unsigned long long* epa_count;     // followed by one more counter (distance work)
};

// Whole batch in stages (bucket, intersect, EPA, distance); bins: 64 unsigned scratch.
cudaError_t launch_shape_batch(const ShapeLaunch& L, unsigned* bins, cudaStream_t s);
// fcl::collide with enable_contact = false: the boolean of every pair into L.hit (no
// contact, no EPA, no distance).
cudaError_t launch_shape_collide_only(const ShapeLaunch& L, cudaStream_t s);

}  // namespace fclgpu
