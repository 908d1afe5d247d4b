// Definition of the opaque shape-set handle of include/fclgpu.h (internal).
#pragma once
#include <string>
#include <vector>

#include "../../include/fclgpu.h"
#include "gjk_epa.cuh"

struct fclgpu_shapeset_s {
  fclgpu::DevShape* shapes = nullptr;
  double* verts = nullptr;
  int32_t n = 0;
  int64_t nv = 0;
  std::vector<fclgpu::DevShape> host;  // host copies, for world-AABB records
  std::vector<double> host_verts;
};

namespace fclgpu {
// Sets the text fclgpu_last_error_detail() returns on this thread.
void set_error_detail(const std::string& what);
}  // namespace fclgpu
