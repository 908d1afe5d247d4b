// Definition of the opaque mesh handle of include/fclgpu.h (internal).
#pragma once
#include <vector>

#include "../../include/fclgpu.h"
#include "fclgpu_types.h"

struct fclgpu_mesh_s {
  fclgpu::DevMesh dev;
  fclgpu_mesh_info info;
  std::vector<void*> allocations;
};
