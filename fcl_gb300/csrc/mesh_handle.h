// Definition of the opaque mesh handle of include/fclgpu.h (internal).
#pragma once
#include <vector>

#include "../../include/fclgpu.h"
#include "fclgpu_types.h"

struct fclgpu_mesh_s {
  fclgpu::DevMesh dev;
  fclgpu_mesh_info info;
  std::vector<void*> allocations;
  // BVHModel::computeLocalAABB (geometry/bvh/BVH_model-inl.h:1080-1100): aabb_local
  // (min, max), aabb_center, aabb_radius; and the first vertex
  double aabb_local[6];
  double aabb_center[3];
  double aabb_radius;
  double first_vertex[3];
};
