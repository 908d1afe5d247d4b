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
  // bottom-up refit (fclgpu_mesh_update): internal node ids grouped by depth (level l
  // = levels[level_off[l] .. level_off[l+1]) on the device), the previous frame's
  // vertices and the magnitude-bound scratch (allocated at the first update)
  int32_t* levels = nullptr;
  std::vector<int64_t> level_off;
  void* prev_verts = nullptr;
  void* bounds = nullptr;
};
