// Host BVH construction (FCL's BVHModel<OBBRSS> build) and FP32 packing.
#pragma once
#include <stdint.h>

#include <vector>

#include "fclgpu_types.h"

namespace fclgpu {

struct HostBVH {
  std::vector<NodeD> nodes;
  std::vector<RssD> rss;
  int max_depth = 0;
};

struct PackedF32 {
  std::vector<float> nodes32;  // 16 floats per node
  std::vector<double> size64;  // per node
  std::vector<float> rss32;    // 20 floats per node
  std::vector<float> tri32;    // 12 floats per triangle
  double cmax = 0.0;
  double rmax = 0.0;
};

// Returns 0 on success, -1 for an empty model.
int build_obbrss(const double* verts, int64_t nv, const int32_t* tris, int64_t nt, HostBVH& out);
void pack_fp32(const double* verts, const int32_t* tris, int64_t nt, const HostBVH& bvh, PackedF32& pk);

}  // namespace fclgpu
