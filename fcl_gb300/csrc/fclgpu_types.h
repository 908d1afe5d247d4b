// Shared host/device layouts of the BVH store.
//
// HBM layout per mesh (all arrays indexed by FCL's node id or triangle id):
//   FP64 mirror (reference precision, read by the plain FP64 form and by rechecks)
//     NodeD  nodes64[n_nodes]   128 B: obb.axis (row-major 9), obb.To, obb.extent,
//                                     first_child (FCL encoding, BV_node_base.h:50-76)
//     RssD   rss64[n_nodes]     120 B: rss.To, rss.l[2], rss.r, rss.axis (row-major 9;
//                                     equal to obb.axis after a build, BV_fitter-inl.h:465,
//                                     different after a bottom-up refit)
//     double verts64[3*nv], int32 tris[3*nt]
//   FP32 packed store (read by the FP32 traversal)
//     float4 nodes32[4*n_nodes]  64 B: (axis col k, To[k]) k=0..2, (extent, first_child bits)
//     double size64[n_nodes]      8 B: obb extent.squaredNorm() (OBB-inl.h:205-209),
//                                     kept in FP64 so firstOverSecond is exact
//     float4 rss32[5*n_nodes]    80 B: (rss.To, r), (l0, l1, 0, 0), (rss axis col k, 0)
//     float4 tri32[3*nt]         48 B: P1 as a float pair (hi, lo), then P2-P1 and
//                                     P3-P1 rounded from FP64 differences
#pragma once
#include <stdint.h>

namespace fclgpu {

struct NodeD {
  double axis[9];  // row-major; column k is the k-th box axis
  double To[3];
  double ext[3];
  int32_t child;
  int32_t pad;
};
static_assert(sizeof(NodeD) == 128, "NodeD layout");

struct RssD {
  double To[3];
  double l[2];
  double r;
  double axis[9];  // row-major; column k is the k-th rectangle axis
};
static_assert(sizeof(RssD) == 120, "RssD layout");

// Device view of one mesh (copied into a device table; all pointers are device).
struct DevMesh {
  const NodeD* nodes64;
  const RssD* rss64;
  const double* verts64;
  const int32_t* tris;
  const void* nodes32;  // float4
  const double* size64;
  const void* rss32;    // float4
  const void* tri32;    // float4
  int32_t n_nodes;
  int32_t n_tris;
  int32_t n_verts;
  int32_t max_depth;
  double vmax;  // max |vertex coordinate|
  double cmax;  // max ||obb.To||_2
  double rmax;  // max ||rss.To||_2
  // 1 after a bottom-up refit: FCL's OBB and RSS merges need not contain the
  // children's geometry, so bounds of this mesh are not valid lower bounds
  int32_t refitted;
  int32_t pad2;
};

}  // namespace fclgpu
