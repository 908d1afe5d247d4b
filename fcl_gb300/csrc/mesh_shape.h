// Launch interface of the batched mesh-shape kernel (mesh_shape.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "fclgpu_types.h"
#include "gjk_epa.cuh"

namespace fclgpu {

struct MeshShapeLaunch {
  const DevMesh* meshes;
  const DevShape* shapes;
  const double* sverts;
  int64_t n;
  const int32_t* mesh_idx;
  const int32_t* shape_idx;
  const double* tfm;  // 12 per pair: the mesh's pose
  const double* tfs;  // 12 per pair: the shape's pose
  int32_t mode;       // 0 collide, 1 distance
  int32_t max_contacts;
  int32_t* counts;
  double* dist;
  int32_t* tri;
  double* pts;        // 6 per pair: point on the mesh, point on the shape
  int64_t* nbv;
  int64_t* nleaf;
  unsigned* status;
  // optional precomputed shape BVs: pair i uses ShapeBV bv_table[bv_src[i]] (records of
  // mesh_shape.cuh) instead of fitting its own; null = fit per pair
  const void* bv_table = nullptr;
  const int32_t* bv_src = nullptr;
  // optional early stop across pairs (collide): pairs of one group (a broadphase query)
  // add their contacts to group_count[group[i]] and stop once it reaches group_max
  const int32_t* group = nullptr;
  unsigned long long* group_count = nullptr;
  int64_t group_max = 0;
  // optional contact list (collide, split form): the intersecting triangles of every
  // pair in the order FCL's traversal adds them (Contact b1; b2 is NONE), at most
  // max_contacts per pair: offsets[n + 1] and tris[] are device arrays, tris holding
  // list_cap entries; *list_total (host) receives the total, and tris is filled only
  // when it fits
  int64_t* list_offsets = nullptr;
  int32_t* list_tris = nullptr;
  int64_t list_cap = 0;
  int64_t* list_total = nullptr;
  // optional contact geometry of the listed contacts (device, 3 / 3 / 1 doubles each)
  double* list_pos = nullptr;
  double* list_normal = nullptr;
  double* list_depth = nullptr;
  // record scratch of the list (set inside the split form)
  int4* rec = nullptr;
  unsigned long long* nrec = nullptr;
};

// One thread per pair runs the whole FCL traversal (exact statistics).
cudaError_t launch_mesh_shape(const MeshShapeLaunch& L, int stack_entries, cudaStream_t s);
// Split form, same results, no statistics (nbv / nleaf ignored).  Collide: rounds of a
// resumable per-pair DFS and one thread per leaf test, with the early stop at
// max_contacts (synchronises s once per round).  Distance: BVH traversal per pair, one
// thread per leaf test, per-pair reduction (synchronises s once).
cudaError_t run_mesh_shape_split(const MeshShapeLaunch& L, int stack_entries, cudaStream_t s);

}  // namespace fclgpu
