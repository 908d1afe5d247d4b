// Internal launch interface between the C ABI layer and the CUDA kernels.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

#include "fclgpu_types.h"

namespace fclgpu {

// Device status word bits (written by kernels, read by the host after a batch).
enum : uint32_t {
  DEV_ERR_STACK = 1u,     // traversal stack overflow
  DEV_ERR_RECORDS = 2u,   // contact record scratch overflow
  DEV_ERR_ITEMS = 4u,     // work-item scratch overflow
  DEV_ERR_PAIR = 8u,      // a query's pair index lies outside the pair table
  DEV_ERR_BARRIER = 16u,  // a persistent launch's grid barrier timed out
  DEV_ERR_ITERATIONS = 32u,  // a conservative-advancement query reached its iteration cap
};

// Counters shared by one batch launch (device scratch).
struct BatchCounters {
  unsigned long long work;      // next query to fetch
  unsigned long long records;   // contact-record slots reserved
  unsigned int status;          // DEV_ERR_* bits
  unsigned int pad;
  unsigned long long items;     // items allocated so far (split batches; starts at n)
  unsigned long long capped_split;
};

struct CollideLaunch {
  const DevMesh* meshes;
  const int2* pairs;
  const int32_t* pair_of_query;  // may be null (all queries use pair 0)
  const double* tf1;             // may be null (identity)
  const double* tf2;
  int64_t n;
  int32_t num_max_contacts;
  int32_t want_stats;
  BatchCounters* ctr;
  int4* records;                 // (item, rank, b1, b2)
  int64_t record_cap;
  int32_t* counts;
  int64_t* nbv;
  int64_t* nleaf;
  int64_t* nrecheck;
  // work splitting: items [item_lo, item_hi) run this round; item i < n is query i
  // at the root pair, later items are items[i] = (query, b1, b2, -)
  int4* items;
  int64_t item_cap;
  int64_t item_lo, item_hi;
  int64_t budget;                // BV tests per item per round
  int32_t wb_steps;              // FP32 form: DFS steps a lane runs between warp leaf batches
  int32_t wb_variant;            // FP32 form: 0 = unbounded registers, 1 = 128 registers
  int32_t stack_limit;           // > 0: traversal stack entries allowed, below STACK (testing)
  int32_t* own;                  // per item: contacts found by the item itself
  int32_t* child_start;          // per item: id of its first child item
  int32_t* child_count;          // per item: number of child items (0 = finished)
};

cudaError_t launch_collide_round(const CollideLaunch& L, int precision, int stack_entries, int grid, int block,
                                 cudaStream_t s);

// Control block of the persistent (one-launch) collide rounds, in device memory.  The
// host sets lo = 0, hi = n, nblocks = the grid, max_rounds, timeout_ns and zeroes the
// rest; afterwards [lo, hi) is the range still to run (empty when all rounds ran), the
// round table holds the ranges of the nrounds rounds that ran, and err has
// DEV_ERR_BARRIER if a barrier wait gave up.
struct PersistCtl {
  unsigned long long lo, hi;
  unsigned int arrive, gen;
  unsigned int nblocks, stop;
  unsigned int nrounds, max_rounds;
  unsigned long long timeout_ns;
  unsigned int err, pad;
};
constexpr unsigned long long kBarrierMaxSpins = 1ull << 32;
// One cooperative launch of all rounds of L's batch (the FP32 forms and the plain FP64
// form alike); table receives 2 x max_rounds range entries.
cudaError_t launch_collide_persistent(const CollideLaunch& L, int precision, int stack_entries, int grid,
                                      PersistCtl* ctl, int64_t* table, cudaStream_t s);
// Grid of the persistent launch (all blocks resident); 0 when cooperative launches are
// not available.
int collide_persistent_grid(int precision, int stack_entries, int variant);
cudaError_t launch_item_totals(const CollideLaunch& L, int64_t lo, int64_t hi, int64_t* total, cudaStream_t s);
// counts[q] = min(total[q], num_max_contacts); queries that were split and reached the
// cap are listed in capped[] (their statistics need the exact serial pass).
cudaError_t launch_item_counts(const CollideLaunch& L, const int64_t* total, int32_t* capped, cudaStream_t s);
cudaError_t launch_item_starts(const CollideLaunch& L, int64_t lo, int64_t hi, const int64_t* total,
                               int64_t* rel_start, cudaStream_t s);
cudaError_t launch_scatter_items(const CollideLaunch& L, int64_t nrec, const int64_t* rel_start,
                                 const int64_t* offsets, int32_t* contacts, cudaStream_t s);
// Serial exact traversal of the listed queries, statistics only (counts untouched).
cudaError_t launch_collide_stats(const CollideLaunch& L, const int32_t* list, int64_t nlist, int precision,
                                 int stack_entries, cudaStream_t s);
int collide_round_grid(int precision, int stack_entries, int block, int variant);

struct DistanceLaunch {
  const DevMesh* meshes;
  const int2* pairs;
  int32_t num_pairs;              // entries of pairs[]; a query naming another index is skipped
  const int32_t* pair_of_query;
  const double* tf1;
  const double* tf2;
  int64_t n;
  int32_t nearest;
  int32_t want_stats;
  BatchCounters* ctr;
  double* dist;
  int32_t* ids;
  double* points;
  const double* margins;
  int32_t* within;
  int64_t* nbv;
  int64_t* nleaf;
  int64_t* nrecheck;
};

// Contact information of a collide batch (enable_contact): the intersecting triangle
// pairs listed by the pair traversal, query after query (plist at poff[q]), get their
// contacts; see mesh_contact.cu.
struct ContactLaunch {
  const DevMesh* meshes;
  const int2* pairs;
  const int32_t* pair_of_query;
  const double* tf1;
  const double* tf2;
  int64_t n;                 // queries
  const int64_t* poff;       // n + 1 offsets into plist
  const int2* plist;         // (b1, b2) per intersecting triangle pair
  int64_t npairs;
  int32_t max_contacts;      // CollisionRequest::num_max_contacts
  int32_t pair_cap;          // the cap the pair traversal ran with
  int32_t* qid;              // per pair: its query
  int32_t* nc;               // per pair: contacts (0, 1 or 2)
  double* info;              // per pair: pos[2][3], normal[3], depth (world frame)
  const int64_t* G;          // npairs + 1: exclusive scan of nc
};
cudaError_t launch_contact_info(const ContactLaunch& L, cudaStream_t s);
cudaError_t launch_contact_counts(const ContactLaunch& L, const int32_t* pair_counts, int32_t* counts,
                                  unsigned int* incomplete, cudaStream_t s);
cudaError_t launch_contact_emit(const ContactLaunch& L, const int64_t* out_off, int32_t* ids, double* pos,
                                double* normal, double* depth, cudaStream_t s);

// Continuous collide (naive solver): sampled poses of every query,
// then the first colliding sample; see ccd.cu.
struct CcdLaunch {
  const int32_t* pair_of_query;
  const double* tf1_beg;     // may be null (identity at both ends)
  const double* tf1_end;
  const double* tf2_beg;
  const double* tf2_end;
  int64_t n;                 // queries
  int64_t n_iter;            // samples per query (>= 2)
  int32_t motion;            // MOTION_TRANS / MOTION_LINEAR / MOTION_SCREW (motion.cuh)
  double* tfa;               // n * n_iter sampled transforms of object 1 (12 doubles)
  double* tfb;               // ... of object 2
  int32_t* pq_expanded;      // n * n_iter pair indices
  int32_t* is_collide;
  double* toc;
  double* contact_tf1;       // may be null
  double* contact_tf2;       // may be null
  // conservative advancement (launch_ccd_ca): mesh and pair tables, the collide counts at
  // the start poses, the iteration cap and count, the status word
  const DevMesh* meshes;
  const int2* pairs;
  int32_t num_pairs;
  const int32_t* hit0;
  int64_t max_iterations;
  int32_t* iterations;       // may be null
  unsigned* status;
};
cudaError_t launch_ccd_poses(const CcdLaunch& L, cudaStream_t s);
// One thread per motion: FCL's conservative advancement with the oriented OBBRSS node.
cudaError_t launch_ccd_ca(const CcdLaunch& L, int stack_entries, cudaStream_t s);
cudaError_t launch_ccd_reduce(const CcdLaunch& L, const int32_t* counts, cudaStream_t s);

// precision: 0 = plain FP64, 1 = FP32 with FP64 recheck.  stack_entries: 64 or 256.
cudaError_t launch_mesh_collide(const CollideLaunch& L, int precision, int stack_entries, int grid, int block,
                                cudaStream_t s);
cudaError_t launch_mesh_distance(const DistanceLaunch& L, int precision, int stack_entries, int grid, int block,
                                 cudaStream_t s);
// offsets[0..n] = exclusive scan of counts (int32 -> int64), using tmp (>= 2*ceil(n/4096)+2 int64).
cudaError_t launch_exclusive_scan(const int32_t* counts, int64_t n, int64_t* offsets, int64_t* tmp, cudaStream_t s);
// contacts[offsets[q] + rank] = (b1, b2) for every valid record.
cudaError_t launch_scatter_contacts(const int4* records, int64_t nrec, const int64_t* offsets, int32_t* contacts,
                                    cudaStream_t s);
int collide_grid(int precision, int stack_entries, int block);
int distance_grid(int precision, int stack_entries, int block);

// Front-list collide (mesh_front.cu): one thread per query; the COUNT launch fills
// ncont and nseg (kept originals, kept appended entries, append list), the FILL launch
// writes contacts at cont_off, the new front at front_out_off and the statistics.
struct FrontLaunch {
  const DevMesh* meshes;
  const int2* pairs;
  int32_t num_pairs;
  const int32_t* pair_of_query;
  const double* tf1;
  const double* tf2;
  int64_t n;
  int32_t num_max_contacts;
  const int64_t* front_in_off;  // n + 1, or null (no fronts)
  const int32_t* front_in;      // (b1, b2) pairs
  int32_t* ncont;
  int32_t* nseg;                // 3 per query
  const int64_t* cont_off;
  int32_t* contacts;
  const int64_t* front_out_off;
  int32_t* front_out;
  int64_t* nbv;
  int64_t* nleaf;
  unsigned* status;
};
cudaError_t launch_collide_front(const FrontLaunch& L, int precision, int stack_entries, bool fill, cudaStream_t s);
cudaError_t launch_front_lengths(const int32_t* nseg, int64_t n, int32_t* len, cudaStream_t s);

// Device construction of an OBBRSS tree (bvh_build_device.cu), bit-identical to the host
// build: V (3 doubles per vertex) and T (3 int32 per triangle) on the device; writes the
// 2 nt - 1 nodes and RSS volumes, the internal node ids by depth (level_ids, nt - 1
// entries, offsets in level_off) and the depth of the deepest leaf.  Synchronises s.
cudaError_t build_bvh_device(const double* V, const int32_t* T, int nt, NodeD* nodes, RssD* rss,
                             std::vector<int64_t>& level_off, int32_t* level_ids, int* max_depth, cudaStream_t s);

extern int64_t g_kernel_launches;
extern double g_last_shape_ms;

}  // namespace fclgpu
