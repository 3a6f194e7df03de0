// ear_internal.h -- device-side data layout shared by the LBVH builder, the
// trace kernels and the C-ABI implementation.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "ear_math.cuh"

namespace ear {

// BVH2 node, 64 bytes, both child boxes stored in the parent so one visit
// tests two boxes with four 16-byte loads.  Child index >= 0 is an internal
// node; < 0 is a leaf: ~child = first triangle (leaf order) | (count-1) << 27.
struct __align__(32) Node {
  float4 a;  // c0.lo.x c0.hi.x c0.lo.y c0.hi.y
  float4 b;  // c0.lo.z c0.hi.z c1.lo.x c1.hi.x
  float4 c;  // c1.lo.y c1.hi.y c1.lo.z c1.hi.z
  int4 d;    // child0 child1 parent depth
};

// 4-wide node, 128 bytes, built top-down from the binary tree: a node's
// children are the up to four subtrees left after repeatedly opening the
// largest-area internal child of its binary node.  Boxes per axis for the
// four slots; a child >= 0 is an internal Node4, < 0 a leaf code as in
// Node.
struct __align__(32) Node4 {
  float4 lox, hix, loy, hiy, loz, hiz;
  int4 child;
  int4 meta;  // x: parent Node4 (-1 at the root), y: mask of occupied slots
};
// levels of the 64-bit traversal trail; a deeper 4-wide tree is not kept
// and the scene traverses its binary tree
constexpr int kMaxDepth4 = 16;

constexpr int kLeafCountShift = 27;
constexpr int kLeafStartMask = (1 << kLeafCountShift) - 1;

// Triangles in leaf order, 64 bytes each (two 32-byte loads):
//   tri[4i+0] = (v0.xyz, original index as int bits)
//   tri[4i+1] = (e1 = v1 - v0, 0), tri[4i+2] = (e2 = v2 - v0, 0)
//   tri[4i+3] = (unit normal, material id bits), read once per hit.

struct DeviceScene {
  int64_t num_tris = 0;
  int64_t num_nodes = 0;
  int max_depth = 0;
  float box_pad = 0.0f;
  int max_leaf = 1;
  int builder = 1;
  int wide = 0;  // traverse the 4-wide tree
  // order of the visibility (any-hit) tests: 0 automatic, 1 nearest hit
  // child first, 2 farthest first; any_far is the order in use
  int any_order = 0;
  int any_far = 0;
  Node* nodes = nullptr;
  Node4* nodes4 = nullptr;
  int64_t num_nodes4 = 0;
  int depth4 = 0;
  float4* tris = nullptr;
  // inputs kept on the device in file order
  float* vertices = nullptr;  // [n][9]
  int32_t* mat_ids = nullptr;
};

constexpr int kMaxRecorders = 32;
constexpr int kMaxTracks = 2 * kMaxRecorders;

struct DevMaterial {
  float survival[3];
  float p_reflect[3];
  float spec[3];
  uint32_t always_reflect;
  float refl[3];  // the MAT values, for the adjoint's score terms
  float refr[3];  // (0 when opaque)
};

struct DevRecorder {
  float loc[3];
  float right[3];
  float head_size;
  float habs[3];
  int channels;
  int track0;  // first histogram track (global over a batch)
  int job;     // batch job the recorder belongs to (0 outside batches)
  int vis_index;  // its list set in the scene's visibility maps (-1: none)
};

// One scene as the trace kernel addresses it.  A batch keeps a table of
// these in shared memory; a single render builds one from its TraceArgs.
struct __align__(16) SceneRef {
  const Node* nodes2;   // binary tree
  const Node4* nodes4;  // 4-wide tree
  const float4* tris;
  const float4* shade;  // tris + 3: shading data at stride 4
  int num_tris;
  int num_nodes;  // nodes of the tree in use
  float box_pad;
  int mat_base;  // first material of the scene in the launch's table
  int num_mats;
  int traverse_budget;
  int wide;     // 1: traverse nodes4, 0: nodes2
  int any_far;  // visibility tests visit the farthest hit child first
  // listener visibility maps of the recorders (vis_res = 0: none); a cell
  // holding more than vis_cap entries is left to the tree traversal
  const float4* vis_cells;    // 4 float4 (64 bytes) per cell (VisMap)
  const float4* vis_entries;  // kVisEntryVecs float4 per entry
  int vis_res;
  int vis_cap;
};

// One (scene, source position, recorder set) of a batch.  Its work items
// are bands x num_rays, numbered from item_end of the previous job.
struct BatchJob {
  uint64_t num_rays;
  float src[3];
  uint32_t context;
  int scene;
  int rec_base;  // first recorder in the launch's recorder table
  int num_recs;
  float inv_amount;  // 1 / (float ray count), for the finalize step
  float gain2;
  int pad[3];
};

// Everything one trace launch needs, passed by value (param space).
struct TraceArgs {
  const Node* nodes;
  const Node4* nodes4;
  int wide;
  int any_far;
  const float4* tris;
  int num_tris;
  int num_nodes;
  const DevMaterial* mats;
  int num_mats;
  const DevRecorder* recs;  // uniform index in the recorder loop
  int num_recs;
  // source
  float src[3];
  const float4* emitter;  // [n][4]: (a, area) (b, 0) (c, 0) (normal, 0)
  int num_emitter;
  float emitter_total_area;
  // rng
  uint32_t k0, k1, context;
  // work: item w -> band = bands[w / num_rays], ray = ray0 + w % num_rays
  uint64_t num_rays;
  uint64_t ray0;
  uint64_t num_items;
  int bands[3];
  int max_bounces;
  double cutoff;
  float air[3];  // 1 - air absorption, per band
  float box_pad;
  // histogram [track][band][stride]
  float* hist;
  int stride;
  int num_bins;
  int num_tracks;
  int2* first_last;  // [track][band]
  int* direct_vis;   // [recorder] direct-path visibility, or null
  // listener visibility maps of a single render's recorders (as in SceneRef)
  const float4* vis_cells;
  const float4* vis_entries;
  int vis_res;
  int vis_cap;
  // adjoint mode: upstream gradient of the raw splat sums [track][band][stride]
  // and the gradient accumulators [material][band][2 = absorption, refraction]
  const float* adj_g;
  double* adj_grad;
  // batch mode: scene and job tables, cumulative item ends per job
  const SceneRef* scenes;
  int num_scenes;
  const BatchJob* jobs;
  const uint64_t* job_end;
  int num_jobs;
  unsigned long long* counters;  // [0] work, [1] segments, [2] shadow, [3] contrib, [4] overflow
  int* error_flag;
  int traverse_budget;
  // debug
  int dbg_band;
  int dbg_max_record;
  int64_t dbg_rays;
  int32_t* dbg_hit;
  uint8_t* dbg_bt;
  uint32_t* dbg_vis;
};

enum Counter {
  kWork = 0,
  kSegments = 1,
  kShadow = 2,
  kContrib = 3,
  kOverflow = 4,
  kNodeVisits = 5,  // internal-node visits (64 B each)
  kTriTests = 6,    // Moller-Trumbore tests (48 B each)
  kSplatBins = 7,   // histogram bins written
  kMapEntries = 8,  // visibility-map entries read (8 B each)
  kNumCounters = 9
};
enum ErrorBits { kErrBudget = 1, kErrIndex = 2 };

// LBVH build (bvh_build.cu).  Returns a cudaError_t; `err` receives a
// message on failure.
// Binary BVH over the scene's triangles: builder kBuilderLbvh (Karras
// 2012; subtrees of at most max_leaf (1..16) triangles become one leaf) or
// kBuilderPloc (locally-ordered clustering within +-radius positions;
// single-triangle leaves).
enum { kBuilderLbvh = 1, kBuilderPloc = 2 };
cudaError_t build_lbvh(DeviceScene& s, float box_pad, int max_leaf, int builder, int radius,
                       cudaStream_t stream, char* err, size_t errlen);

// Listener visibility maps (vismap.cu): per recorder, a cube map of
// res x res cells per face around its location; cell c lists the triangles
// whose padded box meets the cell's cone of directions, nearest first (by
// the distance of the padded box from the recorder), as the entries from
// its cell's start to its end.  Cell index: ((recorder * 6 + face) * res +
// iv) * res + iu, face = 2 * major axis + (major component < 0).
// A visibility-list entry carries its triangle's test data inline, so a
// walk reads one array: float4 (v0, distance bits of the padded box from
// the recorder), float4 (e1 = v1 - v0, leaf position bits), float4 (e2 =
// v2 - v0, 0) -- the same floats as the triangle record, so the test gives
// the same result as the tree's.
constexpr int kVisEntryVecs = 3;
constexpr size_t kVisEntryBytes = sizeof(float) * 4 * kVisEntryVecs;
// A cell is four float4s, 64 bytes: (start bits, end bits, d1, d2), then
// its first entry (three float4s as in entries[], its distance d0 in the
// first one's w; zeros and d0 = +inf for an empty list) -- so a walk counts
// from the cell alone which of its first three entries lie nearer than the
// vertex, and tests the first while the next ones load.
constexpr int kVisCellDists = 3;
constexpr size_t kVisCellBytes = 64;
struct VisMap {
  float4* cells = nullptr;
  float4* entries = nullptr;
  int res = 0;
  int num_recs = 0;
  uint64_t num_entries = 0;
  size_t bytes = 0;
};
// Cell of the direction ratio u in [-1, 1]; monotonic in u.
__host__ __device__ __forceinline__ int vis_cell(float u, int res) {
  const int i = (int)((u + 1.0f) * (0.5f * (float)res));
  return i < 0 ? 0 : (i >= res ? res - 1 : i);
}
// Builds the maps of nrec recorder locations.  `too_large` is set (and no
// map built) when the lists would hold more than max_entries entries.
cudaError_t build_vis_map(const DeviceScene& s, const float (*locs)[3], int nrec, int res,
                          uint64_t max_entries, cudaStream_t st, VisMap* out, bool* too_large,
                          char* err, size_t errlen);
void free_vis_map(VisMap* m);

// Trace launches, one set per instantiation (trace_exact.cu, trace_fast.cu).
// kModeBatch traces many jobs (scene, source, recorders) from one work
// counter; the others trace one.
enum TraceMode { kModeForward = 0, kModeDebug = 1, kModeAdjoint = 2, kModeBatch = 3 };
constexpr int kTraceMaxBlock = 256;
struct TraceOps {
  cudaError_t (*trace)(const TraceArgs& a, int grid, int block, size_t smem, int mode,
                       cudaStream_t s);
  cudaError_t (*occupancy)(int mode, int block, size_t smem, int* blocks_per_sm);
  // blocked count of n seeded centroid -> recorder segments (occlusion probe)
  cudaError_t (*probe)(const TraceArgs& a, int n, unsigned* blocked, cudaStream_t s);
  int block;  // default block size
};
// Dynamic shared memory of a trace launch.
size_t trace_smem_bytes(int num_mats, int num_tracks, int mode, int block, int num_scenes = 0);
extern const TraceOps kTraceExact;
extern const TraceOps kTraceFast;

}  // namespace ear
