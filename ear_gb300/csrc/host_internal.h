// host_internal.h -- host-side pieces shared by the C-ABI translation units
// (api.cu: scenes and single renders; batch.cu: batched renders and the
// autotuner): error reporting, the derived per-material / per-recorder
// constants, the scene object and the end-of-render kernels.
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "../../include/ear_gb300.h"
#include "ear_internal.h"

namespace ear {

// Thread-local message returned by ear_last_error.
extern thread_local char g_err[512];
ear_status fail(ear_status st, const char* fmt, ...);

#define CU(x)                                                                             \
  do {                                                                                    \
    cudaError_t e_ = (x);                                                                 \
    if (e_ != cudaSuccess)                                                                \
      return ::ear::fail(e_ == cudaErrorMemoryAllocation ? EAR_ERR_OUT_OF_MEMORY          \
                                                         : EAR_ERR_CUDA,                  \
                         "%s: %s", #x, cudaGetErrorString(e_));                           \
  } while (0)

// Material::Material (src/Material.cpp:26-72), per band.
bool derive_material(const ear_material& m, DevMaterial* o);

// MonoRecorder / StereoRecorder constructors (src/StereoRecorder.cpp:53-57):
// writes one DevRecorder per recorder into out[0 .. nrec-1] with tracks
// numbered from track_base; `job` is stored in each.  Returns the number of
// tracks, or -1 (with the error set) for an invalid recorder.  Writes into
// the caller's array so that the no-allocation render shares it.
int derive_recorders(const ear_recorder* recs, int nrec, int track_base, int job,
                     DevRecorder* out);

template <typename T>
cudaError_t grow(T** p, size_t* cap, size_t n) {
  if (n <= *cap && *p) return cudaSuccess;
  if (*p) cudaFree(*p);
  *p = nullptr;
  *cap = 0;
  cudaError_t e = cudaMalloc((void**)p, sizeof(T) * std::max<size_t>(n, 1));
  if (e == cudaSuccess) *cap = n;
  return e;
}

// End of Scene::Render for every (recorder, band): 1/amount scaling, the
// direct sound, gain^2.  With `jobs` set, the source, 1/amount and gain^2
// of each recorder's batch job replace the single-render values.
struct FinalizeArgs {
  float* hist;
  int stride;
  int num_bins;
  int2* first_last;
  const DevRecorder* recs;
  const int* direct_vis;  // null: no direct sound
  const BatchJob* jobs;   // null: single render
  float src[3];
  float air[3];
  float dry;
  float inv_amount;
  float gain2;
  uint32_t bands;
};

cudaError_t launch_init_first_last(int2* fl, int n, cudaStream_t st);
cudaError_t launch_finalize(const FinalizeArgs& f, int num_recorders, cudaStream_t st);

// float ray count of Scene::Render (src/Scene.cpp:122,127): exact to 2^24
// rays, then stuck at 2^24.
inline float ray_amount(uint64_t num_rays) {
  return num_rays <= 16777216ull ? (float)num_rays : 16777216.0f;
}

// Iteration budget of one traversal.  Binary tree: every node is visited
// once and climbed through at most twice.  4-wide tree: visited once,
// re-entered at most three times, climbed through at most four times.
inline int traverse_budget(int64_t num_nodes, bool wide) {
  return (int)std::min<int64_t>((wide ? 8 : 4) * num_nodes + 64, (int64_t)1 << 30);
}

// Triangle count from which a scene traverses its 4-wide tree by default
// (measured: +21% segments/s at 2,000,000 triangles, +2.5% at 20,000;
// -36% at 12, where the cheaper binary visits win).
constexpr int64_t kWideFrom = 4096;

void fill_stats(const unsigned long long* cnt, uint64_t num_items, double kernel_ms,
                ear_render_stats* stats);

// Visibility-map cells with more entries than this are left to the tree.
constexpr int kVisWalkCap = 96;

// Cells per face edge of the automatic visibility maps of a scene:
// 4 sqrt(triangles), a multiple of 64 in [64, 2816] (measured on the 2 M
// triangle nave: 1536 -> 2048 -> 2560 -> 2816 cells per edge +4.9%, +2.9%,
// +1.2%; at 2816 its nine recorders' lists hold 943 M entries, under the
// automatic limit of 2^30, which 3072 would exceed).
inline int vis_auto_res(int64_t num_tris) {
  const double r = 4.0 * std::sqrt((double)num_tris);
  return (int)std::min(2816.0, std::max(64.0, std::floor(r / 64.0) * 64.0));
}

}  // namespace ear

struct ear_scene {
  int device = 0;
  ear::DeviceScene ds;
  int num_mats = 0;
  ear::DevMaterial* mats = nullptr;
  bool bvh = false;
  int sm_count = 0;
  // render scratch, grown on demand and reused
  float* hist = nullptr;
  size_t hist_cap = 0;
  int2* fl = nullptr;
  size_t fl_cap = 0;
  unsigned long long* counters = nullptr;
  size_t counters_cap = 0;
  int* err = nullptr;
  size_t err_cap = 0;
  int* dvis = nullptr;
  size_t dvis_cap = 0;
  ear::DevRecorder* recs = nullptr;
  size_t recs_cap = 0;
  float4* emitter = nullptr;
  size_t emitter_cap = 0;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  // automatic visibility order: occlusion probe result for one recorder set
  unsigned* probe = nullptr;
  uint64_t probe_key = 0;
  bool probe_valid = false;
  // listener visibility maps of one recorder set (ear_bvh_opts.visibility_map)
  int vis_opt = 0;
  ear::VisMap vis;
  uint64_t vis_key = 0;
  bool vis_valid = false;   // `vis` (or vis_refused) belongs to vis_key
  bool vis_refused = false;  // the set's lists were above the entry limit
  uint64_t bvh_gen = 0;       // counts ear_scene_build_bvh calls (leaf order changes)
};
