// batch.cu -- batched rendering and the schedule autotuner (C ABI in
// include/ear_gb300.h, "batches").
//
// A batch is a sweep of renders -- rooms x source/listener pairs x
// keyframes -- planned once: the jobs' recorders are derived as for
// ear_render, every (job, track, band) gets one histogram row, and the
// work of all jobs (bands x rays each) is numbered consecutively so one
// persistent trace launch (kModeBatch) drains it from a device counter.
// A run is a fixed sequence -- clear, refresh the material tables, trace,
// finalize -- captured once into a CUDA graph and replayed.
//
// The autotuner times trial launches (every job with a fraction of its
// rays) over block size x resident blocks per SM (x BVH leaf size) and
// keeps the fastest; results can be cached in a text file keyed by the
// device and the batch's shape.

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/ear_gb300.h"
#include "ear_internal.h"
#include "host_internal.h"

using namespace ear;

struct ear_batch {
  int device = 0;
  int sm_count = 0;
  std::vector<ear_scene*> scenes;
  std::vector<BatchJob> jobs;          // host copy of the job table
  std::vector<uint64_t> job_end;       // cumulative work items
  std::vector<int> first_track;        // per job
  std::vector<int> tracks;             // per job
  std::vector<DevRecorder> recs;
  std::vector<int> mat_base;           // per scene
  int total_mats = 0;
  int total_tracks = 0;
  ear_render_params params{};
  TraceArgs a{};
  const TraceOps* ops = nullptr;
  ear_batch_config cfg{};
  // device
  SceneRef* d_scenes = nullptr;
  std::vector<SceneRef> h_scenes;      // what d_scenes holds
  BatchJob* d_jobs = nullptr;
  uint64_t* d_job_end = nullptr;
  DevRecorder* d_recs = nullptr;
  DevMaterial* d_mats = nullptr;
  float* d_hist = nullptr;
  int2* d_fl = nullptr;
  int* d_dvis = nullptr;
  unsigned long long* d_counters = nullptr;
  int* d_err = nullptr;
  // trial tables for the autotuner (fewer rays per job)
  BatchJob* d_trial_jobs = nullptr;
  uint64_t* d_trial_end = nullptr;
  // launch
  cudaStream_t cap_stream = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  // listener visibility maps, one per scene over the distinct recorder
  // locations of its jobs, and the tree generation / setting they follow
  std::vector<VisMap> maps;
  std::vector<uint64_t> map_gen;
  std::vector<int> map_opt;
  double map_build_ms = 0.0;  // spent since the last run
  // results of the last run
  std::vector<int2> fl;
  bool ran = false;
};

namespace {

size_t hist_stride(int num_bins) { return (size_t)((num_bins + 3) & ~3); }

void free_graph(ear_batch* b) {
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  b->exec = nullptr;
  b->graph = nullptr;
}

SceneRef scene_ref(const ear_scene* s, int mat_base, const VisMap& m) {
  SceneRef r;
  std::memset(&r, 0, sizeof r);  // the table is compared bytewise
  r.nodes2 = s->ds.nodes;
  r.nodes4 = s->ds.nodes4;
  r.wide = s->ds.wide;
  r.any_far = s->ds.any_far;
  r.tris = s->ds.tris;
  r.shade = s->ds.tris ? s->ds.tris + 3 : nullptr;
  r.num_tris = (int)s->ds.num_tris;
  r.num_nodes = (int)(s->ds.wide ? s->ds.num_nodes4 : s->ds.num_nodes);
  r.box_pad = s->ds.box_pad;
  r.mat_base = mat_base;
  r.num_mats = s->num_mats;
  r.traverse_budget = traverse_budget(s->ds.wide ? s->ds.num_nodes4 : s->ds.num_nodes, s->ds.wide != 0);
  r.vis_cells = m.cells;
  r.vis_entries = m.entries;
  r.vis_res = m.cells ? m.res : 0;
  r.vis_cap = kVisWalkCap;
  return r;
}

// Most cells of one scene's automatic maps in a batch (256 MiB of list
// starts): the resolution drops as the scene's recorder count grows.
constexpr uint64_t kBatchMapCells = 1ull << 26;

// (Re)builds the visibility maps of the scenes whose tree or setting
// changed: one map per scene over the distinct locations of its jobs'
// recorders (more than kMaxRecorders keep the tree).  Automatic setting:
// when the scene's jobs trace at least as many paths as it has
// triangles, at the single-render resolution capped by kBatchMapCells and
// lowered while the lists exceed EAR_VISMAP_AUTO_MAX_ENTRIES.  Each
// recorder's vis_index names its list set (-1: no map).
ear_status build_batch_maps(ear_batch* b) {
  const size_t ns = b->scenes.size();
  b->maps.resize(ns);
  b->map_gen.resize(ns, ~0ull);
  b->map_opt.resize(ns, 0);
  int nb = 0;
  for (int k = 0; k < 3; ++k) nb += (b->params.bands_mask >> k) & 1;
  bool recs_changed = false;
  cudaStream_t st = (cudaStream_t)b->params.stream;
  for (size_t i = 0; i < ns; ++i) {
    ear_scene* s = b->scenes[i];
    if (b->map_gen[i] == s->bvh_gen && b->map_opt[i] == s->vis_opt) continue;
    free_vis_map(&b->maps[i]);
    b->map_gen[i] = s->bvh_gen;
    b->map_opt[i] = s->vis_opt;
    recs_changed = true;
    std::vector<float> locs;  // distinct locations, 3 floats each
    std::vector<int> index(b->recs.size(), -1);
    uint64_t work = 0;
    for (const BatchJob& j : b->jobs) {
      if ((size_t)j.scene != i) continue;
      work += j.num_rays * (uint64_t)nb;
      for (int r = j.rec_base; r < j.rec_base + j.num_recs; ++r) {
        const float* l = b->recs[(size_t)r].loc;
        size_t k = 0;
        while (k < locs.size() / 3 && std::memcmp(&locs[3 * k], l, 3 * sizeof(float)) != 0) ++k;
        if (k == locs.size() / 3) locs.insert(locs.end(), l, l + 3);
        index[(size_t)r] = (int)k;
      }
    }
    const int nloc = (int)(locs.size() / 3);
    const bool automatic = s->vis_opt == 0;
    int res = automatic ? vis_auto_res(s->ds.num_tris) : s->vis_opt;
    bool use = s->vis_opt >= 0 && nloc > 0 && nloc <= kMaxRecorders && s->ds.num_tris > 0;
    if (automatic) {
      use = use && work >= (uint64_t)s->ds.num_tris;
      const int cap = (int)std::sqrt((double)kBatchMapCells / (6.0 * std::max(nloc, 1)));
      res = std::max(8, std::min(res, cap / 32 * 32));
    }
    if (use) {
      size_t free_b = 0, total_b = 0;
      CU(cudaMemGetInfo(&free_b, &total_b));
      const uint64_t fit = (uint64_t)(free_b / 2) / (24 + kVisEntryBytes + kVisCellBytes);
      const uint64_t limit = std::min<uint64_t>(
          automatic ? (uint64_t)EAR_VISMAP_AUTO_MAX_ENTRIES : (1ull << 31) - 1, fit);
      char msg[256] = "";
      bool too_large = false;
      CU(cudaEventRecord(b->ev0, st));
      for (;;) {
        const cudaError_t e = build_vis_map(s->ds, reinterpret_cast<const float(*)[3]>(locs.data()),
                                            nloc, res, limit, st, &b->maps[i], &too_large, msg,
                                            sizeof msg);
        if (e == cudaErrorMemoryAllocation && automatic) {
          // the automatic maps are an accelerator: without room the tree serves
          cudaGetLastError();
          too_large = true;
          break;
        }
        if (e != cudaSuccess)
          return fail(e == cudaErrorMemoryAllocation ? EAR_ERR_OUT_OF_MEMORY : EAR_ERR_CUDA,
                      "batch visibility map build (scene %zu): %s", i,
                      msg[0] ? msg : cudaGetErrorString(e));
        if (!too_large || !automatic || res <= 64) break;
        res = std::max(64, (res * 3 / 4) / 32 * 32);
      }
      CU(cudaEventRecord(b->ev1, st));
      CU(cudaEventSynchronize(b->ev1));
      float ms = 0.0f;
      CU(cudaEventElapsedTime(&ms, b->ev0, b->ev1));
      b->map_build_ms += ms;
      use = !too_large;
    }
    for (size_t r = 0; r < b->recs.size(); ++r)
      if (b->jobs[(size_t)b->recs[r].job].scene == (int)i) b->recs[r].vis_index = use ? index[r] : -1;
  }
  if (recs_changed && !b->recs.empty())
    CU(cudaMemcpy(b->d_recs, b->recs.data(), sizeof(DevRecorder) * b->recs.size(), cudaMemcpyHostToDevice));
  return EAR_OK;
}

// Re-reads the scenes' device pointers (a BVH rebuild replaces them) and
// their visibility maps; a change re-uploads the scene table and drops the
// captured graph.
ear_status sync_scenes(ear_batch* b) {
  ear_status rc = build_batch_maps(b);
  if (rc != EAR_OK) return rc;
  std::vector<SceneRef> now(b->scenes.size());
  for (size_t i = 0; i < b->scenes.size(); ++i) {
    if (!b->scenes[i]->bvh) return fail(EAR_ERR_STATE, "batch scene %zu has no LBVH", i);
    now[i] = scene_ref(b->scenes[i], b->mat_base[i], b->maps[i]);
  }
  if (!b->h_scenes.empty() && std::memcmp(now.data(), b->h_scenes.data(), sizeof(SceneRef) * now.size()) == 0)
    return EAR_OK;
  CU(cudaMemcpy(b->d_scenes, now.data(), sizeof(SceneRef) * now.size(), cudaMemcpyHostToDevice));
  b->h_scenes = now;
  free_graph(b);
  return EAR_OK;
}

struct Schedule {
  int block;
  int grid;
  size_t smem;
};

ear_status schedule(ear_batch* b, const ear_batch_config& c, Schedule* out) {
  const int block = c.block > 0 ? c.block : b->ops->block;
  if (block < 32 || block > kTraceMaxBlock || block % 32)
    return fail(EAR_ERR_INVALID_ARG, "block must be a multiple of 32 in [32, %d]", kTraceMaxBlock);
  const size_t smem = trace_smem_bytes(b->total_mats, 0, kModeBatch, block, (int)b->scenes.size());
  int per_sm = 0;
  CU(b->ops->occupancy(kModeBatch, block, smem, &per_sm));
  if (per_sm < 1) return fail(EAR_ERR_UNSUPPORTED, "the batch's tables do not fit one block");
  if (c.blocks_per_sm > 0) per_sm = std::min(per_sm, c.blocks_per_sm);
  out->block = block;
  out->grid = b->sm_count * per_sm;
  out->smem = smem;
  return EAR_OK;
}

// The scenes' current materials into the batch's table
// (ear_scene_set_materials may change them between runs).
cudaError_t refresh_materials(ear_batch* b, cudaStream_t st) {
  cudaError_t e = cudaSuccess;
  for (size_t i = 0; i < b->scenes.size() && e == cudaSuccess; ++i)
    if (b->scenes[i]->num_mats)
      e = cudaMemcpyAsync(b->d_mats + b->mat_base[i], b->scenes[i]->mats,
                          sizeof(DevMaterial) * b->scenes[i]->num_mats, cudaMemcpyDeviceToDevice, st);
  return e;
}

// The launch sequence of one run on stream st.
cudaError_t enqueue(ear_batch* b, const Schedule& sc, const TraceArgs& a, cudaStream_t st) {
  const size_t stride = hist_stride(b->params.num_bins);
  const size_t rows = (size_t)b->total_tracks * 3;
  cudaError_t e = cudaMemsetAsync(b->d_hist, 0, sizeof(float) * std::max<size_t>(rows, 1) * stride, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(b->d_counters, 0, sizeof(unsigned long long) * kNumCounters, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(b->d_err, 0, sizeof(int), st);
  if (e == cudaSuccess) e = refresh_materials(b, st);
  if (e == cudaSuccess) e = launch_init_first_last(b->d_fl, (int)rows, st);
  if (e == cudaSuccess && a.num_items > 0) e = b->ops->trace(a, sc.grid, sc.block, sc.smem, kModeBatch, st);
  if (e == cudaSuccess && !(b->params.flags & EAR_FLAG_RAW)) {
    FinalizeArgs f = {};
    f.hist = b->d_hist;
    f.stride = (int)stride;
    f.num_bins = b->params.num_bins;
    f.first_last = b->d_fl;
    f.recs = b->d_recs;
    f.direct_vis = a.direct_vis;
    f.jobs = b->d_jobs;
    for (int k = 0; k < 3; ++k) f.air[k] = a.air[k];
    f.dry = b->params.dry_level;
    f.bands = b->params.bands_mask;
    e = launch_finalize(f, (int)b->recs.size(), st);
  }
  return e;
}

ear_status check_errors(ear_batch* b) {
  int errflag = 0;
  CU(cudaMemcpy(&errflag, b->d_err, sizeof(int), cudaMemcpyDeviceToHost));
  if (errflag & kErrIndex)
    return fail(EAR_ERR_CUDA, "internal: a device-side index check failed (corrupt BVH or scene data)");
  if (errflag & kErrBudget)
    return fail(EAR_ERR_DEVICE_BUDGET, "a BVH traversal exceeded its iteration budget");
  return EAR_OK;
}

// Trial launch for the autotuner: the trace kernel alone over the trial
// job table, timed with events on the batch's stream.
ear_status trial(ear_batch* b, const ear_batch_config& c, uint64_t trial_items, float* ms) {
  Schedule sc;
  ear_status rc = schedule(b, c, &sc);
  if (rc != EAR_OK) return rc;
  rc = sync_scenes(b);
  if (rc != EAR_OK) return rc;
  cudaStream_t st = (cudaStream_t)b->params.stream;
  TraceArgs a = b->a;
  a.jobs = b->d_trial_jobs;
  a.job_end = b->d_trial_end;
  a.num_items = trial_items;
  a.direct_vis = nullptr;
  const size_t stride = hist_stride(b->params.num_bins);
  const size_t rows = (size_t)b->total_tracks * 3;
  CU(cudaMemsetAsync(b->d_counters, 0, sizeof(unsigned long long) * kNumCounters, st));
  CU(cudaMemsetAsync(b->d_err, 0, sizeof(int), st));
  CU(cudaMemsetAsync(b->d_hist, 0, sizeof(float) * std::max<size_t>(rows, 1) * stride, st));
  CU(refresh_materials(b, st));
  CU(launch_init_first_last(b->d_fl, (int)rows, st));
  CU(cudaEventRecord(b->ev0, st));
  CU(b->ops->trace(a, sc.grid, sc.block, sc.smem, kModeBatch, st));
  CU(cudaEventRecord(b->ev1, st));
  CU(cudaStreamSynchronize(st));
  rc = check_errors(b);
  if (rc != EAR_OK) return rc;
  CU(cudaEventElapsedTime(ms, b->ev0, b->ev1));
  b->ran = false;  // the histograms now hold trial data
  return EAR_OK;
}

std::string tune_key(const ear_batch* b, bool leaf, bool width) {
  cudaDeviceProp prop;
  cudaGetDeviceProperties(&prop, b->device);
  uint64_t tris = 0, rays = 0;
  for (const ear_scene* s : b->scenes) tris += (uint64_t)s->ds.num_tris;
  for (const BatchJob& j : b->jobs) rays += j.num_rays;
  // shape buckets: powers of two of triangles and rays
  auto lg = [](uint64_t x) { return x ? 64 - __builtin_clzll(x) : 0; };
  std::ostringstream k;
  k << "sm" << prop.major << prop.minor << "x" << b->sm_count << ":scenes" << b->scenes.size()
    << ":jobs" << lg((uint64_t)b->jobs.size()) << ":tris" << lg(tris) << ":rays" << lg(rays)
    << ":mats" << b->total_mats << ":rec" << b->recs.size() << ":bands" << b->params.bands_mask
    << ":exact" << ((b->params.flags & EAR_FLAG_EXACT) ? 1 : 0) << ":leaf" << (leaf ? 1 : 0)
    << ":width" << (width ? 1 : 0);
  return k.str();
}

bool cache_lookup(const char* path, const std::string& key, ear_batch_config* c, float* ms) {
  if (!path) return false;
  std::ifstream in(path);
  std::string line;
  bool found = false;
  while (std::getline(in, line)) {
    std::istringstream ls(line);
    std::string k;
    ear_batch_config t{};
    float m = 0.0f;
    if (ls >> k >> t.block >> t.blocks_per_sm >> t.max_leaf_size >> t.bvh_width >> m && k == key) {
      *c = t;
      *ms = m;
      found = true;  // the last entry for a key wins
    }
  }
  return found;
}

void cache_store(const char* path, const std::string& key, const ear_batch_config& c, float ms) {
  if (!path) return;
  std::ofstream out(path, std::ios::app);
  out << key << " " << c.block << " " << c.blocks_per_sm << " " << c.max_leaf_size << " "
      << c.bvh_width << " " << ms << "\n";
}

ear_status set_width(ear_batch* b, int width) {
  for (ear_scene* s : b->scenes) {
    // a scene without a 4-wide tree (deeper than its trail) stays binary
    const ear_status rc = ear_scene_set_bvh_width(s, width == 4 && !s->ds.nodes4 ? 2 : width);
    if (rc != EAR_OK) return rc;
  }
  return sync_scenes(b);
}

ear_status rebuild_scenes(ear_batch* b, int leaf) {
  for (ear_scene* s : b->scenes) {
    if (s->ds.max_leaf == leaf || s->ds.builder == kBuilderPloc) continue;
    ear_bvh_opts o;
    std::memset(&o, 0, sizeof o);
    o.box_pad = s->ds.box_pad;  // keep the padding the scene was built with
    o.max_leaf_size = leaf;
    o.builder = EAR_BVH_LBVH;
    o.visibility_order = s->ds.any_order;
    o.visibility_map = s->vis_opt;
    const ear_status rc = ear_scene_build_bvh(s, &o);
    if (rc != EAR_OK) return rc;
  }
  return sync_scenes(b);
}

}  // namespace

extern "C" {

ear_status ear_batch_create(ear_scene* const* scenes, int32_t num_scenes, const ear_batch_job* jobs,
                            int32_t num_jobs, const ear_render_params* p, ear_batch** out) {
  g_err[0] = 0;
  if (!scenes || !jobs || !p || !out) return fail(EAR_ERR_INVALID_ARG, "null argument");
  *out = nullptr;
  if (num_scenes <= 0 || num_jobs <= 0) return fail(EAR_ERR_INVALID_ARG, "empty batch");
  if (num_scenes > 1024) return fail(EAR_ERR_INVALID_ARG, "at most 1024 scenes per batch");
  if (p->num_bins <= 0 || p->num_bins > (1 << 30)) return fail(EAR_ERR_INVALID_ARG, "bad num_bins");
  if (p->bands_mask == 0 || (p->bands_mask & ~7u)) return fail(EAR_ERR_INVALID_ARG, "bad bands_mask");
  if (p->max_bounces < 0) return fail(EAR_ERR_INVALID_ARG, "negative max_bounces");
  const int device = scenes[0] ? scenes[0]->device : 0;
  int total_mats = 0;
  std::vector<int> mat_base((size_t)num_scenes);
  for (int i = 0; i < num_scenes; ++i) {
    if (!scenes[i]) return fail(EAR_ERR_INVALID_ARG, "scene %d is null", i);
    if (!scenes[i]->bvh) return fail(EAR_ERR_STATE, "scene %d: ear_scene_build_bvh has not been called", i);
    if (scenes[i]->device != device) return fail(EAR_ERR_INVALID_ARG, "the batch's scenes are on different devices");
    mat_base[(size_t)i] = total_mats;
    total_mats += scenes[i]->num_mats;
  }
  if (total_mats > 1024) return fail(EAR_ERR_UNSUPPORTED, "at most 1024 materials over a batch's scenes");
  int nb = 0;
  for (int b = 0; b < 3; ++b) nb += (p->bands_mask >> b) & 1;

  ear_batch* b = new ear_batch();
  b->device = device;
  b->scenes.assign(scenes, scenes + num_scenes);
  b->mat_base = mat_base;
  b->total_mats = total_mats;
  b->params = *p;
  b->ops = (p->flags & EAR_FLAG_EXACT) ? &kTraceExact : &kTraceFast;
  uint64_t items = 0;
  int tracks = 0;
  for (int j = 0; j < num_jobs; ++j) {
    const ear_batch_job& J = jobs[j];
    if (J.scene < 0 || J.scene >= num_scenes || J.num_recorders < 1 || J.num_recorders > kMaxRecorders ||
        !J.recorders || J.num_rays == 0 || J.num_rays > (1ull << 47)) {
      delete b;
      return fail(EAR_ERR_INVALID_ARG, "job %d: bad scene, recorders or ray count", j);
    }
    BatchJob d;
    std::memset(&d, 0, sizeof d);
    d.num_rays = J.num_rays;
    for (int k = 0; k < 3; ++k) d.src[k] = J.source[k];
    d.context = J.context;
    d.scene = J.scene;
    d.rec_base = (int)b->recs.size();
    d.num_recs = J.num_recorders;
    d.inv_amount = 1.0f / ray_amount(J.num_rays);
    d.gain2 = J.gain * J.gain;
    const size_t rbase = b->recs.size();
    b->recs.resize(rbase + (size_t)std::max(0, J.num_recorders));
    const int t = derive_recorders(J.recorders, J.num_recorders, tracks, j, b->recs.data() + rbase);
    if (t < 0) {
      delete b;
      return EAR_ERR_INVALID_ARG;
    }
    b->first_track.push_back(tracks);
    b->tracks.push_back(t);
    tracks += t;
    items += J.num_rays * (uint64_t)nb;
    b->jobs.push_back(d);
    b->job_end.push_back(items);
  }
  b->total_tracks = tracks;
  const size_t rows = (size_t)tracks * 3;
  const size_t stride = hist_stride(p->num_bins);
  if ((double)rows * (double)stride > 9.0e18 / 4.0) {
    delete b;
    return fail(EAR_ERR_INVALID_ARG, "batch histograms too large");
  }

  cudaError_t e = cudaSetDevice(device);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&b->sm_count, cudaDevAttrMultiProcessorCount, device);
  const size_t nj = b->jobs.size(), nr = b->recs.size();
  if (e == cudaSuccess) e = cudaMalloc(&b->d_scenes, sizeof(SceneRef) * (size_t)num_scenes);
  if (e == cudaSuccess) e = cudaMalloc(&b->d_jobs, sizeof(BatchJob) * nj);
  if (e == cudaSuccess) e = cudaMalloc(&b->d_job_end, sizeof(uint64_t) * nj);
  if (e == cudaSuccess) e = cudaMalloc(&b->d_trial_jobs, sizeof(BatchJob) * nj);
  if (e == cudaSuccess) e = cudaMalloc(&b->d_trial_end, sizeof(uint64_t) * nj);
  if (e == cudaSuccess) e = cudaMalloc(&b->d_recs, sizeof(DevRecorder) * nr);
  if (e == cudaSuccess) e = cudaMalloc(&b->d_mats, sizeof(DevMaterial) * (size_t)std::max(total_mats, 1));
  if (e == cudaSuccess) e = cudaMalloc(&b->d_hist, sizeof(float) * std::max<size_t>(rows, 1) * stride);
  if (e == cudaSuccess) e = cudaMalloc(&b->d_fl, sizeof(int2) * std::max<size_t>(rows, 1));
  if (e == cudaSuccess) e = cudaMalloc(&b->d_dvis, sizeof(int) * nr);
  if (e == cudaSuccess) e = cudaMalloc(&b->d_counters, sizeof(unsigned long long) * kNumCounters);
  if (e == cudaSuccess) e = cudaMalloc(&b->d_err, sizeof(int));
  if (e == cudaSuccess)
    e = cudaMemcpy(b->d_jobs, b->jobs.data(), sizeof(BatchJob) * nj, cudaMemcpyHostToDevice);
  if (e == cudaSuccess)
    e = cudaMemcpy(b->d_job_end, b->job_end.data(), sizeof(uint64_t) * nj, cudaMemcpyHostToDevice);
  if (e == cudaSuccess)
    e = cudaMemcpy(b->d_recs, b->recs.data(), sizeof(DevRecorder) * nr, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->cap_stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreate(&b->ev0);
  if (e == cudaSuccess) e = cudaEventCreate(&b->ev1);
  if (e != cudaSuccess) {
    ear_batch_destroy(b);
    return fail(e == cudaErrorMemoryAllocation ? EAR_ERR_OUT_OF_MEMORY : EAR_ERR_CUDA,
                "batch allocation: %s", cudaGetErrorString(e));
  }
  ear_status rc = sync_scenes(b);
  if (rc != EAR_OK) {
    ear_batch_destroy(b);
    return rc;
  }

  TraceArgs& a = b->a;
  std::memset(&a, 0, sizeof a);
  a.mats = b->d_mats;
  a.num_mats = total_mats;
  a.recs = b->d_recs;
  a.num_recs = (int)nr;
  a.k0 = (uint32_t)p->seed;
  a.k1 = (uint32_t)(p->seed >> 32);
  int k = 0;
  for (int band = 0; band < 3; ++band) {
    a.bands[band] = -1;
    if (p->bands_mask & (1u << band)) a.bands[k++] = band;
    a.air[band] = 1.0f - p->air_absorption[band];
  }
  a.num_rays = 0;
  a.num_items = items;
  a.max_bounces = p->max_bounces;
  a.cutoff = p->cutoff;
  a.hist = b->d_hist;
  a.stride = (int)stride;
  a.num_bins = p->num_bins;
  a.num_tracks = tracks;
  a.first_last = b->d_fl;
  const bool direct = !(p->flags & (EAR_FLAG_RAW | EAR_FLAG_NO_DIRECT));
  a.direct_vis = direct ? b->d_dvis : nullptr;
  a.counters = b->d_counters;
  a.error_flag = b->d_err;
  a.dbg_band = -1;
  a.scenes = b->d_scenes;
  a.num_scenes = num_scenes;
  a.jobs = b->d_jobs;
  a.job_end = b->d_job_end;
  a.num_jobs = (int)nj;
  int leaf = scenes[0]->ds.max_leaf;
  for (int i = 1; i < num_scenes; ++i)
    if (scenes[i]->ds.max_leaf != leaf) leaf = 0;
  b->cfg.max_leaf_size = leaf;
  *out = b;
  return EAR_OK;
}

ear_status ear_batch_set_config(ear_batch* b, const ear_batch_config* c) {
  g_err[0] = 0;
  if (!b || !c) return fail(EAR_ERR_INVALID_ARG, "null argument");
  ear_batch_config n = *c;
  n.max_leaf_size = b->cfg.max_leaf_size;
  if (n.bvh_width != 0 && n.bvh_width != 2 && n.bvh_width != 4)
    return fail(EAR_ERR_INVALID_ARG, "bvh_width must be 0, 2 or 4");
  if (n.bvh_width) {
    const ear_status rc = set_width(b, n.bvh_width);
    if (rc != EAR_OK) return rc;
  }
  Schedule sc;
  const ear_status rc = schedule(b, n, &sc);
  if (rc != EAR_OK) return rc;
  b->cfg = n;
  free_graph(b);
  return EAR_OK;
}

ear_status ear_batch_get_config(const ear_batch* b, ear_batch_config* c) {
  if (!b || !c) return fail(EAR_ERR_INVALID_ARG, "null argument");
  *c = b->cfg;
  return EAR_OK;
}

ear_status ear_batch_set_sources(ear_batch* b, const float* pos) {
  g_err[0] = 0;
  if (!b || !pos) return fail(EAR_ERR_INVALID_ARG, "null argument");
  for (size_t j = 0; j < b->jobs.size(); ++j) {
    for (int k = 0; k < 3; ++k) {
      if (!std::isfinite(pos[3 * j + k])) return fail(EAR_ERR_INVALID_ARG, "non-finite source position");
      b->jobs[j].src[k] = pos[3 * j + k];
    }
  }
  CU(cudaSetDevice(b->device));
  cudaStream_t st = (cudaStream_t)b->params.stream;
  CU(cudaMemcpyAsync(b->d_jobs, b->jobs.data(), sizeof(BatchJob) * b->jobs.size(),
                     cudaMemcpyHostToDevice, st));
  CU(cudaStreamSynchronize(st));
  b->ran = false;
  return EAR_OK;
}

ear_status ear_batch_run(ear_batch* b, ear_render_stats* stats) {
  g_err[0] = 0;
  if (!b) return fail(EAR_ERR_INVALID_ARG, "null batch");
  CU(cudaSetDevice(b->device));
  ear_status rc = sync_scenes(b);
  if (rc != EAR_OK) return rc;
  Schedule sc;
  rc = schedule(b, b->cfg, &sc);
  if (rc != EAR_OK) return rc;
  cudaStream_t st = (cudaStream_t)b->params.stream;
  if (!b->cfg.no_graph && !b->exec) {
    // capture on the batch's own stream (the legacy default stream cannot
    // be captured); the graph is then launched into the caller's stream
    CU(cudaStreamBeginCapture(b->cap_stream, cudaStreamCaptureModeThreadLocal));
    const cudaError_t e = enqueue(b, sc, b->a, b->cap_stream);
    cudaGraph_t g = nullptr;
    const cudaError_t e2 = cudaStreamEndCapture(b->cap_stream, &g);
    if (e != cudaSuccess || e2 != cudaSuccess) {
      if (g) cudaGraphDestroy(g);
      return fail(EAR_ERR_CUDA, "batch graph capture: %s",
                  cudaGetErrorString(e != cudaSuccess ? e : e2));
    }
    b->graph = g;
    const cudaError_t e3 = cudaGraphInstantiate(&b->exec, b->graph, 0);
    if (e3 != cudaSuccess) {
      free_graph(b);
      return fail(EAR_ERR_CUDA, "batch graph instantiation: %s", cudaGetErrorString(e3));
    }
  }
  CU(cudaEventRecord(b->ev0, st));
  if (b->cfg.no_graph) {
    CU(enqueue(b, sc, b->a, st));
  } else {
    CU(cudaGraphLaunch(b->exec, st));
  }
  CU(cudaEventRecord(b->ev1, st));
  const size_t rows = (size_t)b->total_tracks * 3;
  b->fl.resize(std::max<size_t>(rows, 1));
  unsigned long long cnt[kNumCounters];
  CU(cudaMemcpyAsync(b->fl.data(), b->d_fl, sizeof(int2) * rows, cudaMemcpyDeviceToHost, st));
  CU(cudaMemcpyAsync(cnt, b->d_counters, sizeof cnt, cudaMemcpyDeviceToHost, st));
  CU(cudaStreamSynchronize(st));
  rc = check_errors(b);
  if (rc != EAR_OK) return rc;
  float ms = 0.0f;
  CU(cudaEventElapsedTime(&ms, b->ev0, b->ev1));
  fill_stats(cnt, b->a.num_items, ms, stats);
  if (stats) {
    stats->map_build_ms = b->map_build_ms;
    for (const VisMap& m : b->maps) {
      stats->map_bytes += m.bytes;
      stats->map_res = std::max(stats->map_res, m.cells ? m.res : 0);
    }
  }
  b->map_build_ms = 0.0;
  b->ran = true;
  return EAR_OK;
}

ear_status ear_batch_histograms(const ear_batch* b, int32_t job, ear_histograms* out) {
  g_err[0] = 0;
  if (!b || !out || !out->data) return fail(EAR_ERR_INVALID_ARG, "null argument");
  if (job < 0 || job >= (int32_t)b->jobs.size()) return fail(EAR_ERR_INVALID_ARG, "job %d out of range", job);
  if (!b->ran) return fail(EAR_ERR_STATE, "ear_batch_run has not completed since the last change");
  CU(cudaSetDevice(b->device));
  const int nb = b->params.num_bins;
  const size_t stride = hist_stride(nb);
  const int row0 = 3 * b->first_track[(size_t)job];
  const int rows = 3 * b->tracks[(size_t)job];
  const cudaMemcpyKind kind = out->on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
  CU(cudaMemcpy2D(out->data, sizeof(float) * nb, b->d_hist + (size_t)row0 * stride,
                  sizeof(float) * stride, sizeof(float) * nb, (size_t)rows, kind));
  std::vector<int32_t> f((size_t)rows), l((size_t)rows);
  for (int i = 0; i < rows; ++i) {
    f[(size_t)i] = std::min(b->fl[(size_t)(row0 + i)].x, nb);
    l[(size_t)i] = std::min(b->fl[(size_t)(row0 + i)].y, nb);
  }
  const cudaMemcpyKind k2 = out->on_device ? cudaMemcpyHostToDevice : cudaMemcpyHostToHost;
  if (out->first_sample) CU(cudaMemcpy(out->first_sample, f.data(), sizeof(int32_t) * rows, k2));
  if (out->last_sample) CU(cudaMemcpy(out->last_sample, l.data(), sizeof(int32_t) * rows, k2));
  return EAR_OK;
}

ear_status ear_batch_device_view(const ear_batch* b, const float** data, int32_t* stride,
                                 int64_t* rows, int32_t* first_track, int32_t max_jobs) {
  if (!b) return fail(EAR_ERR_INVALID_ARG, "null batch");
  if (data) *data = b->d_hist;
  if (stride) *stride = (int32_t)hist_stride(b->params.num_bins);
  if (rows) *rows = (int64_t)b->total_tracks * 3;
  if (first_track)
    for (int32_t j = 0; j < max_jobs && j < (int32_t)b->jobs.size(); ++j) first_track[j] = b->first_track[(size_t)j];
  return EAR_OK;
}

void ear_batch_destroy(ear_batch* b) {
  if (!b) return;
  cudaSetDevice(b->device);
  free_graph(b);
  cudaFree(b->d_scenes);
  cudaFree(b->d_jobs);
  cudaFree(b->d_job_end);
  cudaFree(b->d_trial_jobs);
  cudaFree(b->d_trial_end);
  cudaFree(b->d_recs);
  cudaFree(b->d_mats);
  cudaFree(b->d_hist);
  cudaFree(b->d_fl);
  cudaFree(b->d_dvis);
  cudaFree(b->d_counters);
  cudaFree(b->d_err);
  for (VisMap& m : b->maps) free_vis_map(&m);
  if (b->cap_stream) cudaStreamDestroy(b->cap_stream);
  if (b->ev0) cudaEventDestroy(b->ev0);
  if (b->ev1) cudaEventDestroy(b->ev1);
  delete b;
}

ear_status ear_render_batch(ear_scene* const* scenes, int32_t num_scenes, const ear_batch_job* jobs,
                            int32_t num_jobs, const ear_render_params* params, ear_histograms* outs,
                            ear_render_stats* stats) {
  if (!outs) return fail(EAR_ERR_INVALID_ARG, "null outputs");
  ear_batch* b = nullptr;
  ear_status rc = ear_batch_create(scenes, num_scenes, jobs, num_jobs, params, &b);
  if (rc != EAR_OK) return rc;
  ear_batch_config c{};
  c.no_graph = 1;  // a single run gains nothing from capturing
  rc = ear_batch_set_config(b, &c);
  if (rc == EAR_OK) rc = ear_batch_run(b, stats);
  for (int32_t j = 0; rc == EAR_OK && j < num_jobs; ++j) rc = ear_batch_histograms(b, j, &outs[j]);
  ear_batch_destroy(b);
  return rc;
}

ear_status ear_batch_tune(ear_batch* b, const ear_tune_opts* opts, ear_tune_result* result) {
  g_err[0] = 0;
  if (!b) return fail(EAR_ERR_INVALID_ARG, "null batch");
  ear_tune_opts o;
  std::memset(&o, 0, sizeof o);
  if (opts) o = *opts;
  const double frac = o.trial_fraction > 0.0 ? std::min(o.trial_fraction, 1.0) : 0.02;
  const uint64_t min_rays = o.min_trial_rays ? o.min_trial_rays : 256;
  const int repeats = o.repeats > 0 ? o.repeats : 2;
  CU(cudaSetDevice(b->device));
  ear_tune_result res;
  std::memset(&res, 0, sizeof res);
  const std::string key = tune_key(b, o.tune_leaf_size != 0, o.tune_width != 0);
  ear_batch_config cached{};
  float cached_ms = 0.0f;
  if (cache_lookup(o.cache_path, key, &cached, &cached_ms)) {
    if (o.tune_leaf_size && cached.max_leaf_size > 0) {
      const ear_status rc = rebuild_scenes(b, cached.max_leaf_size);
      if (rc != EAR_OK) return rc;
      b->cfg.max_leaf_size = cached.max_leaf_size;
    }
    if (o.tune_width && (cached.bvh_width == 2 || cached.bvh_width == 4)) {
      const ear_status rc = set_width(b, cached.bvh_width);
      if (rc != EAR_OK) return rc;
      b->cfg.bvh_width = cached.bvh_width;
    }
    ear_batch_config c = cached;
    c.no_graph = b->cfg.no_graph;
    const ear_status rc = ear_batch_set_config(b, &c);
    if (rc != EAR_OK) return rc;
    res.best = b->cfg;
    res.best_ms = cached_ms;
    res.from_cache = 1;
    if (result) *result = res;
    return EAR_OK;
  }
  // trial tables: every job, a fraction of its rays
  int nb = 0;
  for (int band = 0; band < 3; ++band) nb += (b->params.bands_mask >> band) & 1;
  std::vector<BatchJob> tj = b->jobs;
  std::vector<uint64_t> tend(tj.size());
  uint64_t items = 0;
  for (size_t j = 0; j < tj.size(); ++j) {
    const uint64_t r = std::max<uint64_t>(std::min<uint64_t>(min_rays, tj[j].num_rays),
                                          (uint64_t)std::llround((double)tj[j].num_rays * frac));
    tj[j].num_rays = std::min<uint64_t>(r, tj[j].num_rays);
    items += tj[j].num_rays * (uint64_t)nb;
    tend[j] = items;
  }
  CU(cudaMemcpy(b->d_trial_jobs, tj.data(), sizeof(BatchJob) * tj.size(), cudaMemcpyHostToDevice));
  CU(cudaMemcpy(b->d_trial_end, tend.data(), sizeof(uint64_t) * tend.size(), cudaMemcpyHostToDevice));

  // leaf sizes apply to LBVH scenes only (PLOC builds single-triangle leaves)
  bool all_lbvh = true;
  for (const ear_scene* sc : b->scenes) all_lbvh = all_lbvh && sc->ds.builder != kBuilderPloc;
  const bool tune_leaf = o.tune_leaf_size && all_lbvh;
  std::vector<int> leaves = {b->cfg.max_leaf_size > 0 ? b->cfg.max_leaf_size : 1};
  if (tune_leaf) leaves = {1, 2, 4};
  const int blocks[] = {128, 256};
  std::vector<int> widths = {0};
  if (o.tune_width) widths = {2, 4};
  ear_batch_config best{};
  float best_ms = 0.0f;
  bool have = false;
  for (int leaf : leaves)
  for (int width : widths) {
    if (tune_leaf) {
      const ear_status rc = rebuild_scenes(b, leaf);
      if (rc != EAR_OK) return rc;
      b->cfg.max_leaf_size = leaf;
    }
    if (width) {
      const ear_status rc = set_width(b, width);
      if (rc != EAR_OK) return rc;
    }
    for (int block : blocks) {
      ear_batch_config probe{};
      probe.block = block;
      Schedule sc;
      ear_status rc = schedule(b, probe, &sc);
      if (rc != EAR_OK) return rc;
      // resident blocks per SM: the occupancy limit, one less, and half
      const int max_per_sm = sc.grid / b->sm_count;
      std::vector<int> per = {max_per_sm};
      if (max_per_sm > 1) per.push_back(max_per_sm - 1);
      if (max_per_sm > 3) per.push_back(max_per_sm / 2);
      for (int q : per) {
        ear_batch_config c{};
        c.block = block;
        c.blocks_per_sm = q;
        c.max_leaf_size = leaf;
        c.bvh_width = width;
        float ms = 0.0f, best_here = 0.0f;
        // one untimed warm-up, then the best of `repeats`
        rc = trial(b, c, items, &ms);
        if (rc != EAR_OK) return rc;
        for (int r = 0; r < repeats; ++r) {
          rc = trial(b, c, items, &ms);
          if (rc != EAR_OK) return rc;
          best_here = r == 0 ? ms : std::min(best_here, ms);
        }
        ++res.candidates;
        if (leaf == leaves[0] && width == widths[0] && block == b->ops->block && q == max_per_sm)
          res.default_ms = best_here;
        if (!have || best_here < best_ms) {
          best = c;
          best_ms = best_here;
          have = true;
        }
      }
    }
  }
  if (tune_leaf) {
    const ear_status rc = rebuild_scenes(b, best.max_leaf_size);
    if (rc != EAR_OK) return rc;
    b->cfg.max_leaf_size = best.max_leaf_size;
  }
  if (o.tune_width) {
    const ear_status rc = set_width(b, best.bvh_width);
    if (rc != EAR_OK) return rc;
  }
  best.no_graph = b->cfg.no_graph;
  const ear_status rc = ear_batch_set_config(b, &best);
  if (rc != EAR_OK) return rc;
  cache_store(o.cache_path, key, b->cfg, best_ms);
  res.best = b->cfg;
  res.best_ms = best_ms;
  if (result) *result = res;
  return EAR_OK;
}

}  // extern "C"
