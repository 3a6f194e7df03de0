// api.cu -- implementation of the C ABI in include/ear_gb300.h.
//
// Host side of the drop-in boundary: validates arguments, derives the
// per-material and per-recorder constants exactly as the reference's
// constructors do (src/Material.cpp:26-72, src/StereoRecorder.cpp:53-57),
// owns the device buffers of a scene, launches the trace kernels and runs
// the end-of-render steps of Scene::Render (src/Scene.cpp:286-316).
// Host code in this file is compiled with -ffp-contract=off.

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <vector>

#include "../../include/ear_gb300.h"
#include "ear_internal.h"
#include "ear_record.cuh"
#include "host_internal.h"

namespace ear {

// Layout of the trace kernel's dynamic shared memory: the material table
// (16-byte aligned), then per (track, band) first/last bookkeeping for a
// single render or the scene table for a batch, then the adjoint's
// accumulators.
size_t trace_smem_bytes(int num_mats, int num_tracks, int mode, int block, int num_scenes) {
  size_t b = (sizeof(DevMaterial) * (size_t)num_mats + 15) & ~(size_t)15;
  if (mode == kModeBatch) return b + sizeof(SceneRef) * (size_t)num_scenes;
  b += sizeof(int) * 6 * (size_t)num_tracks;
  if (mode == kModeAdjoint) {
    b = (b + 7) & ~(size_t)7;
    b += sizeof(double) * 6 * (size_t)num_mats + sizeof(float) * 2 * (size_t)num_mats * (size_t)block;
  }
  return b;
}

thread_local char g_err[512] = "";

// Builder of ear_scene_build_bvh when the options leave it open: PLOC
// (measured +4..6% segments/s over the LBVH on the 20,000- and
// 2,000,000-triangle scenes).
constexpr int kDefaultBuilder = EAR_BVH_PLOC;

ear_status fail(ear_status st, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof g_err, fmt, ap);
  va_end(ap);
  return st;
}

// Material::Material (src/Material.cpp:26-72) and Material::Bounce
// (src/Material.cpp:76-83), per band.
bool derive_material(const ear_material& m, DevMaterial* o) {
  o->always_reflect = 0;
  for (int i = 0; i < 3; ++i) {
    float a = 1.0f;
    a -= m.reflection[i] - 1e-9f;
    if (m.has_refraction) a -= m.refraction[i] - 1e-9f;
    if (a < 0.0f) return false;
    o->survival[i] = 1.0f - a;
    const float fl = m.reflection[i];
    const float fr = m.has_refraction ? m.refraction[i] : 0.0f;
    if ((double)fl < 0.0001 && (double)fr < 0.0001) o->always_reflect |= 1u << i;
    o->p_reflect[i] = fl / (fl + fr);
    o->spec[i] = m.has_specularity ? m.specularity[i] : 0.0f;
    o->refl[i] = fl;
    o->refr[i] = fr;
  }
  return true;
}

int derive_recorders(const ear_recorder* recs, int nrec, int track_base, int job,
                     DevRecorder* out) {
  int tracks = 0;
  for (int i = 0; i < nrec; ++i) {
    const ear_recorder& r = recs[i];
    if (r.channels != 1 && r.channels != 2) {
      fail(EAR_ERR_INVALID_ARG, "recorder %d: channels must be 1 or 2", i);
      return -1;
    }
    DevRecorder& d = out[i];
    for (int k = 0; k < 3; ++k) {
      d.loc[k] = r.location[k];
      d.right[k] = r.right_ear[k];
      // std::max(0.0f, powf(1.0f - h, 4)) (src/StereoRecorder.cpp:56)
      const float h = powf_portable(1.0f - r.head_absorption[k], 4.0f);
      d.habs[k] = (0.0f < h) ? h : 0.0f;
    }
    d.head_size = r.head_size;
    d.channels = r.channels;
    d.track0 = track_base + tracks;
    d.job = job;
    d.vis_index = i;
    tracks += r.channels;
  }
  return tracks;
}

void fill_stats(const unsigned long long* cnt, uint64_t num_items, double kernel_ms,
                ear_render_stats* stats) {
  if (!stats) return;
  stats->rays = std::min<unsigned long long>(cnt[kWork], num_items);
  stats->segments = cnt[kSegments];
  stats->shadow_queries = cnt[kShadow];
  stats->contributions = cnt[kContrib];
  stats->sampler_overflows = cnt[kOverflow];
  stats->node_visits = cnt[kNodeVisits];
  stats->triangle_tests = cnt[kTriTests];
  stats->splat_bins = cnt[kSplatBins];
  stats->kernel_ms = kernel_ms;
  stats->map_entries = cnt[kMapEntries];
  stats->map_build_ms = 0.0;
  stats->map_bytes = 0;
  stats->map_res = 0;
  stats->reserved1 = 0;
}

namespace fin {

__global__ void k_init_first_last(int2* fl, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) fl[i] = make_int2(kInitialFirstSample, 0);
}

// End of Scene::Render (src/Scene.cpp:286-316) for one (recorder, band),
// one block each: Recorder::Multiply(1/amount) over every track's
// [first_sample, real_length) (src/Recorder.cpp:85-89), the direct-sound
// lobe INV_SPHERE_2(len) * air^len * dry recorded at len / 343 s when the
// trace kernel found the listener-source segment unblocked, then
// Multiply(gain^2).  The block owns its rows, so the lobe is added with
// plain stores by one thread, in the reference's order.

__device__ void scale_rows(const FinalizeArgs& f, const DevRecorder& R, int band, float x) {
  for (int k = 0; k < R.channels; ++k) {
    const int tb = (R.track0 + k) * 3 + band;
    const int2 r = f.first_last[tb];
    const int hi = r.y < f.num_bins ? r.y : f.num_bins;
    float* h = f.hist + (size_t)tb * f.stride;
    for (int i = r.x + (int)threadIdx.x; i < hi; i += (int)blockDim.x) h[i] *= x;
  }
}

__global__ void k_finalize(const FinalizeArgs f) {
  const int ri = blockIdx.x / 3, band = blockIdx.x % 3;
  if (!((f.bands >> band) & 1u)) return;
  const DevRecorder R = f.recs[ri];
  const float* sp = f.src;
  float inv_amount = f.inv_amount, gain2 = f.gain2;
  if (f.jobs) {
    const BatchJob& J = f.jobs[R.job];
    sp = J.src;
    inv_amount = J.inv_amount;
    gain2 = J.gain2;
  }
  scale_rows(f, R, band, inv_amount);
  __syncthreads();
  if (threadIdx.x == 0 && f.direct_vis && f.direct_vis[ri]) {
    const V3 loc = mk(R.loc[0], R.loc[1], R.loc[2]);
    const V3 src = mk(sp[0], sp[1], sp[2]);
    const V3 dist = sub(loc, src);
    const float len = length(dist);
    const V3 dir = normalized(dist);
    const float amp = inv_sphere_2(len) * powf_portable(f.air[band], len) * f.dry;
    const SplatPlan p = record_plan<false>(R, band, dir, amp, len / 343.0f, len);
    for (int k = 0; k < p.tracks; ++k) {
      const int tb = (R.track0 + k) * 3 + band;
      float* row = f.hist + (size_t)tb * f.stride;
      int2 fl = f.first_last[tb];
      float v = p.ampl[k];
      for (int i = 0; i < p.w; ++i) {
        const long long pos = p.s[k] + i;
        if (pos >= 0) {
          const int c = (int)(pos < f.num_bins ? pos : f.num_bins);
          if (c > fl.y) fl.y = c;
          if (c < fl.x) fl.x = c;
          if (pos < f.num_bins) row[pos] += v;
        }
        v -= p.step[k];
      }
      f.first_last[tb] = fl;
    }
  }
  __syncthreads();
  scale_rows(f, R, band, gain2);
}

}  // namespace fin

using namespace fin;

cudaError_t launch_init_first_last(int2* fl, int n, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  k_init_first_last<<<(n + 127) / 128, 128, 0, st>>>(fl, n);
  return cudaGetLastError();
}

cudaError_t launch_finalize(const FinalizeArgs& f, int num_recorders, cudaStream_t st) {
  if (num_recorders <= 0) return cudaSuccess;
  k_finalize<<<num_recorders * 3, 256, 0, st>>>(f);
  return cudaGetLastError();
}

}  // namespace ear

using namespace ear;

extern "C" {

const char* ear_last_error(void) { return g_err; }
const char* ear_version(void) { return "ear_gb300 0.1 (sm_103a)"; }
int32_t ear_abi_version(void) { return EAR_ABI_VERSION; }

int32_t ear_num_tracks(const ear_recorder* recorders, int32_t num_recorders) {
  int32_t n = 0;
  for (int32_t i = 0; i < num_recorders; ++i) n += recorders[i].channels == 2 ? 2 : 1;
  return n;
}

ear_status ear_scene_create(const ear_scene_desc* desc, ear_scene** out) {
  g_err[0] = 0;
  if (!desc || !out) return fail(EAR_ERR_INVALID_ARG, "null argument");
  *out = nullptr;
  if (desc->num_triangles < 0 || (desc->num_triangles > 0 && (!desc->vertices || !desc->material_ids)))
    return fail(EAR_ERR_INVALID_ARG, "bad triangle arrays");
  if (desc->num_triangles >= (int64_t)kLeafStartMask)
    return fail(EAR_ERR_INVALID_ARG, "at most %d triangles per scene", kLeafStartMask - 1);
  if (desc->num_materials < 0 || (desc->num_materials > 0 && !desc->materials))
    return fail(EAR_ERR_INVALID_ARG, "bad material array");
  if (desc->num_materials > 4096) return fail(EAR_ERR_INVALID_ARG, "at most 4096 materials");
  std::vector<DevMaterial> mats((size_t)desc->num_materials);
  for (int i = 0; i < desc->num_materials; ++i)
    if (!derive_material(desc->materials[i], &mats[(size_t)i]))
      return fail(EAR_ERR_INVALID_ARG, "Invalid material settings (material %d)", i);
  for (int64_t i = 0; i < desc->num_triangles; ++i) {
    const int m = desc->material_ids[i];
    if (m < 0 || m >= desc->num_materials)
      return fail(EAR_ERR_INVALID_ARG, "material id %d out of range at triangle %lld", m,
                  (long long)i);
  }
  for (int64_t i = 0; i < desc->num_triangles * 9; ++i)
    if (!std::isfinite(desc->vertices[i]))
      return fail(EAR_ERR_INVALID_ARG, "non-finite vertex coordinate at triangle %lld",
                  (long long)(i / 9));
  CU(cudaSetDevice(desc->device));
  ear_scene* s = new ear_scene();
  s->device = desc->device;
  s->ds.num_tris = desc->num_triangles;
  s->num_mats = desc->num_materials;
  cudaDeviceGetAttribute(&s->sm_count, cudaDevAttrMultiProcessorCount, s->device);
  cudaError_t e = cudaSuccess;
  const size_t nt = (size_t)desc->num_triangles;
  if (nt) {
    e = cudaMalloc(&s->ds.vertices, sizeof(float) * 9 * nt);
    if (e == cudaSuccess) e = cudaMalloc(&s->ds.mat_ids, sizeof(int32_t) * nt);
    if (e == cudaSuccess)
      e = cudaMemcpy(s->ds.vertices, desc->vertices, sizeof(float) * 9 * nt, cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
      e = cudaMemcpy(s->ds.mat_ids, desc->material_ids, sizeof(int32_t) * nt, cudaMemcpyHostToDevice);
  }
  if (e == cudaSuccess) e = cudaMalloc(&s->mats, sizeof(DevMaterial) * std::max<size_t>(mats.size(), 1));
  if (e == cudaSuccess && !mats.empty())
    e = cudaMemcpy(s->mats, mats.data(), sizeof(DevMaterial) * mats.size(), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaEventCreate(&s->ev0);
  if (e == cudaSuccess) e = cudaEventCreate(&s->ev1);
  if (e != cudaSuccess) {
    ear_scene_destroy(s);
    return fail(e == cudaErrorMemoryAllocation ? EAR_ERR_OUT_OF_MEMORY : EAR_ERR_CUDA,
                "scene upload: %s", cudaGetErrorString(e));
  }
  *out = s;
  return EAR_OK;
}

ear_status ear_scene_build_bvh(ear_scene* s, const ear_bvh_opts* opts) {
  g_err[0] = 0;
  if (!s) return fail(EAR_ERR_INVALID_ARG, "null scene");
  CU(cudaSetDevice(s->device));
  char msg[256] = "";
  const float pad = opts ? opts->box_pad : -1.0f;
  const int max_leaf = opts && opts->max_leaf_size > 0 ? opts->max_leaf_size : 1;
  if (max_leaf > 16) return fail(EAR_ERR_INVALID_ARG, "max_leaf_size above 16");
  int builder = opts ? opts->builder : EAR_BVH_DEFAULT;
  if (builder == EAR_BVH_DEFAULT) builder = kDefaultBuilder;
  if (builder != EAR_BVH_LBVH && builder != EAR_BVH_PLOC)
    return fail(EAR_ERR_INVALID_ARG, "unknown BVH builder %d", builder);
  // PLOC search radius: 4 measured best for traversal of the 4-wide tree
  // (+11% segments/s over 16 on the 20,000- and 2,000,000-triangle scenes)
  const int radius = opts && opts->ploc_radius > 0 ? opts->ploc_radius : 4;
  if (radius > 256) return fail(EAR_ERR_INVALID_ARG, "ploc_radius above 256");
  const int width = opts ? opts->width : 0;
  if (width != 0 && width != 2 && width != 4) return fail(EAR_ERR_INVALID_ARG, "width must be 0, 2 or 4");
  const int order = opts ? opts->visibility_order : 0;
  if (order < 0 || order > 2) return fail(EAR_ERR_INVALID_ARG, "visibility_order must be 0, 1 or 2");
  const int vmap = opts ? opts->visibility_map : 0;
  if (vmap < -1 || (vmap > 0 && (vmap < 8 || vmap > 4096)))
    return fail(EAR_ERR_INVALID_ARG, "visibility_map must be -1, 0 or 8..4096");
  cudaError_t e = build_lbvh(s->ds, pad, max_leaf, builder == EAR_BVH_PLOC ? kBuilderPloc : kBuilderLbvh,
                             radius, 0, msg, sizeof msg);
  // the triangles' leaf order changed: the visibility maps address them
  free_vis_map(&s->vis);
  s->vis_valid = false;
  ++s->bvh_gen;
  s->vis_opt = vmap;
  // a 4-wide tree deeper than its traversal trail is not kept (nodes4 null)
  s->ds.wide = s->ds.nodes4 != nullptr && (width == 4 || (width == 0 && s->ds.num_tris >= kWideFrom));
  s->ds.any_order = order;
  s->ds.any_far = order == 2 ? 1 : 0;
  s->probe_valid = false;
  if (e != cudaSuccess) {
    s->bvh = false;
    return fail(e == cudaErrorMemoryAllocation ? EAR_ERR_OUT_OF_MEMORY : EAR_ERR_CUDA,
                "LBVH build: %s", msg[0] ? msg : cudaGetErrorString(e));
  }
  s->bvh = true;
  return EAR_OK;
}

ear_status ear_scene_set_bvh_width(ear_scene* s, int32_t width) {
  g_err[0] = 0;
  if (!s) return fail(EAR_ERR_INVALID_ARG, "null scene");
  if (!s->bvh) return fail(EAR_ERR_STATE, "ear_scene_build_bvh has not been called");
  if (width != 2 && width != 4) return fail(EAR_ERR_INVALID_ARG, "width must be 2 or 4");
  if (width == 4 && !s->ds.nodes4)
    return fail(EAR_ERR_STATE, "the scene has no 4-wide tree (deeper than %d levels)", kMaxDepth4);
  s->ds.wide = width == 4;
  return EAR_OK;
}

ear_status ear_scene_bvh_width(const ear_scene* s, int32_t* width) {
  g_err[0] = 0;
  if (!s || !width) return fail(EAR_ERR_INVALID_ARG, "null argument");
  if (!s->bvh) return fail(EAR_ERR_STATE, "ear_scene_build_bvh has not been called");
  *width = s->ds.wide ? 4 : 2;
  return EAR_OK;
}

ear_status ear_scene_info(const ear_scene* s, int64_t* num_triangles, int64_t* num_nodes,
                          int32_t* max_depth, float* box_pad, int64_t* device_bytes) {
  if (!s) return fail(EAR_ERR_INVALID_ARG, "null scene");
  if (num_triangles) *num_triangles = s->ds.num_tris;
  if (num_nodes) *num_nodes = s->ds.num_nodes;
  if (max_depth) *max_depth = s->ds.max_depth;
  if (box_pad) *box_pad = s->ds.box_pad;
  if (device_bytes)
    *device_bytes = (int64_t)(s->ds.num_nodes * sizeof(Node) + s->ds.num_nodes4 * sizeof(Node4) +
                              s->ds.num_tris * (64 + 36 + 4));
  return EAR_OK;
}

ear_status ear_scene_sah_cost(const ear_scene* s, int32_t width, float node_cost,
                              float triangle_cost, double* cost) {
  if (!s || !cost || (width != 2 && width != 4))
    return fail(EAR_ERR_INVALID_ARG, "ear_scene_sah_cost: bad arguments");
  if (!s->bvh) return fail(EAR_ERR_STATE, "ear_scene_sah_cost before ear_scene_build_bvh");
  CU(cudaSetDevice(s->device));
  auto area = [](float lx, float hx, float ly, float hy, float lz, float hz) {
    const double dx = std::max(0.0, (double)hx - lx), dy = std::max(0.0, (double)hy - ly),
                 dz = std::max(0.0, (double)hz - lz);
    return 2.0 * (dx * dy + dy * dz + dz * dx);
  };
  auto leaf_count = [](int child) { return (((uint32_t)~child) >> kLeafCountShift) + 1; };
  // every node is entered through its parent's box: internal children cost
  // node_cost, leaves triangle_cost per triangle, each weighted by the box
  // area over the root's
  double sum = 0.0, root = 0.0;
  if (width == 2) {
    std::vector<Node> n((size_t)s->ds.num_nodes);
    CU(cudaMemcpy(n.data(), s->ds.nodes, sizeof(Node) * n.size(), cudaMemcpyDeviceToHost));
    for (size_t i = 0; i < n.size(); ++i) {
      const Node& q = n[i];
      const double a0 = area(q.a.x, q.a.y, q.a.z, q.a.w, q.b.x, q.b.y);
      const double a1 = area(q.b.z, q.b.w, q.c.x, q.c.y, q.c.z, q.c.w);
      const int ch[2] = {q.d.x, q.d.y};
      const double ar[2] = {a0, a1};
      for (int j = 0; j < 2; ++j)
        sum += ch[j] >= 0 ? node_cost * ar[j] : triangle_cost * leaf_count(ch[j]) * ar[j];
      if (i == 0) {
        root = area(std::min(q.a.x, q.b.z), std::max(q.a.y, q.b.w), std::min(q.a.z, q.c.x),
                    std::max(q.a.w, q.c.y), std::min(q.b.x, q.c.z), std::max(q.b.y, q.c.w));
      }
    }
  } else {
    if (!s->ds.nodes4) return fail(EAR_ERR_STATE, "the scene has no 4-wide tree");
    std::vector<Node4> n((size_t)s->ds.num_nodes4);
    CU(cudaMemcpy(n.data(), s->ds.nodes4, sizeof(Node4) * n.size(), cudaMemcpyDeviceToHost));
    for (size_t i = 0; i < n.size(); ++i) {
      const Node4& q = n[i];
      const float* lx = &q.lox.x;
      const float* hx = &q.hix.x;
      const float* ly = &q.loy.x;
      const float* hy = &q.hiy.x;
      const float* lz = &q.loz.x;
      const float* hz = &q.hiz.x;
      const int* ch = &q.child.x;
      float u[6] = {1e30f, -1e30f, 1e30f, -1e30f, 1e30f, -1e30f};
      for (int j = 0; j < 4; ++j) {
        if (!((q.meta.y >> j) & 1)) continue;
        const double a = area(lx[j], hx[j], ly[j], hy[j], lz[j], hz[j]);
        sum += ch[j] >= 0 ? node_cost * a : triangle_cost * leaf_count(ch[j]) * a;
        u[0] = std::min(u[0], lx[j]);
        u[1] = std::max(u[1], hx[j]);
        u[2] = std::min(u[2], ly[j]);
        u[3] = std::max(u[3], hy[j]);
        u[4] = std::min(u[4], lz[j]);
        u[5] = std::max(u[5], hz[j]);
      }
      if (i == 0) root = area(u[0], u[1], u[2], u[3], u[4], u[5]);
    }
  }
  // the root node itself is always entered
  *cost = root > 0 ? node_cost + sum / root : 0.0;
  return EAR_OK;
}

void ear_scene_destroy(ear_scene* s) {
  if (!s) return;
  cudaSetDevice(s->device);
  cudaFree(s->ds.nodes);
  cudaFree(s->ds.nodes4);
  cudaFree(s->ds.tris);
  cudaFree(s->ds.vertices);
  cudaFree(s->ds.mat_ids);
  cudaFree(s->mats);
  cudaFree(s->hist);
  cudaFree(s->fl);
  cudaFree(s->counters);
  cudaFree(s->err);
  cudaFree(s->dvis);
  cudaFree(s->recs);
  cudaFree(s->emitter);
  cudaFree(s->probe);
  free_vis_map(&s->vis);
  if (s->ev0) cudaEventDestroy(s->ev0);
  if (s->ev1) cudaEventDestroy(s->ev1);
  delete s;
}

}  // extern "C"

namespace {

// Automatic visibility order (ear_bvh_opts.visibility_order = 0): traversal
// of the visibility tests visits the farthest hit child first when the
// occlusion probe finds more than 15% of 4096 seeded centroid -> recorder
// segments blocked -- occluders between the surfaces and the listeners are
// then met sooner (measured: +12% segments/s on the 2,000,000-triangle nave
// with its columns, 53% of whose visibility tests are blocked; -2.4% on the
// open 20,000-triangle hall, 0% blocked).  The probe runs again only when
// the recorder set or the tree changes.  Results never depend on the order.
ear_status choose_visibility_order(ear_scene* s, const ear_recorder* recs, int32_t nrec,
                                   TraceArgs& a, const TraceOps* ops, cudaStream_t st) {
  if (s->ds.any_order != 0 || nrec <= 0) {
    a.any_far = s->ds.any_far;
    return EAR_OK;
  }
  uint64_t key = 1469598103934665603ull ^ (uint64_t)(uintptr_t)s->ds.nodes4;
  for (int32_t i = 0; i < nrec; ++i)
    for (int k = 0; k < 3; ++k) {
      uint32_t bits;
      std::memcpy(&bits, &recs[i].location[k], sizeof bits);
      key = (key ^ bits) * 1099511628211ull;
    }
  if (!s->probe_valid || key != s->probe_key) {
    constexpr int kProbeSegments = 4096;
    if (!s->probe) CU(cudaMalloc(&s->probe, sizeof(unsigned)));
    CU(cudaMemsetAsync(s->probe, 0, sizeof(unsigned), st));
    // the cached order must not depend on a caller's traversal budget
    TraceArgs pa = a;
    pa.traverse_budget = traverse_budget(s->ds.wide ? s->ds.num_nodes4 : s->ds.num_nodes, s->ds.wide != 0);
    CU(ops->probe(pa, kProbeSegments, s->probe, st));
    unsigned blocked = 0;
    CU(cudaMemcpyAsync(&blocked, s->probe, sizeof blocked, cudaMemcpyDeviceToHost, st));
    CU(cudaStreamSynchronize(st));
    s->ds.any_far = blocked > kProbeSegments * 15 / 100 ? 1 : 0;
    s->probe_key = key;
    s->probe_valid = true;
  }
  a.any_far = s->ds.any_far;
  return EAR_OK;
}

// Listener visibility maps for the recorder set (ear_bvh_opts.
// visibility_map): built on first use, reused while the set, the tree and
// the setting stay the same.  A set whose lists would exceed the entry
// limit keeps the tree traversal.  *build_ms receives the build time.
// Identity of a recorder set's maps: the requested resolution, the tree
// generation and the recorder locations (FNV-1a over their bits).
uint64_t vis_map_key(const ear_scene* s, const ear_recorder* recs, int32_t nrec, int res) {
  uint64_t key = (1469598103934665603ull ^ (uint64_t)res) * 1099511628211ull;
  key = (key ^ s->bvh_gen) * 1099511628211ull;
  for (int32_t i = 0; i < nrec; ++i)
    for (int k = 0; k < 3; ++k) {
      uint32_t bits;
      std::memcpy(&bits, &recs[i].location[k], sizeof bits);
      key = (key ^ bits) * 1099511628211ull;
    }
  return (key ^ (uint64_t)nrec) * 1099511628211ull;
}

void set_vis_args(const ear_scene* s, TraceArgs& a) {
  a.vis_cells = s->vis.cells;
  a.vis_entries = s->vis.entries;
  a.vis_res = s->vis.res;
  a.vis_cap = kVisWalkCap;
}

ear_status use_visibility_maps(ear_scene* s, const ear_recorder* recs, int32_t nrec, TraceArgs& a,
                               cudaStream_t st, double* build_ms) {
  *build_ms = 0.0;
  a.vis_res = 0;
  if (nrec <= 0 || s->vis_opt < 0 || s->ds.num_tris <= 0) return EAR_OK;
  const bool automatic = s->vis_opt == 0;
  int res = s->vis_opt;
  if (automatic) res = vis_auto_res(s->ds.num_tris);
  const uint64_t key = vis_map_key(s, recs, nrec, res);
  if (!s->vis_valid || key != s->vis_key) {
    // automatic: a render of fewer paths than the scene has triangles
    // does not repay the build (a new recorder set per short render)
    if (automatic && a.num_items < (uint64_t)s->ds.num_tris) return EAR_OK;
    free_vis_map(&s->vis);
    s->vis_valid = false;
    float locs[kMaxRecorders][3];
    for (int32_t i = 0; i < nrec; ++i)
      for (int k = 0; k < 3; ++k) locs[i][k] = recs[i].location[k];
    size_t free_b = 0, total_b = 0;
    CU(cudaMemGetInfo(&free_b, &total_b));
    // build peak: 24 bytes per entry for the sort plus the 48 kept; the
    // automatic setting keeps at most EAR_VISMAP_AUTO_MAX_ENTRIES and
    // lowers the resolution by a quarter until the lists fit
    const uint64_t fit = (uint64_t)(free_b / 2) / (24 + kVisEntryBytes + kVisCellBytes);
    const uint64_t limit = std::min<uint64_t>(
        automatic ? (uint64_t)EAR_VISMAP_AUTO_MAX_ENTRIES : (1ull << 31) - 1, fit);
    char msg[256] = "";
    bool too_large = false;
    CU(cudaEventRecord(s->ev0, st));
    for (;;) {
      const cudaError_t e = build_vis_map(s->ds, locs, nrec, res, limit, st, &s->vis, &too_large,
                                          msg, sizeof msg);
      if (e == cudaErrorMemoryAllocation && automatic) {
        // the automatic maps are an accelerator: without room the tree serves
        cudaGetLastError();
        too_large = true;
        break;
      }
      if (e != cudaSuccess)
        return fail(e == cudaErrorMemoryAllocation ? EAR_ERR_OUT_OF_MEMORY : EAR_ERR_CUDA,
                    "visibility map build: %s", msg[0] ? msg : cudaGetErrorString(e));
      if (!too_large || !automatic || res <= 64) break;
      res = std::max(64, (res * 3 / 4) / 32 * 32);
    }
    CU(cudaEventRecord(s->ev1, st));
    CU(cudaEventSynchronize(s->ev1));
    float ms = 0.0f;
    CU(cudaEventElapsedTime(&ms, s->ev0, s->ev1));
    *build_ms = ms;
    s->vis_refused = too_large;
    s->vis_key = key;
    s->vis_valid = true;
  }
  if (s->vis_refused) return EAR_OK;
  set_vis_args(s, a);
  return EAR_OK;
}

void map_stats(const ear_scene* s, const TraceArgs& a, ear_render_stats* stats) {
  stats->map_bytes = a.vis_res > 0 ? (uint64_t)s->vis.bytes : 0;
  stats->map_res = a.vis_res;
  stats->reserved1 = 0;
}

struct Prepared {
  TraceArgs a;
  int num_tracks;
  size_t smem;
  int grid;
  int block;
  const TraceOps* ops;
};

ear_status prepare(ear_scene* s, const ear_source* src, const ear_recorder* recs, int32_t nrec,
                   const ear_render_params* p, uint32_t bands_mask, Prepared* out,
                   int mode = kModeForward) {
  if (!s || !src || !p || (nrec > 0 && !recs)) return fail(EAR_ERR_INVALID_ARG, "null argument");
  if (!s->bvh) return fail(EAR_ERR_STATE, "ear_scene_build_bvh has not been called");
  if (nrec < 0 || nrec > kMaxRecorders)
    return fail(EAR_ERR_INVALID_ARG, "between 0 and %d recorders", kMaxRecorders);
  if (p->num_bins <= 0 || p->num_bins > (1 << 30)) return fail(EAR_ERR_INVALID_ARG, "bad num_bins");
  if (bands_mask == 0 || (bands_mask & ~7u)) return fail(EAR_ERR_INVALID_ARG, "bad bands_mask");
  if (p->max_bounces < 0) return fail(EAR_ERR_INVALID_ARG, "negative max_bounces");
  if (p->traverse_budget < 0) return fail(EAR_ERR_INVALID_ARG, "negative traverse_budget");
  if (p->num_rays > (1ull << 47) || p->first_ray > (1ull << 47) - p->num_rays)
    return fail(EAR_ERR_INVALID_ARG, "first_ray + num_rays above 2^47");
  if (src->num_emitter_triangles < 0 || (src->num_emitter_triangles > 0 && !src->emitter_vertices))
    return fail(EAR_ERR_INVALID_ARG, "bad emitter triangles");
  std::vector<DevRecorder> dr((size_t)nrec);
  const int tracks = derive_recorders(recs, nrec, 0, 0, dr.data());
  if (tracks < 0) return EAR_ERR_INVALID_ARG;
  TraceArgs& a = out->a;
  std::memset(&a, 0, sizeof a);
  const bool exact = (p->flags & EAR_FLAG_EXACT) != 0;
  out->ops = exact ? &kTraceExact : &kTraceFast;
  a.nodes = s->ds.nodes;
  a.nodes4 = s->ds.nodes4;
  a.wide = s->ds.wide;
  a.any_far = s->ds.any_far;
  a.tris = s->ds.tris;
  a.num_tris = (int)s->ds.num_tris;
  a.num_nodes = (int)(s->ds.wide ? s->ds.num_nodes4 : s->ds.num_nodes);
  a.mats = s->mats;
  a.num_mats = s->num_mats;
  a.num_recs = nrec;
  for (int k = 0; k < 3; ++k) a.src[k] = src->location[k];
  a.k0 = (uint32_t)p->seed;
  a.k1 = (uint32_t)(p->seed >> 32);
  a.context = p->context;
  int nb = 0;
  for (int b = 0; b < 3; ++b) {
    a.bands[b] = -1;
    if (bands_mask & (1u << b)) a.bands[nb++] = b;
    a.air[b] = 1.0f - p->air_absorption[b];
  }
  a.num_rays = p->num_rays;
  a.ray0 = p->first_ray;
  a.num_items = p->num_rays * (uint64_t)nb;
  a.max_bounces = p->max_bounces;
  a.cutoff = p->cutoff;
  a.box_pad = s->ds.box_pad;
  a.num_bins = p->num_bins;
  a.stride = (p->num_bins + 3) & ~3;
  a.num_tracks = tracks;
  a.traverse_budget = p->traverse_budget > 0 ? p->traverse_budget
                                             : traverse_budget(s->ds.wide ? s->ds.num_nodes4 : s->ds.num_nodes,
                                                               s->ds.wide != 0);
  a.dbg_band = -1;
  out->num_tracks = tracks;

  CU(cudaSetDevice(s->device));
  CU(grow(&s->recs, &s->recs_cap, (size_t)std::max(nrec, 1)));
  CU(grow(&s->fl, &s->fl_cap, (size_t)std::max(tracks * 3, 1)));
  CU(grow(&s->counters, &s->counters_cap, (size_t)kNumCounters));
  CU(grow(&s->err, &s->err_cap, (size_t)1));
  CU(grow(&s->dvis, &s->dvis_cap, (size_t)std::max(nrec, 1)));
  CU(grow(&s->hist, &s->hist_cap, (size_t)std::max(tracks * 3, 1) * (size_t)a.stride));
  a.recs = s->recs;
  a.hist = s->hist;
  a.first_last = s->fl;
  const bool direct = !(p->flags & (EAR_FLAG_RAW | EAR_FLAG_NO_DIRECT)) &&
                      src->num_emitter_triangles <= 0 && nrec > 0 && mode != kModeAdjoint;
  a.direct_vis = direct ? s->dvis : nullptr;
  a.counters = s->counters;
  a.error_flag = s->err;
  cudaStream_t st = (cudaStream_t)p->stream;
  if (nrec) CU(cudaMemcpyAsync(s->recs, dr.data(), sizeof(DevRecorder) * nrec, cudaMemcpyHostToDevice, st));
  // emitter: (a, area) (b, 0) (c, 0) (normal, 0) per triangle
  if (src->num_emitter_triangles > 0) {
    const int64_t ne = src->num_emitter_triangles;
    if (ne > (1 << 24)) return fail(EAR_ERR_INVALID_ARG, "emitter too large");
    std::vector<float4> em((size_t)ne * 4);
    float total = 0.0f;
    for (int64_t i = 0; i < ne; ++i) {
      const float* v = src->emitter_vertices + 9 * i;
      const V3 A = mk(v[0], v[1], v[2]), B = mk(v[3], v[4], v[5]), C = mk(v[6], v[7], v[8]);
      const V3 nn = normalized(cross(sub(B, A), sub(C, A)));
      // Triangle::calcArea: |edge(0) x edge(1)| / 2 (src/Triangle.cpp:26-30)
      const float area = length(cross(sub(B, A), sub(C, B))) / 2.0f;
      total += area;  // Mesh::Mesh (src/Mesh.cpp:90)
      em[(size_t)i * 4 + 0] = make_float4(A.x, A.y, A.z, area);
      em[(size_t)i * 4 + 1] = make_float4(B.x, B.y, B.z, 0.0f);
      em[(size_t)i * 4 + 2] = make_float4(C.x, C.y, C.z, 0.0f);
      em[(size_t)i * 4 + 3] = make_float4(nn.x, nn.y, nn.z, 0.0f);
    }
    CU(grow(&s->emitter, &s->emitter_cap, em.size()));
    CU(cudaMemcpyAsync(s->emitter, em.data(), sizeof(float4) * em.size(), cudaMemcpyHostToDevice, st));
    a.emitter = s->emitter;
    a.num_emitter = (int)ne;
    a.emitter_total_area = total;
  }
  CU(cudaMemsetAsync(s->hist, 0, sizeof(float) * (size_t)std::max(tracks * 3, 1) * a.stride, st));
  CU(cudaMemsetAsync(s->counters, 0, sizeof(unsigned long long) * kNumCounters, st));
  CU(cudaMemsetAsync(s->err, 0, sizeof(int), st));
  if (tracks) {
    k_init_first_last<<<(tracks * 3 + 127) / 128, 128, 0, st>>>(s->fl, tracks * 3);
    CU(cudaGetLastError());
  }
  out->block = out->ops->block;
  out->smem = trace_smem_bytes(s->num_mats, tracks, mode, out->block);
  if (out->smem > 200 * 1024) return fail(EAR_ERR_INVALID_ARG, "too many materials for one launch");
  int per_sm = 0;
  CU(out->ops->occupancy(mode, out->block, out->smem, &per_sm));
  if (per_sm < 1) per_sm = 1;
  out->grid = s->sm_count * per_sm;
  return EAR_OK;
}

ear_status finish(ear_scene* s, const ear_render_params* p, const Prepared& pr, double* kernel_ms) {
  cudaStream_t st = (cudaStream_t)p->stream;
  CU(cudaStreamSynchronize(st));
  int errflag = 0;
  CU(cudaMemcpy(&errflag, s->err, sizeof(int), cudaMemcpyDeviceToHost));
  if (kernel_ms) {
    float ms = 0.0f;
    CU(cudaEventElapsedTime(&ms, s->ev0, s->ev1));
    *kernel_ms = ms;
  }
  if (errflag & kErrIndex)
    return fail(EAR_ERR_CUDA, "internal: a device-side index check failed (corrupt BVH or scene data)");
  if (errflag & kErrBudget)
    return fail(EAR_ERR_DEVICE_BUDGET, "a BVH traversal exceeded its iteration budget");
  return EAR_OK;
}

}  // namespace

extern "C" ear_status ear_render(ear_scene* s, const ear_source* src, const ear_recorder* recs,
                                 int32_t nrec, const ear_render_params* p, ear_histograms* out,
                                 ear_render_stats* stats) {
  g_err[0] = 0;
  if (!out || !out->data) return fail(EAR_ERR_INVALID_ARG, "null output");
  if (!p) return fail(EAR_ERR_INVALID_ARG, "null params");
  Prepared pr;
  ear_status rc = prepare(s, src, recs, nrec, p, p->bands_mask, &pr);
  if (rc != EAR_OK) return rc;
  TraceArgs& a = pr.a;
  cudaStream_t st = (cudaStream_t)p->stream;
  rc = choose_visibility_order(s, recs, nrec, a, pr.ops, st);
  if (rc != EAR_OK) return rc;
  double map_ms = 0.0;
  rc = use_visibility_maps(s, recs, nrec, a, st, &map_ms);
  if (rc != EAR_OK) return rc;
  CU(cudaEventRecord(s->ev0, st));
  // with no rays the launch still computes the direct-sound visibility
  CU(pr.ops->trace(a, a.num_items > 0 ? pr.grid : 1, pr.block, pr.smem, kModeForward, st));
  CU(cudaEventRecord(s->ev1, st));
  const int rows = pr.num_tracks * 3;
  std::vector<int2> fl_raw((size_t)std::max(rows, 1));
  const bool want_raw = rows > 0 && (out->raw_first_sample || out->raw_last_sample);
  if (want_raw)
    CU(cudaMemcpyAsync(fl_raw.data(), a.first_last, sizeof(int2) * rows, cudaMemcpyDeviceToHost, st));
  if (!(p->flags & EAR_FLAG_RAW) && nrec > 0) {
    // amount is a float incremented once per ray (src/Scene.cpp:122,127):
    // exact to 2^24 rays, then stuck at 2^24.
    const float amount = p->num_rays <= 16777216ull ? (float)p->num_rays : 16777216.0f;
    FinalizeArgs f = {};
    f.hist = a.hist;
    f.stride = a.stride;
    f.num_bins = a.num_bins;
    f.first_last = a.first_last;
    f.recs = a.recs;
    f.direct_vis = a.direct_vis;
    for (int k = 0; k < 3; ++k) {
      f.src[k] = a.src[k];
      f.air[k] = a.air[k];
    }
    f.dry = p->dry_level;
    f.inv_amount = 1.0f / amount;
    f.gain2 = src->gain * src->gain;
    f.bands = p->bands_mask;
    k_finalize<<<nrec * 3, 256, 0, st>>>(f);
    CU(cudaGetLastError());
  }
  if (rows > 0) {
    const cudaMemcpyKind kind = out->on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    CU(cudaMemcpy2DAsync(out->data, sizeof(float) * a.num_bins, a.hist, sizeof(float) * a.stride,
                         sizeof(float) * a.num_bins, (size_t)rows, kind, st));
  }
  std::vector<int2> fl((size_t)std::max(rows, 1));
  if (rows > 0) CU(cudaMemcpyAsync(fl.data(), a.first_last, sizeof(int2) * rows, cudaMemcpyDeviceToHost, st));
  unsigned long long cnt[kNumCounters];
  CU(cudaMemcpyAsync(cnt, a.counters, sizeof cnt, cudaMemcpyDeviceToHost, st));
  double ms = 0.0;
  rc = finish(s, p, pr, &ms);
  if (rc != EAR_OK) return rc;
  const cudaMemcpyKind k2 = out->on_device ? cudaMemcpyHostToDevice : cudaMemcpyHostToHost;
  for (int pass = 0; pass < 2; ++pass) {
    const std::vector<int2>& src_fl = pass == 0 ? fl : fl_raw;
    int32_t* dst_f = pass == 0 ? out->first_sample : out->raw_first_sample;
    int32_t* dst_l = pass == 0 ? out->last_sample : out->raw_last_sample;
    if ((!dst_f && !dst_l) || rows == 0) continue;
    std::vector<int32_t> f((size_t)rows), l((size_t)rows);
    for (int i = 0; i < rows; ++i) {
      f[(size_t)i] = std::min(src_fl[(size_t)i].x, a.num_bins);
      l[(size_t)i] = std::min(src_fl[(size_t)i].y, a.num_bins);
    }
    if (dst_f) CU(cudaMemcpy(dst_f, f.data(), sizeof(int32_t) * rows, k2));
    if (dst_l) CU(cudaMemcpy(dst_l, l.data(), sizeof(int32_t) * rows, k2));
  }
  if (stats) {
    stats->rays = std::min<unsigned long long>(cnt[kWork], a.num_items);
    stats->segments = cnt[kSegments];
    stats->shadow_queries = cnt[kShadow];
    stats->contributions = cnt[kContrib];
    stats->sampler_overflows = cnt[kOverflow];
    stats->node_visits = cnt[kNodeVisits];
    stats->triangle_tests = cnt[kTriTests];
    stats->splat_bins = cnt[kSplatBins];
    stats->kernel_ms = ms;
    stats->map_entries = cnt[kMapEntries];
    stats->map_build_ms = map_ms;
    map_stats(s, a, stats);
  }
  return EAR_OK;
}

extern "C" ear_status ear_trace_debug(ear_scene* s, const ear_source* src,
                                      const ear_recorder* recs, int32_t nrec,
                                      const ear_render_params* p, int32_t band, int32_t max_record,
                                      int32_t* hit_tri, uint8_t* bounce_type, uint32_t* visible) {
  g_err[0] = 0;
  if (!p || !hit_tri || !bounce_type || !visible || max_record <= 0 || band < 0 || band > 2)
    return fail(EAR_ERR_INVALID_ARG, "bad debug arguments");
  Prepared pr;
  ear_status rc = prepare(s, src, recs, nrec, p, 1u << band, &pr, kModeDebug);
  if (rc != EAR_OK) return rc;
  TraceArgs& a = pr.a;
  double map_ms = 0.0;
  rc = use_visibility_maps(s, recs, nrec, a, (cudaStream_t)p->stream, &map_ms);
  if (rc != EAR_OK) return rc;
  const size_t n = (size_t)p->num_rays * (size_t)max_record;
  if (n > ((size_t)1 << 31)) return fail(EAR_ERR_INVALID_ARG, "debug record too large");
  int32_t* dh = nullptr;
  uint8_t* db = nullptr;
  uint32_t* dv = nullptr;
  cudaStream_t st = (cudaStream_t)p->stream;
  std::vector<int32_t> init(n, -2);
  cudaError_t e = cudaMalloc(&dh, sizeof(int32_t) * std::max<size_t>(n, 1));
  if (e == cudaSuccess) e = cudaMalloc(&db, std::max<size_t>(n, 1));
  if (e == cudaSuccess) e = cudaMalloc(&dv, sizeof(uint32_t) * std::max<size_t>(n, 1));
  if (e == cudaSuccess && n) e = cudaMemcpyAsync(dh, init.data(), sizeof(int32_t) * n, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess && n) e = cudaMemsetAsync(db, 0, n, st);
  if (e == cudaSuccess && n) e = cudaMemsetAsync(dv, 0, sizeof(uint32_t) * n, st);
  if (e == cudaSuccess) {
    a.dbg_band = band;
    a.dbg_rays = (int64_t)p->num_rays;
    a.dbg_max_record = max_record;
    a.dbg_hit = dh;
    a.dbg_bt = db;
    a.dbg_vis = dv;
    e = cudaEventRecord(s->ev0, st);
    if (e == cudaSuccess && a.num_items > 0) e = pr.ops->trace(a, pr.grid, pr.block, pr.smem, kModeDebug, st);
    if (e == cudaSuccess) e = cudaEventRecord(s->ev1, st);
    if (e == cudaSuccess && n) e = cudaMemcpyAsync(hit_tri, dh, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess && n) e = cudaMemcpyAsync(bounce_type, db, n, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess && n) e = cudaMemcpyAsync(visible, dv, sizeof(uint32_t) * n, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  }
  cudaFree(dh);
  cudaFree(db);
  cudaFree(dv);
  if (e != cudaSuccess) return fail(EAR_ERR_CUDA, "debug trace: %s", cudaGetErrorString(e));
  return finish(s, p, pr, nullptr);
}

// ---------------------------------------------------------- materials
extern "C" ear_status ear_scene_set_materials(ear_scene* s, const ear_material* materials,
                                              int32_t num_materials) {
  g_err[0] = 0;
  if (!s || (num_materials > 0 && !materials)) return fail(EAR_ERR_INVALID_ARG, "null argument");
  if (num_materials != s->num_mats)
    return fail(EAR_ERR_INVALID_ARG, "expected %d materials, got %d", s->num_mats, num_materials);
  std::vector<DevMaterial> mats((size_t)num_materials);
  for (int i = 0; i < num_materials; ++i)
    if (!derive_material(materials[i], &mats[(size_t)i]))
      return fail(EAR_ERR_INVALID_ARG, "Invalid material settings (material %d)", i);
  CU(cudaSetDevice(s->device));
  if (num_materials)
    CU(cudaMemcpy(s->mats, mats.data(), sizeof(DevMaterial) * mats.size(), cudaMemcpyHostToDevice));
  return EAR_OK;
}

// ------------------------------------------------------------- adjoint
namespace {

// Upstream gradient of the finalized histogram -> gradient of the raw splat
// sums: bins scaled by 1/N inside the pre-direct [first, real_length) and
// by gain^2 inside the final one (src/Scene.cpp:291,314).
__global__ void k_adjoint_scale(const float* g, int g_pitch, float* out, int stride, int nb,
                                int rows, const int4* ranges, float inv_amount, float gain2,
                                int scaled) {
  const int row = blockIdx.y;
  if (row >= rows) return;
  const int4 r = ranges[row];  // raw first, raw last, final first, final last
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < stride; i += gridDim.x * blockDim.x) {
    float v = 0.0f;
    if (i < nb) {
      v = g[(size_t)row * g_pitch + i];
      if (scaled) {
        if (i >= r.x && i < r.y) v *= inv_amount;
        if (i >= r.z && i < r.w) v *= gain2;
      }
    }
    out[(size_t)row * stride + i] = v;
  }
}

}  // namespace

extern "C" ear_status ear_render_adjoint(ear_scene* s, const ear_source* src,
                                         const ear_recorder* recs, int32_t nrec,
                                         const ear_render_params* p, const float* d_hist,
                                         int32_t d_hist_on_device, const int32_t* raw_first,
                                         const int32_t* raw_last, const int32_t* first,
                                         const int32_t* last, double* grad,
                                         ear_render_stats* stats) {
  g_err[0] = 0;
  if (!p || !d_hist || !grad) return fail(EAR_ERR_INVALID_ARG, "null argument");
  const bool scaled = !(p->flags & EAR_FLAG_RAW);
  if (scaled && (!raw_first || !raw_last || !first || !last))
    return fail(EAR_ERR_INVALID_ARG, "the bookkeeping of the forward render is required");
  if (s && s->num_mats > 32) return fail(EAR_ERR_UNSUPPORTED, "the adjoint supports at most 32 materials");
  Prepared pr;
  ear_status rc = prepare(s, src, recs, nrec, p, p->bands_mask, &pr, kModeAdjoint);
  if (rc != EAR_OK) return rc;
  TraceArgs& a = pr.a;
  cudaStream_t st = (cudaStream_t)p->stream;
  double map_ms = 0.0;
  rc = use_visibility_maps(s, recs, nrec, a, st, &map_ms);
  if (rc != EAR_OK) return rc;
  const int rows = pr.num_tracks * 3;
  // scaled upstream gradient in the (otherwise idle) histogram scratch
  float* g_in = nullptr;
  int4* ranges = nullptr;
  double* dgrad = nullptr;
  const size_t ngrad = (size_t)s->num_mats * 6;
  cudaError_t e = cudaSuccess;
  std::vector<int4> hr((size_t)std::max(rows, 1));
  for (int i = 0; i < rows; ++i)
    hr[(size_t)i] = scaled ? make_int4(raw_first[i], raw_last[i], first[i], last[i]) : make_int4(0, 0, 0, 0);
  if (rows) {
    if (!d_hist_on_device) {
      e = cudaMalloc(&g_in, sizeof(float) * (size_t)rows * a.num_bins);
      if (e == cudaSuccess)
        e = cudaMemcpyAsync(g_in, d_hist, sizeof(float) * (size_t)rows * a.num_bins,
                            cudaMemcpyHostToDevice, st);
    }
    if (e == cudaSuccess) e = cudaMalloc(&ranges, sizeof(int4) * rows);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(ranges, hr.data(), sizeof(int4) * rows, cudaMemcpyHostToDevice, st);
  }
  if (e == cudaSuccess) e = cudaMalloc(&dgrad, sizeof(double) * std::max<size_t>(ngrad, 1));
  if (e == cudaSuccess) e = cudaMemsetAsync(dgrad, 0, sizeof(double) * std::max<size_t>(ngrad, 1), st);
  if (e == cudaSuccess && rows) {
    const float amount = p->num_rays <= 16777216ull ? (float)p->num_rays : 16777216.0f;
    const dim3 grid((unsigned)std::min(1024, (a.stride + 255) / 256), (unsigned)rows);
    k_adjoint_scale<<<grid, 256, 0, st>>>(d_hist_on_device ? d_hist : g_in, a.num_bins, a.hist,
                                          a.stride, a.num_bins, rows, ranges, 1.0f / amount,
                                          src->gain * src->gain, scaled ? 1 : 0);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) {
    a.adj_g = a.hist;
    a.adj_grad = dgrad;
    e = cudaEventRecord(s->ev0, st);
    if (e == cudaSuccess && a.num_items > 0) e = pr.ops->trace(a, pr.grid, pr.block, pr.smem, kModeAdjoint, st);
    if (e == cudaSuccess) e = cudaEventRecord(s->ev1, st);
  }
  unsigned long long cnt[kNumCounters] = {0};
  if (e == cudaSuccess) e = cudaMemcpyAsync(grad, dgrad, sizeof(double) * ngrad, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(cnt, a.counters, sizeof cnt, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  cudaFree(g_in);
  cudaFree(ranges);
  cudaFree(dgrad);
  if (e != cudaSuccess) return fail(EAR_ERR_CUDA, "adjoint: %s", cudaGetErrorString(e));
  double ms = 0.0;
  rc = finish(s, p, pr, &ms);
  if (rc != EAR_OK) return rc;
  if (stats) {
    stats->rays = std::min<unsigned long long>(cnt[kWork], a.num_items);
    stats->segments = cnt[kSegments];
    stats->shadow_queries = cnt[kShadow];
    stats->contributions = cnt[kContrib];
    stats->sampler_overflows = cnt[kOverflow];
    stats->node_visits = cnt[kNodeVisits];
    stats->triangle_tests = cnt[kTriTests];
    stats->splat_bins = cnt[kSplatBins];
    stats->kernel_ms = ms;
    stats->map_entries = cnt[kMapEntries];
    stats->map_build_ms = map_ms;
    map_stats(s, a, stats);
  }
  return EAR_OK;
}

// ------------------------------------------------- FloatBuffer post-process
extern "C" {

ear_status ear_track_power(float* data, int32_t first, int32_t last, float a) {
  if (!data && last > first) return fail(EAR_ERR_INVALID_ARG, "null track");
  for (int32_t i = first; i < last; ++i) {
    const float f = std::pow(std::fabs(data[i]), a);
    data[i] = data[i] < 0 ? (f * -1.0f) : f;
  }
  return EAR_OK;
}

float ear_track_maximum(const float* data, int32_t first, int32_t last) {
  float x = 0.0f;
  for (int32_t i = first; i < last; ++i) {
    const float a = std::fabs(data[i]);
    if (a > x) x = a;
  }
  return x;
}

ear_status ear_track_multiply(float* data, int32_t first, int32_t last, float f) {
  if (!data && last > first) return fail(EAR_ERR_INVALID_ARG, "null track");
  for (int32_t i = first; i < last; ++i) data[i] *= f;
  return EAR_OK;
}

int32_t ear_track_length(const float* data, int32_t capacity, int32_t first, int32_t last,
                         float tresh) {
  if (tresh < 0.0f) return last;
  int32_t mx = 0;
  for (int32_t i = first; i < capacity; ++i)
    if (std::fabs(data[i]) >= tresh) mx = i;
  return mx + 1;
}

float ear_track_t60(const float* data, int32_t first, int32_t last) {
  const float attenuation_gain = std::pow(10.0f, 60.0f / 20.0f);
  float min_gain = 0.0f;
  int last_significant_offset = 0, direct_sound_offset = 0;
  float previous_sample = -1.0f;
  bool inside_indirect_lobe = false;
  for (int32_t j = first; j < last; ++j) {
    const float sample = data[j];
    if (inside_indirect_lobe) {
      if (sample > min_gain) last_significant_offset = j;
    } else if (sample < previous_sample) {
      inside_indirect_lobe = true;
      min_gain = previous_sample / attenuation_gain;
      direct_sound_offset = j;
    }
    previous_sample = sample;
  }
  return (float)(last_significant_offset - direct_sound_offset) / 44100.0f;
}

ear_status ear_statistical_t60(const float* vertices, const int64_t* block_triangles,
                               int32_t num_blocks, const ear_material* first_block_material,
                               float air_absorption_mid, float* out) {
  g_err[0] = 0;
  if (!vertices || !block_triangles || num_blocks <= 0 || !first_block_material || !out)
    return fail(EAR_ERR_INVALID_ARG, "bad arguments");
  DevMaterial m;
  if (!derive_material(*first_block_material, &m))
    return fail(EAR_ERR_INVALID_ARG, "Invalid material settings");
  // Mesh::Mesh: absorption = 1 - absorption_coefficient[1] (src/Mesh.cpp:85)
  const float absorption = 1.0f - m.survival[1];
  float total_area = 0.0f, weighted = 0.0f, volume = 0.0f;
  int64_t t = 0;
  for (int32_t b = 0; b < num_blocks; ++b) {
    float block_area = 0.0f;
    for (int64_t i = 0; i < block_triangles[b]; ++i, ++t) {
      const float* v = vertices + 9 * t;
      const V3 p1 = mk(v[0], v[1], v[2]), p2 = mk(v[3], v[4], v[5]), p3 = mk(v[6], v[7], v[8]);
      const float area = length(cross(sub(p2, p1), sub(p3, p2))) / 2.0f;
      block_area += area;
      if (b == 0) weighted += area * absorption;
      // Triangle::SignedVolume (src/Triangle.cpp:55-67)
      const float v321 = p3.x * p2.y * p1.z;
      const float v231 = p2.x * p3.y * p1.z;
      const float v312 = p3.x * p1.y * p2.z;
      const float v132 = p1.x * p3.y * p2.z;
      const float v213 = p2.x * p1.y * p3.z;
      const float v123 = p1.x * p2.y * p3.z;
      volume += (1.0f / 6.0f) * (-v321 + v231 + v312 - v132 - v213 + v123);
    }
    total_area += block_area;
  }
  const float V = volume, A = weighted, S = total_area, a = weighted / total_area;
  const float mm = air_absorption_mid;
  out[0] = V;
  out[1] = S;
  out[2] = A;
  out[3] = 0.1611f * V / (A + 4.0f * mm * V);
  out[4] = 0.1611f * V / (-S * std::log(1.0f - a) + 4.0f * mm * V);
  return EAR_OK;
}

}  // extern "C"

// ------------------------------------------------------------------------
// ear_render_noalloc: ear_render for callers that must not allocate.
//
// Everything the render needs beyond the caller's inputs and outputs (the
// recorder table, the FloatBuffer first/last bookkeeping, the path
// counters, the error flag and the direct-sound visibility flags) lives in
// one file-scope device array, so a call makes no cudaMalloc / cudaFree and
// no host heap allocation.  Histograms accumulate straight into the
// caller's device buffer.
namespace {

constexpr int kNoAllocScratchBytes = 16384;
constexpr size_t kNaCounters = 0;      // kNumCounters x u64 path counters
constexpr size_t kNaError = 96;        // error flag
constexpr size_t kNaRecs = 128;        // kMaxRecorders DevRecorder
constexpr size_t kNaVis = kNaRecs + sizeof(DevRecorder) * kMaxRecorders;
constexpr size_t kNaFirstLast = 2048;  // kMaxTracks x 3 int2
static_assert(kNaVis + sizeof(int) * kMaxRecorders <= kNaFirstLast, "no-alloc scratch layout");
static_assert(kNaCounters + sizeof(unsigned long long) * kNumCounters <= kNaError &&
                  kNaError + sizeof(int) <= kNaRecs,
              "no-alloc scratch layout");
static_assert(kNaFirstLast + sizeof(int2) * 3 * kMaxTracks <= (size_t)kNoAllocScratchBytes,
              "no-alloc scratch layout");

// Shared by every call on a device; holds the last call's contents.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

constexpr int kNoAllocMaxDevices = 64;
std::mutex g_noalloc_mu;
unsigned char* g_noalloc_ptr[kNoAllocMaxDevices] = {};

// Device address of the scratch array on `device` (which must be current).
// The first call per device resolves it with cudaGetSymbolAddress.
ear_status noalloc_scratch(int device, unsigned char** out) {
  if (device < 0 || device >= kNoAllocMaxDevices)
    return fail(EAR_ERR_INVALID_ARG, "device ordinal %d out of range", device);
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_ptr[device]) {
    void* ptr = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
    if (e != cudaSuccess)
      return fail(EAR_ERR_CUDA, "cudaGetSymbolAddress(no-alloc scratch): %s", cudaGetErrorString(e));
    g_noalloc_ptr[device] = static_cast<unsigned char*>(ptr);
  }
  *out = g_noalloc_ptr[device];
  return EAR_OK;
}

}  // namespace

extern "C" ear_status ear_render_noalloc(ear_scene* s, const ear_source* src,
                                         const ear_recorder* recs, int32_t nrec,
                                         const ear_render_params* p, float* hist,
                                         int32_t* first_sample, int32_t* last_sample,
                                         ear_render_stats* stats) {
  g_err[0] = 0;
  if (!s || !src || !p || !hist || (nrec > 0 && !recs))
    return fail(EAR_ERR_INVALID_ARG, "null argument");
  if (!s->bvh) return fail(EAR_ERR_STATE, "ear_scene_build_bvh has not been called");
  if (nrec < 0 || nrec > kMaxRecorders)
    return fail(EAR_ERR_INVALID_ARG,
                "ear_render_noalloc: %d recorders exceed its fixed scratch (at most %d)", nrec,
                kMaxRecorders);
  if (src->num_emitter_triangles != 0)
    return fail(EAR_ERR_UNSUPPORTED,
                "ear_render_noalloc: area emitters need per-call scratch; use ear_render");
  if (p->num_bins <= 0 || p->num_bins > (1 << 30) || (p->num_bins & 3))
    return fail(EAR_ERR_INVALID_ARG,
                "ear_render_noalloc: num_bins must be a positive multiple of 4 (got %d)",
                p->num_bins);
  if (((uintptr_t)hist) & 15)
    return fail(EAR_ERR_INVALID_ARG, "ear_render_noalloc: hist must be 16-byte aligned");
  if (p->bands_mask == 0 || (p->bands_mask & ~7u)) return fail(EAR_ERR_INVALID_ARG, "bad bands_mask");
  if (p->max_bounces < 0) return fail(EAR_ERR_INVALID_ARG, "negative max_bounces");
  if (p->traverse_budget < 0) return fail(EAR_ERR_INVALID_ARG, "negative traverse_budget");
  if (p->num_rays > (1ull << 47) || p->first_ray > (1ull << 47) - p->num_rays)
    return fail(EAR_ERR_INVALID_ARG, "first_ray + num_rays above 2^47");
  DevRecorder dr[kMaxRecorders];
  const int tracks = derive_recorders(recs, nrec, 0, 0, dr);
  if (tracks < 0) return EAR_ERR_INVALID_ARG;
  CU(cudaSetDevice(s->device));
  unsigned char* scratch = nullptr;
  ear_status rc = noalloc_scratch(s->device, &scratch);
  if (rc != EAR_OK) return rc;

  TraceArgs a;
  std::memset(&a, 0, sizeof a);
  const TraceOps* ops = (p->flags & EAR_FLAG_EXACT) ? &kTraceExact : &kTraceFast;
  a.nodes = s->ds.nodes;
  a.nodes4 = s->ds.nodes4;
  a.wide = s->ds.wide;
  a.any_far = s->ds.any_far;
  a.tris = s->ds.tris;
  a.num_tris = (int)s->ds.num_tris;
  a.num_nodes = (int)(s->ds.wide ? s->ds.num_nodes4 : s->ds.num_nodes);
  a.mats = s->mats;
  a.num_mats = s->num_mats;
  a.num_recs = nrec;
  DevRecorder* recs_dev = reinterpret_cast<DevRecorder*>(scratch + kNaRecs);
  a.recs = recs_dev;
  for (int k = 0; k < 3; ++k) a.src[k] = src->location[k];
  a.k0 = (uint32_t)p->seed;
  a.k1 = (uint32_t)(p->seed >> 32);
  a.context = p->context;
  int nb = 0;
  for (int b = 0; b < 3; ++b) {
    a.bands[b] = -1;
    if (p->bands_mask & (1u << b)) a.bands[nb++] = b;
    a.air[b] = 1.0f - p->air_absorption[b];
  }
  a.num_rays = p->num_rays;
  a.ray0 = p->first_ray;
  a.num_items = p->num_rays * (uint64_t)nb;
  a.max_bounces = p->max_bounces;
  a.cutoff = p->cutoff;
  a.box_pad = s->ds.box_pad;
  a.hist = hist;
  a.stride = p->num_bins;
  a.num_bins = p->num_bins;
  a.num_tracks = tracks;
  a.first_last = reinterpret_cast<int2*>(scratch + kNaFirstLast);
  const bool direct = !(p->flags & (EAR_FLAG_RAW | EAR_FLAG_NO_DIRECT)) && nrec > 0;
  a.direct_vis = direct ? reinterpret_cast<int*>(scratch + kNaVis) : nullptr;
  a.counters = reinterpret_cast<unsigned long long*>(scratch + kNaCounters);
  a.error_flag = reinterpret_cast<int*>(scratch + kNaError);
  a.traverse_budget = p->traverse_budget > 0 ? p->traverse_budget
                                             : traverse_budget(s->ds.wide ? s->ds.num_nodes4 : s->ds.num_nodes,
                                                               s->ds.wide != 0);
  a.dbg_band = -1;
  // listener visibility maps an earlier ear_render built for this recorder
  // set are read; none is built here (a build allocates)
  if (nrec > 0 && s->vis_opt >= 0 && s->vis_valid && !s->vis_refused && s->vis.cells) {
    const int res = s->vis_opt > 0 ? s->vis_opt : vis_auto_res(s->ds.num_tris);
    if (vis_map_key(s, recs, nrec, res) == s->vis_key) set_vis_args(s, a);
  }

  // launch limits are checked before any device work is queued, so a
  // rejected call leaves the caller's histogram and the scratch untouched
  const size_t smem = trace_smem_bytes(s->num_mats, tracks, kModeForward, ops->block);
  if (smem > 200 * 1024) return fail(EAR_ERR_INVALID_ARG, "too many materials for one launch");
  int per_sm = 0;
  CU(ops->occupancy(kModeForward, ops->block, smem, &per_sm));
  if (per_sm < 1) per_sm = 1;
  cudaStream_t st = (cudaStream_t)p->stream;
  const int rows = tracks * 3;
  // the shared scratch keeps the previous call's contents: clear it
  CU(cudaMemsetAsync(scratch, 0, kNaRecs, st));
  if (nrec) CU(cudaMemcpyAsync(recs_dev, dr, sizeof(DevRecorder) * nrec, cudaMemcpyHostToDevice, st));
  if (rows) {
    CU(cudaMemsetAsync(hist, 0, sizeof(float) * (size_t)rows * (size_t)p->num_bins, st));
    k_init_first_last<<<(rows + 127) / 128, 128, 0, st>>>(a.first_last, rows);
    CU(cudaGetLastError());
  }
  CU(cudaEventRecord(s->ev0, st));
  CU(ops->trace(a, a.num_items > 0 ? s->sm_count * per_sm : 1, ops->block, smem, kModeForward, st));
  CU(cudaEventRecord(s->ev1, st));
  if (!(p->flags & EAR_FLAG_RAW) && nrec > 0) {
    const float amount = p->num_rays <= 16777216ull ? (float)p->num_rays : 16777216.0f;
    FinalizeArgs f = {};
    f.hist = hist;
    f.stride = p->num_bins;
    f.num_bins = p->num_bins;
    f.first_last = a.first_last;
    f.recs = a.recs;
    f.direct_vis = a.direct_vis;
    for (int k = 0; k < 3; ++k) {
      f.src[k] = a.src[k];
      f.air[k] = a.air[k];
    }
    f.dry = p->dry_level;
    f.inv_amount = 1.0f / amount;
    f.gain2 = src->gain * src->gain;
    f.bands = p->bands_mask;
    k_finalize<<<nrec * 3, 256, 0, st>>>(f);
    CU(cudaGetLastError());
  }
  int2 fl[3 * kMaxTracks];
  unsigned long long cnt[kNumCounters];
  int errflag = 0;
  if (rows) CU(cudaMemcpyAsync(fl, a.first_last, sizeof(int2) * rows, cudaMemcpyDeviceToHost, st));
  CU(cudaMemcpyAsync(cnt, a.counters, sizeof cnt, cudaMemcpyDeviceToHost, st));
  CU(cudaMemcpyAsync(&errflag, a.error_flag, sizeof(int), cudaMemcpyDeviceToHost, st));
  CU(cudaStreamSynchronize(st));
  if (errflag & kErrIndex)
    return fail(EAR_ERR_CUDA, "internal: a device-side index check failed (corrupt BVH or scene data)");
  if (errflag & kErrBudget)
    return fail(EAR_ERR_DEVICE_BUDGET, "a BVH traversal exceeded its iteration budget");
  for (int i = 0; i < rows; ++i) {
    if (first_sample) first_sample[i] = std::min(fl[i].x, p->num_bins);
    if (last_sample) last_sample[i] = std::min(fl[i].y, p->num_bins);
  }
  if (stats) {
    float ms = 0.0f;
    CU(cudaEventElapsedTime(&ms, s->ev0, s->ev1));
    stats->rays = std::min<unsigned long long>(cnt[kWork], a.num_items);
    stats->segments = cnt[kSegments];
    stats->shadow_queries = cnt[kShadow];
    stats->contributions = cnt[kContrib];
    stats->sampler_overflows = cnt[kOverflow];
    stats->node_visits = cnt[kNodeVisits];
    stats->triangle_tests = cnt[kTriTests];
    stats->splat_bins = cnt[kSplatBins];
    stats->kernel_ms = ms;
    stats->map_entries = cnt[kMapEntries];
    stats->map_build_ms = 0.0;
    map_stats(s, a, stats);
  }
  return EAR_OK;
}
