/*
 * ear_gb300.h -- C ABI of the GB300 (sm_103a) acoustic ray-tracing core.
 *
 * This is the drop-in boundary for E.A.R's ray-tracing path.  The reference
 * (aothms/ear) has no plugin or FFI layer; its seam is the C++ method
 *
 *   void Scene::Render(int band, int sound, float absorbtion_factor,
 *                      int num_samples, float dry,
 *                      const std::vector<Recorder*>& rec, int keyframeID)
 *                                                   (src/Scene.h:77)
 *
 * called once per (source x keyframe x band) context by
 * SceneContext::operator() (src/SceneContext.h:46-48) from the thread groups
 * in Render() (src/EAR.cpp:193-207).  ear_render() below replaces that call
 * for all bands of one (source, keyframe) context at once; the inner seams
 * Mesh::RayIntersection / Mesh::LineIntersection (src/Mesh.h:54-55) are
 * exposed for parity testing through ear_trace_debug().
 *
 * Conventions
 *  - Plain C types only; every function returns an ear_status.  On failure
 *    ear_last_error() returns a thread-local message.
 *  - Bands are 0 = low, 1 = mid, 2 = high, as in the reference.
 *  - Histogram ("track") layout: float[num_tracks][3][num_bins], tracks in
 *    recorder order (a mono recorder owns 1 track, a stereo recorder 2:
 *    left then right, src/StereoRecorder.cpp:124-129).  Samples are at
 *    44.1 kHz (src/Recorder.h:35).
 *  - Output pointers are host memory unless ear_histograms.on_device is set.
 *  - A scene handle is not re-entrant; distinct handles may be used from
 *    distinct host threads.  All work is issued on ear_render_params.stream
 *    (NULL = the legacy default stream) and the call returns after it is
 *    complete.
 */
#ifndef EAR_GB300_H
#define EAR_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define EAR_ABI_VERSION 2
#define EAR_NUM_BANDS 3
#define EAR_SAMPLE_RATE 44100
/* Loop bound of Scene::Render: 1000 iterations = emission + 999 reflections
 * (src/Scene.cpp:143). */
#define EAR_REFERENCE_MAX_BOUNCES 999
/* Path cut-off of Scene::Render (src/Scene.cpp:275). */
#define EAR_REFERENCE_CUTOFF 1e-8

typedef enum ear_status {
  EAR_OK = 0,
  EAR_ERR_INVALID_ARG = 1,   /* bad pointer, size or value */
  EAR_ERR_OUT_OF_MEMORY = 2, /* device or host allocation failed */
  EAR_ERR_CUDA = 3,          /* a CUDA runtime call failed */
  EAR_ERR_DEVICE_BUDGET = 4, /* a device loop hit its iteration budget */
  EAR_ERR_STATE = 5,         /* e.g. ear_render before ear_scene_build_bvh */
  EAR_ERR_UNSUPPORTED = 6
} ear_status;

/* Render flags. */
#define EAR_FLAG_EXACT 0x1u      /* use the kernels compiled with --fmad=false:
                                    bit-exact with the CPU oracle */
#define EAR_FLAG_RAW 0x2u        /* return raw splat sums: no 1/N scaling, no
                                    direct sound, no gain (for split renders) */
#define EAR_FLAG_NO_DIRECT 0x4u  /* skip the direct-sound lobe only */

typedef struct ear_scene ear_scene; /* opaque: device geometry + LBVH */

/* One MAT block (src/Material.cpp:26-72).  Values are per band.  A block
 * without a refraction triplet is opaque (has_refraction = 0), one without
 * a specularity triplet has specularity 0 (the std::map default read at
 * src/Scene.cpp:163). */
typedef struct ear_material {
  float reflection[3];
  float refraction[3];
  float specularity[3];
  int32_t has_refraction;
  int32_t has_specularity;
} ear_material;

/* All MESH blocks merged in file order, as Scene::addMesh / Mesh::Combine
 * do (src/Scene.cpp:103-106, src/Mesh.cpp:116-123): triangle i of this
 * array is triangle i of the reference's meshes[0]->tris. */
typedef struct ear_scene_desc {
  int64_t num_triangles;
  const float* vertices;       /* host, num_triangles * 9 floats (v0 v1 v2) */
  const int32_t* material_ids; /* host, num_triangles indices into materials */
  int32_t num_materials;
  const ear_material* materials;
  int32_t device;              /* CUDA device ordinal */
} ear_scene_desc;

/* Acceleration options.  "Never changes a result" below means: every hit
   the triangle test reports within the padding of its triangle is found,
   exactly as the brute-force loops find it.  Only a segment grazing a
   triangle's plane can be reported hit farther out, by the test's own
   rounding; such artefacts are not guaranteed to be reproduced (none were
   seen on the test scenes). */
typedef struct ear_bvh_opts {
  /* Padding added to every triangle's bounding box, in scene units.  Values
     < 0 select the default (2^-18 of the largest absolute coordinate plus
     1e-5).  Padding only makes the culling conservative; it never changes
     which triangle is reported. */
  float box_pad;
  /* Subtrees of at most this many triangles (1..16; 0 = 1) become one leaf:
     fewer node visits, more triangle tests per visit.  Never changes which
     triangle is reported. */
  int32_t max_leaf_size;
  /* EAR_BVH_DEFAULT, EAR_BVH_LBVH (Morton-order linear BVH, Karras 2012) or
     EAR_BVH_PLOC (locally-ordered agglomerative clustering over the same
     Morton order, Meister and Bittner 2018: a tree of lower surface-area
     cost, single-triangle leaves).  Never changes which triangle is
     reported. */
  int32_t builder;
  int32_t ploc_radius;     /* PLOC search radius in positions (0 = 4) */
  /* Tree the traversal uses: 2 (binary), 4 (4-wide, built from the binary
     tree: fewer dependent node loads per query, costlier visits) or 0 =
     4-wide from 4096 triangles on.  Both trees are built; the choice can
     be changed later with ear_scene_set_bvh_width.  A 4-wide tree deeper
     than the 16 levels of its traversal trail is not kept: the scene then
     traverses its binary tree (ear_scene_bvh_width reports the tree in
     use).  Never changes a result. */
  int32_t width;
  /* Order of the visibility tests' traversal: 1 nearest hit child first, 2
     farthest first (meets occluders between the surface and the listener
     sooner), 0 = automatic: farthest first when a probe at build time
     finds more than 15% of 8192 segments between triangle pairs blocked.
     Never changes a result. */
  int32_t visibility_order;
  /* Listener visibility maps: per recorder location, a cube map of
     directions around it whose cells list the triangles (padded boxes) in
     their cone, nearest first.  A visibility test then runs the triangle
     test on its cell's entries nearer than the path vertex instead of
     traversing the tree; cells longer than a limit keep the traversal.  A
     render builds them on first use of a recorder set and keeps them until
     the set, the tree or this setting changes; a batch builds one per scene
     over its jobs' recorders.  > 0: on, with this many cells per face edge
     (8..4096; refused, the tests left to the tree, when the lists would
     not fit half the free device memory); -1: off; 0 = automatic: built
     for renders of at least as many rays (times bands) as the scene has
     triangles, with 4 sqrt(triangles) cells per edge (a multiple of 64,
     64..2816), lowered
     while the lists would hold more than EAR_VISMAP_AUTO_MAX_ENTRIES
     entries; used by any render while they match its recorder set.  Never
     changes a result. */
  int32_t visibility_map;
  int32_t reserved;
} ear_bvh_opts;

#define EAR_VISMAP_AUTO_MAX_ENTRIES (1ull << 30) /* 48 GiB of lists (48 B per entry) */

#define EAR_BVH_DEFAULT 0
#define EAR_BVH_LBVH 1
#define EAR_BVH_PLOC 2

/* OUT1 (mono, src/MonoRecorder.cpp:38-59) or OUT2 (stereo,
 * src/StereoRecorder.cpp:33-67) block, evaluated at the keyframe being
 * rendered (Animated<T>::Evaluate, src/Animated.h:89-91). */
typedef struct ear_recorder {
  int32_t channels;           /* 1 = mono, 2 = stereo */
  float location[3];
  float right_ear[3];         /* stereo only */
  float head_size;            /* stereo only */
  float head_absorption[3];   /* stereo only; the value written in the file,
                                 transformed as src/StereoRecorder.cpp:55-57 */
} ear_recorder;

/* SSRC / 3SRC block (src/SoundFile.cpp:33-70, 84-117) at one keyframe. */
typedef struct ear_source {
  float location[3];               /* point source */
  float gain;                      /* squared into the response, :313-314 */
  int64_t num_emitter_triangles;   /* > 0: area (mesh) emitter */
  const float* emitter_vertices;   /* host, num_emitter_triangles * 9 */
} ear_source;

typedef struct ear_render_params {
  uint64_t seed;           /* Philox-4x32-10 key */
  uint32_t context;        /* folded into every RNG counter: distinct
                              (source, keyframe) contexts use distinct ids */
  uint32_t bands_mask;     /* bit b set: trace band b */
  uint64_t num_rays;       /* rays per band (Scene::Render num_samples) */
  int32_t max_bounces;     /* maximum reflections per ray; the reference's
                              loop allows EAR_REFERENCE_MAX_BOUNCES */
  int32_t num_bins;        /* histogram length in samples */
  double cutoff;           /* path ends when intensity < cutoff */
  float air_absorption[3]; /* 'absorption' setting: factor = 1 - a (EAR.cpp:180) */
  float dry_level;         /* 'drylevel' setting */
  uint32_t flags;          /* EAR_FLAG_* */
  int32_t traverse_budget; /* node visits one BVH traversal may make; a
                              traversal that needs more stops, and the call
                              returns EAR_ERR_DEVICE_BUDGET once the launch
                              has ended (the kernel never waits unbounded).
                              0 = automatic: 8 x tree nodes + 64, more than
                              any traversal of a valid tree makes */
  void* stream;            /* cudaStream_t, NULL = default stream */
  uint64_t first_ray;      /* index of this call's first ray: rays
                              first_ray .. first_ray + num_rays - 1 are traced
                              (first_ray + num_rays <= 2^47).  A render split
                              by ray range over calls or GPUs, each with
                              EAR_FLAG_RAW, sums to the unsplit raw render;
                              the 1/N and gain^2 scaling is then applied once. */
} ear_render_params;

/* Selects the tree the traversal uses (2 or 4, see ear_bvh_opts.width)
   without rebuilding; EAR_ERR_STATE for 4 when no 4-wide tree was kept.
   No counterpart in the reference. */
ear_status ear_scene_set_bvh_width(ear_scene* scene, int32_t width);

/* The tree the traversal uses: *width = 2 (binary) or 4.  No counterpart
   in the reference. */
ear_status ear_scene_bvh_width(const ear_scene* scene, int32_t* width);

/* Per-render statistics (counted on the device). */
typedef struct ear_render_stats {
  uint64_t rays;           /* primary rays emitted */
  uint64_t segments;       /* closest-hit queries for bounces k >= 1 */
  uint64_t shadow_queries; /* any-hit (visibility) queries */
  uint64_t contributions;  /* valid recorded path contributions */
  uint64_t sampler_overflows; /* rejection loops that reached their bound */
  uint64_t node_visits;    /* BVH node visits in 64-byte units (a 4-wide
                              node counts 2) */
  uint64_t triangle_tests; /* ray/triangle tests (48 bytes of geometry each) */
  uint64_t splat_bins;     /* histogram bins written by splats */
  double kernel_ms;        /* device time of the trace kernel(s) */
  uint64_t map_entries;    /* listener visibility-map entries read (8 bytes
                              each; see ear_bvh_opts.visibility_map) */
  double map_build_ms;     /* time this call spent building visibility maps
                              (0 when they were reused or are off) */
  uint64_t map_bytes;      /* device bytes of the maps in use (0: none) */
  int32_t map_res;         /* their cells per face edge (0: none) */
  int32_t reserved1;
} ear_render_stats;

typedef struct ear_histograms {
  float* data;             /* [num_tracks][3][num_bins] */
  /* FloatBuffer bookkeeping per [track][band] (src/Recorder.cpp:43-59):
     first_sample = min(132299, smallest index written) and last_sample =
     max(0, largest index written) ("real_length"), both clamped to
     num_bins (num_bins = something was written beyond the window). */
  int32_t* first_sample;   /* optional, [num_tracks][3] */
  int32_t* last_sample;    /* optional, [num_tracks][3] */
  int32_t on_device;       /* data/first/last are device pointers */
  int32_t reserved0;
  /* optional: the same bookkeeping right after tracing, before the 1/N
     scaling and the direct sound (what ear_render_adjoint needs) */
  int32_t* raw_first_sample;
  int32_t* raw_last_sample;
} ear_histograms;

/* ---------------------------------------------------------------- errors */
const char* ear_last_error(void);
const char* ear_version(void);
int32_t ear_abi_version(void);

/* ----------------------------------------------------------------- scene */
/* Replaces the triangle soup of meshes[0] (src/Mesh.cpp:77-123) and the
   static material map (src/Mesh.cpp:178).  Uploads geometry to the device. */
ear_status ear_scene_create(const ear_scene_desc* desc, ear_scene** out);
/* Builds the LBVH on the device.  New: the reference has no acceleration
   structure (src/Scene.h:37-41); brute force is in src/Mesh.cpp:33-71. */
ear_status ear_scene_build_bvh(ear_scene* scene, const ear_bvh_opts* opts);
/* Node count, depth, padding actually used, device bytes. */
ear_status ear_scene_info(const ear_scene* scene, int64_t* num_triangles,
                          int64_t* num_nodes, int32_t* max_depth,
                          float* box_pad, int64_t* device_bytes);

/* Surface-area-heuristic cost of the built tree (width 2: binary, 4:
   4-wide): node_cost per entered internal node plus triangle_cost per
   triangle of an entered leaf, each weighted by its box area over the
   root's, plus the root.  A tree-quality figure to read beside segments/s:
   a worse tree inflates the node and triangle fetches per segment. */
ear_status ear_scene_sah_cost(const ear_scene* scene, int32_t width, float node_cost,
                              float triangle_cost, double* cost);
void ear_scene_destroy(ear_scene* scene);

/* Number of tracks the recorders produce (1 per mono, 2 per stereo). */
int32_t ear_num_tracks(const ear_recorder* recorders, int32_t num_recorders);

/* ---------------------------------------------------------------- render */
/* Replaces Scene::Render (src/Scene.cpp:111-318) for every band in
   params->bands_mask of one (source, keyframe) context.  Tracks of bands not
   in the mask are zeroed.  stats may be NULL. */
ear_status ear_render(ear_scene* scene, const ear_source* source,
                      const ear_recorder* recorders, int32_t num_recorders,
                      const ear_render_params* params, ear_histograms* out,
                      ear_render_stats* stats);

/* Parity probe: traces the same paths as ear_render (same kernel code) for
   band `band` and records, for ray r < num_rays and reflection k in
   [1, max_record]: hit_tri[r*max_record + k-1] = original index of the
   triangle hit (-1 = miss, -2 = path already ended), bounce_type[...] =
   0 REFLECT / 1 REFRACT (src/Material.cpp:76-83), visible[...] = bit j set
   when recorder j is connected (src/Scene.cpp:84-96).  Host pointers. */
ear_status ear_trace_debug(ear_scene* scene, const ear_source* source,
                           const ear_recorder* recorders,
                           int32_t num_recorders,
                           const ear_render_params* params, int32_t band,
                           int32_t max_record, int32_t* hit_tri,
                           uint8_t* bounce_type, uint32_t* visible);

/* Replaces the MAT table of an existing scene (same count, same order)
   without touching the geometry or the LBVH -- for optimisation loops over
   material coefficients.  New: the reference's materials are fixed at parse
   time (src/Scene.cpp:107-109). */
ear_status ear_scene_set_materials(ear_scene* scene,
                                   const ear_material* materials,
                                   int32_t num_materials);

/* Path-replay adjoint of ear_render.  New: the reference has no
   derivatives.  With every material parameterised by its per-band
   absorption a and refraction r (reflection = 1 - a - r), returns
   grad[material][band][0 = a, 1 = r] = d/d(a, r) of sum(d_hist * h), h being
   the histograms ear_render produces with the same arguments (same seed,
   same context: the same paths are re-traced, nothing is stored).  The
   estimator is exact for the survival product along each path (pathwise)
   and unbiased for the REFLECT/REFRACT choices (score function); the path
   cut-off is held fixed.  d_hist: [num_tracks][3][num_bins], host or device
   (d_hist_on_device).  Unless EAR_FLAG_RAW is set, the finalize scaling is
   differentiated too, which needs the forward's bookkeeping:
   raw_first/raw_last (ear_histograms.raw_*) and first/last.  At most 32
   materials.  grad: host, num_materials * 6 doubles. */
ear_status ear_render_adjoint(ear_scene* scene, const ear_source* source,
                              const ear_recorder* recorders,
                              int32_t num_recorders,
                              const ear_render_params* params,
                              const float* d_hist, int32_t d_hist_on_device,
                              const int32_t* raw_first, const int32_t* raw_last,
                              const int32_t* first, const int32_t* last,
                              double* grad, ear_render_stats* stats);

/* ---------------------------------------------------------- batches
 * Many renders -- rooms (scenes) x source/listener pairs x keyframes x
 * bands -- traced by ONE persistent launch that pulls (job, band, ray) work
 * items from a device counter, replayed as a captured CUDA graph.  No
 * counterpart in the reference, which renders one (source, keyframe, band)
 * per Scene::Render call (src/EAR.cpp:225-243); every job of a batch gives
 * the same rays as ear_render with the batch's seed and the job's context,
 * scene, source and recorders. */
typedef struct ear_batch ear_batch;

typedef struct ear_batch_job {
  int32_t scene;                 /* index into the scenes of ear_batch_create */
  int32_t num_recorders;         /* 1..32 */
  const ear_recorder* recorders; /* host; evaluated at this job's keyframe */
  float source[3];               /* point source position at the keyframe */
  float gain;                    /* SSRC gain, squared into the response */
  uint64_t num_rays;             /* rays per band (> 0) */
  uint32_t context;              /* RNG context, as ear_render_params.context */
  int32_t reserved;
} ear_batch_job;

/* Launch schedule of a batch; every field 0 selects the default. */
typedef struct ear_batch_config {
  int32_t block;          /* threads per block: 32..256, multiple of 32 (256) */
  int32_t blocks_per_sm;  /* resident blocks per SM, i.e. rays in flight per
                             SM; capped at the occupancy limit (limit) */
  int32_t max_leaf_size;  /* BVH leaf size the batch's scenes are built with;
                             set by ear_batch_tune (read-only otherwise) */
  int32_t no_graph;       /* 1: launch directly instead of replaying the
                             captured CUDA graph */
  int32_t bvh_width;      /* tree width the batch's scenes traverse (2 or 4:
                             the 4-wide tree of every scene that kept one);
                             set by ear_batch_tune, 0 = the scenes' own */
  int32_t reserved[3];
} ear_batch_config;

/* Plans a batch: validates the jobs, derives the recorder constants,
   allocates the device job tables and one histogram row per (job, track,
   band).  The scenes (with their LBVH built, all on one device) must
   outlive the batch.  From `params`: seed, bands_mask, max_bounces,
   num_bins, cutoff, air_absorption, dry_level, flags (EXACT, RAW,
   NO_DIRECT) and stream; num_rays and context come from each job. */
ear_status ear_batch_create(ear_scene* const* scenes, int32_t num_scenes,
                            const ear_batch_job* jobs, int32_t num_jobs,
                            const ear_render_params* params, ear_batch** out);
ear_status ear_batch_set_config(ear_batch* batch, const ear_batch_config* config);
ear_status ear_batch_get_config(const ear_batch* batch, ear_batch_config* config);
/* Moves every job's point source ([num_jobs][3], host) without re-planning;
   the next run replays the same graph. */
ear_status ear_batch_set_sources(ear_batch* batch, const float* positions);
/* Renders every job (histograms stay on the device) and waits for it.
   stats (optional) sums the batch; kernel_ms is the device time of the
   whole launch sequence. */
ear_status ear_batch_run(ear_batch* batch, ear_render_stats* stats);
/* Job `job`'s finalized tracks after ear_batch_run, as ear_render returns
   them (raw_first_sample / raw_last_sample are not reported). */
ear_status ear_batch_histograms(const ear_batch* batch, int32_t job, ear_histograms* out);
/* Device view of all rows: data[row * stride + bin], rows = 3 * tracks of
   the batch; job `job`'s rows start at 3 * first_track[job]. */
ear_status ear_batch_device_view(const ear_batch* batch, const float** data, int32_t* stride,
                                 int64_t* rows, int32_t* first_track, int32_t max_jobs);
void ear_batch_destroy(ear_batch* batch);

/* One-shot: ear_batch_create + ear_batch_run + ear_batch_histograms for
   every job (outs[num_jobs]) + ear_batch_destroy. */
ear_status ear_render_batch(ear_scene* const* scenes, int32_t num_scenes,
                            const ear_batch_job* jobs, int32_t num_jobs,
                            const ear_render_params* params, ear_histograms* outs,
                            ear_render_stats* stats);

/* Autotuner.  Times trial launches of the batch -- every job with a
   fraction of its rays -- over the schedule space (block size x blocks per
   SM, and with tune_leaf_size the BVH leaf size, which rebuilds the
   batch's scenes; with tune_width the binary or 4-wide tree) and applies
   the fastest.  With cache_path, results are
   kept in that text file under a key of the device and the batch's shape
   and are reused without timing. */
typedef struct ear_tune_opts {
  double trial_fraction;   /* of each job's rays per trial (0 = 0.02) */
  uint64_t min_trial_rays; /* per job and trial (0 = 256) */
  int32_t tune_leaf_size;  /* 1: also try leaf sizes 1, 2, 4 */
  int32_t repeats;         /* timed runs per candidate, best kept (0 = 2) */
  const char* cache_path;  /* NULL: no persistent cache */
  int32_t tune_width;      /* 1: also try binary and 4-wide traversal */
  int32_t reserved[3];
} ear_tune_opts;

typedef struct ear_tune_result {
  ear_batch_config best;
  float best_ms;      /* trial time of the chosen schedule */
  float default_ms;   /* trial time of the default schedule */
  int32_t candidates; /* schedules timed */
  int32_t from_cache; /* 1: taken from cache_path without timing */
} ear_tune_result;

ear_status ear_batch_tune(ear_batch* batch, const ear_tune_opts* opts, ear_tune_result* result);

/* ear_render without any allocation.  No counterpart in the reference.
   For callers that must not allocate while rendering: an audio engine that
   re-renders an impulse response from its real-time thread when a listener
   moves cannot take the unbounded latency and device-wide synchronisation
   of cudaMalloc / cudaFree, and a host that runs the tracer inside a fixed
   GPU memory budget cannot let the library grow its own buffers.  The scene
   handle (created beforehand) and `hist` are the caller's; every other
   buffer the render needs lives in one statically sized device array
   (16 KiB: the recorder table, counters and per-track bookkeeping), so the
   call makes no cudaMalloc, cudaFree or host heap allocation.
   - hist: DEVICE pointer, 16-byte aligned, float[num_tracks][3][num_bins];
     it is zeroed and accumulated in place.  num_bins must be a multiple
     of 4.  first_sample / last_sample / stats are optional HOST pointers
     laid out as in ear_histograms / ear_render_stats.
   - Limits: at most 32 recorders (64 tracks); point sources only (an area
     emitter needs per-call scratch: EAR_ERR_UNSUPPORTED).  Larger requests
     are rejected with EAR_ERR_INVALID_ARG and a message.
   - The call returns only after the render has completed: it reads the
     path counters and the error flag back and synchronises `stream`
     before returning, whether or not first_sample / last_sample / stats
     are requested.  A real-time caller should run it from a worker
     thread, not from the audio callback itself.
   - The first call on a device resolves the array's device address
     (cudaGetSymbolAddress) with that device current; make that first call
     before any stream capture.  The address is cached for the life of
     the process: after cudaDeviceReset (or any other teardown of the
     device's primary context) the cached address is stale, so do not call
     this entry point again in that process.
   - The array is shared by every call on the device and keeps the last
     call's contents (each call clears what must start at zero).  Calls
     whose GPU work overlaps -- e.g. on two streams -- race on it: serialise
     them.
   - Listener visibility maps (ear_bvh_opts.visibility_map) are read when
     an earlier ear_render built them for the same recorder set, never
     built here: render once with ear_render before going real-time. */
ear_status ear_render_noalloc(ear_scene* scene, const ear_source* source,
                              const ear_recorder* recorders,
                              int32_t num_recorders,
                              const ear_render_params* params, float* hist,
                              int32_t* first_sample, int32_t* last_sample,
                              ear_render_stats* stats);

/* --------------------------------------- host post-processing (FloatBuffer)
 * Mirrors of FloatBuffer / RecorderTrack (src/Recorder.cpp:33-118, 303-340)
 * on one track.  `first`/`last` are the bookkeeping values above; the track
 * buffer holds `capacity` samples.  Host memory. */
/* FloatBuffer::Power, src/Recorder.cpp:103-108 */
ear_status ear_track_power(float* data, int32_t first, int32_t last, float a);
/* FloatBuffer::Maximum, src/Recorder.cpp:76-83 */
float ear_track_maximum(const float* data, int32_t first, int32_t last);
/* FloatBuffer::Multiply, src/Recorder.cpp:85-89 */
ear_status ear_track_multiply(float* data, int32_t first, int32_t last, float f);
/* FloatBuffer::getLength(tresh), src/Recorder.cpp:110-118 */
int32_t ear_track_length(const float* data, int32_t capacity, int32_t first,
                         int32_t last, float tresh);
/* RecorderTrack::T60, src/Recorder.cpp:303-340 */
float ear_track_t60(const float* data, int32_t first, int32_t last);

/* Sabine and Norris-Eyring predictions of src/EAR.cpp:264-284.  The
   vertices are the merged MESH blocks (block_triangles[i] triangles each, in
   file order); as in the reference, the volume and area cover every block
   but the total absorption only the first block, whose MAT is
   first_block_material (Mesh::Combine does not add it, src/Mesh.cpp:116-123).
   out[5] = {volume, area, total absorption, sabine, eyring}. */
ear_status ear_statistical_t60(const float* vertices,
                               const int64_t* block_triangles,
                               int32_t num_blocks,
                               const ear_material* first_block_material,
                               float air_absorption_mid, float* out);

/* ------------------------------------------------------------ auralisation
 * The steps of Render() after the impulse responses (src/EAR.cpp:295-386):
 * the band split of each dry sound (SoundFile::Band, src/SoundFile.cpp:
 * 149-160) and the convolution of every recorder track with the dry bands
 * (RecorderContext -> Recorder::Process -> RecorderTrack::Process, then
 * Recorder::Add; src/SceneContext.h:59-73, src/Recorder.cpp:136-292,
 * 343-363, 432-441).  Both run on the GPU.  Pointers are host memory unless
 * EAR_AURAL_DEVICE_MEMORY is set in `flags`; then every pointer is device
 * memory and the work is issued on `stream` (the call still returns after it
 * is complete). */
#define EAR_AURAL_DEVICE_MEMORY 1u

/* Equalizer::Split (lib/equalizer/Equalizer.cpp:81-96) as SoundFile::Band
   calls it: 4th-order Linkwitz-Riley low/high passes at the crossovers
   (f1+f2)/2 and (f2+f3)/2, with f = freq_khz * 1000 (the FREQ block; the
   reference's defaults are 0.2, 1.0 and 2.0 kHz, src/SoundFile.cpp:238-240).
   low = LP(x), high = HP(x), mid = HP(LP(x)) at the two crossovers.  The
   results are bit-identical to the reference's sequential filters, which
   run one sample after another.  With EAR_SPLIT_CHUNKED in `flags` the
   filters run in parallel over chunks of 512 samples (a chunk's response
   from a zero feedback state plus the propagated entry state): the first
   chunk is bit-identical; after it the result keeps the accuracy of the
   FP32 filters (the reference's own sequential FP32 output drifts up to
   ~1e-3 of the peak from exact arithmetic in the low band) without their
   exact rounding. */
#define EAR_SPLIT_CHUNKED 2u
ear_status ear_band_split(const float* dry, int64_t n, const float freq_khz[3],
                          float* low, float* mid, float* high, uint32_t flags,
                          void* stream, int32_t device);

/* Convolution modes of RecorderTrack::Process. */
#define EAR_CONV_FFT 0    /* builds with FFTW (src/Recorder.cpp:145-243): the
                             zero-padded product of transforms; a keyframe pair
                             fades the dry section out under this keyframe's
                             response and in under the next one's */
#define EAR_CONV_DIRECT 1 /* builds without FFTW (src/Recorder.cpp:247-292):
                             the O(N*M) sum, bit-identical to the reference's
                             loop order; a keyframe pair interpolates the two
                             responses linearly over the section */

/* One RecorderContext applied to one recorder track: the response `ir`
   convolved with a section of one band of a dry sound.  The track fields are
   the FloatBuffer bookkeeping after Power(0.335) and the truncation at
   max/256 (src/EAR.cpp:209-228): samples [first, length) are the response
   (the direct mode reads [first, length), the FFT mode [0, length)).
   `capacity` samples are readable at ir; reads beyond it are 0, as the const
   FloatBuffer::operator[] (src/Recorder.cpp:61-66). */
typedef struct ear_conv_context {
  const float* ir;
  int64_t ir_capacity;
  int64_t ir_first;
  int64_t ir_length;
  /* next keyframe's response of the same track and band, or NULL
     (Recorder::Process(sf, r, offset, length), src/Recorder.cpp:352-363) */
  const float* ir_next;
  int64_t ir_next_capacity;
  int64_t ir_next_first;
  int64_t ir_next_length;
  const float* dry;   /* the section: SoundFile::Section, src/SoundFile.cpp:164-173 */
  int64_t dry_length; /* its sample_length (0: an empty section) */
  int64_t offset;     /* its SoundFile::offset: output index of dry sample 0 */
} ear_conv_context;

typedef struct ear_conv_stats {
  float kernel_ms;        /* device time of the convolution kernels */
  int32_t launches;       /* kernels launched */
  int64_t fft_points;     /* FFT mode: sum of the transform sizes */
  double multiply_adds;   /* direct mode: terms of the reference's sums, n * (len - first) per context */
} ear_conv_stats;

/* out[x] += sum over contexts c (in order) of processed_c[x - ...] for x in
   [0, out_length): each context's RecorderTrack::Process result is formed
   on its own and then added, as Recorder::Add sums the processed tracks of
   the (source x keyframe x band) contexts of one recorder
   (src/EAR.cpp:359-377).  In EAR_CONV_DIRECT mode the sums are
   bit-identical to the reference; in EAR_CONV_FFT mode they agree to FP32
   transform accuracy.  stats may be NULL. */
ear_status ear_convolve(const ear_conv_context* contexts, int32_t num_contexts,
                        int32_t mode, float* out, int64_t out_length,
                        uint32_t flags, void* stream, int32_t device,
                        ear_conv_stats* stats);

/* ear_convolve for several output tracks in one call (e.g. every track of
   every recorder): context i is added to output track context_track[i]
   (NULL: all to track 0), each track's contexts in their order in the
   array.  outs[t] holds out_lengths[t] samples.  Host buffers shared by
   several contexts are copied to the device once.  At most 65535 tracks. */
ear_status ear_convolve_tracks(const ear_conv_context* contexts,
                               const int32_t* context_track, int32_t num_contexts,
                               int32_t mode, float* const* outs,
                               const int64_t* out_lengths, int32_t num_tracks,
                               uint32_t flags, void* stream, int32_t device,
                               ear_conv_stats* stats);

/* The FloatBuffer capacity (src/Recorder.cpp:33-59, INITIAL 3 s, growth by
   1 s: src/Recorder.h:36-37) of the track RecorderTrack::Process returns for
   one context in `mode`.  Recorder::Add reads that many samples, so the
   processed recorder track ends at max over its contexts of this value,
   minus one (the WAV length of RecorderTrack::Save). */
int64_t ear_conv_processed_capacity(const ear_conv_context* context, int32_t mode);

/* The FloatBuffer real_length of that track: the highest index
   RecorderTrack::Process wrote (0 when it wrote none).  A context's own
   processed recorder (the debugdir dumps of src/EAR.cpp:362-372) saves this
   many samples. */
int64_t ear_conv_processed_length(const ear_conv_context* context, int32_t mode);

#ifdef __cplusplus
}
#endif

#endif /* EAR_GB300_H */
