// trace_impl.cuh -- the sm_103a bounce-loop kernel.  Included twice:
// trace_exact.cu (EAR_NS = exact, --fmad=false: bit-identical to the CPU
// restatement) and trace_fast.cu (EAR_NS = fast, FMA contraction allowed).
//
// Replaces the per-ray loop of Scene::Render (src/Scene.cpp:124-284) and
// the two brute-force triangle loops it calls (src/Mesh.cpp:33-71).
//
// Structure: a persistent kernel; every warp keeps 32 independent rays in
// flight.  Each loop iteration advances every live lane by one bounce
// (closest hit, material choice, new direction, R visibility queries and
// splats).  Lanes whose path ended are refilled from a global work counter
// with one atomic per warp (ballot + popc + shuffle), so warps stay full
// while path lengths vary from 1 to max_bounces.  Warps reconverge
// (__syncwarp) after every data-dependent loop.  BVH traversal is
// stackless: over the binary tree a 64-bit trail records, per level of the
// current root path, whether the far child is still pending; over the
// 4-wide tree a 128-bit trail holds the mask of pending children per
// level; backtracking climbs parent links.
//
// Batch mode (kModeBatch) runs the same loop over many jobs -- (scene,
// source position, recorders) triples of a sweep over rooms, source /
// listener pairs and keyframes -- from one work counter: a refilled lane
// finds its job by binary search over the jobs' cumulative item ends and
// keeps the job's scene, RNG context and recorder range in registers; the
// scenes' node / triangle pointers come from a table in shared memory.
#pragma once

#ifndef EAR_NS
#error "EAR_NS must name the instantiation namespace"
#endif

#include <limits.h>

#include "ear_internal.h"
#include "ear_record.cuh"
#include "vismap_geom.h"

namespace ear {
namespace EAR_NS {

constexpr unsigned kFull = 0xffffffffu;

// The fast kernels (trace_fast.cu, EAR_FAST_MATH) use the special-function
// unit for powers and are compiled with approximate division; the exact
// kernels keep IEEE operations throughout.
#ifdef EAR_FAST_MATH
constexpr bool kFastMath = true;
#else
constexpr bool kFastMath = false;
#endif

// Relative widening of the t-range culling (2^-16, about 128 ulp of t):
// the slab distances and the triangle test round independently, so a box
// whose entry distance rounds just above the current best hit must not be
// culled.  The boxes' own padding covers the rounding in space.
constexpr float kSlackRel = 1.52587890625e-5f;

// A ray for the slab tests: 1/d and -o/d, so each plane distance
// t = (plane - o) / d is one fused multiply-add, plane * (1/d) + (-o/d).
// Its rounding differs from (plane - o) * (1/d) by a few ulp of the
// coordinates, far inside the boxes' padding: culling stays conservative.
struct Ray {
  float ix, iy, iz;
  float nx, ny, nz;
};

__device__ __forceinline__ float safe_inv(float d) {
  // 1/d with components below 1e-30 in magnitude (zero included) replaced
  // by +-1e-30, so slabs stay finite and 1/d keeps d's sign.
  const float dd = (fabsf(d) >= 1e-30f) ? d : copysignf(1e-30f, d);
  return 1.0f / dd;
}

__device__ __forceinline__ Ray make_ray(V3 o, V3 d) {
  Ray r;
  r.ix = safe_inv(d.x);
  r.iy = safe_inv(d.y);
  r.iz = safe_inv(d.z);
  r.nx = -(o.x * r.ix);
  r.ny = -(o.y * r.iy);
  r.nz = -(o.z * r.iz);
  return r;
}

// Slab test against [lo, hi] for t in [tmin, tmax] (0 <= tmin < tmax, tmin
// given by its bits); conservative only.  The entry distance tn = max(min
// x, min y, min z, tmin) and exit distance tf = min(max x, max y, max z,
// tmax) use 3-input integer min/max
// on the float bit patterns: signed-integer order equals float order among
// non-negative floats and puts every negative float below them, so the
// relu max gives tn exactly, and tf, which is only compared with tn >= 0,
// keeps its sign.
__device__ __forceinline__ bool box_hit(float lx, float hx, float ly, float hy, float lz, float hz,
                                        const Ray& r, float tmax, int tmin_bits, float& tnear) {
  const float tx0 = __fmaf_rn(lx, r.ix, r.nx), tx1 = __fmaf_rn(hx, r.ix, r.nx);
  const float ty0 = __fmaf_rn(ly, r.iy, r.ny), ty1 = __fmaf_rn(hy, r.iy, r.ny);
  const float tz0 = __fmaf_rn(lz, r.iz, r.nz), tz1 = __fmaf_rn(hz, r.iz, r.nz);
  const int tn = __vimax3_s32(__vimax_s32_relu(__float_as_int(fminf(tx0, tx1)),
                                               __float_as_int(fminf(ty0, ty1))),
                              __float_as_int(fminf(tz0, tz1)), tmin_bits);
  const int tf = __vimin3_s32(__float_as_int(fmaxf(tx0, tx1)), __float_as_int(fmaxf(ty0, ty1)),
                              __float_as_int(fminf(fmaxf(tz0, tz1), tmax)));
  tnear = __int_as_float(tn);
  return tn <= tf;
}

// The same test with each axis's near and far plane chosen by the sign of
// the ray's direction (the octant): the plane nearer along the ray is the
// low one for a positive direction, the high one for a negative, so the
// slab distances need no per-axis min / max.  Equal to box_hit's
// distances, which take that min / max of the same two values.
__device__ __forceinline__ bool box_hit_nf(float nx, float fx, float ny, float fy, float nz, float fz,
                                           const Ray& r, float tmax, int tmin_bits, float& tnear) {
  const float a = __fmaf_rn(nx, r.ix, r.nx), b = __fmaf_rn(ny, r.iy, r.ny);
  const float c = __fmaf_rn(nz, r.iz, r.nz);
  const float x = __fmaf_rn(fx, r.ix, r.nx), y = __fmaf_rn(fy, r.iy, r.ny);
  const float z = __fmaf_rn(fz, r.iz, r.nz);
  const int tn = __vimax3_s32(__float_as_int(a), __float_as_int(b),
                              max(__float_as_int(c), tmin_bits));
  const int tf = __vimin3_s32(__float_as_int(x), __float_as_int(y), __float_as_int(fminf(z, tmax)));
  tnear = __int_as_float(tn);
  return tn <= tf;
}

// Moller & Trumbore (1997), non-culling branch, same operation order as the
// CPU restatement of gmtl::intersectDoubleSided (src/Mesh.cpp:40,65).
__device__ __forceinline__ bool mt_intersect(const float4& A, const float4& B, const float4& C,
                                             V3 o, V3 d, float& t) {
  const V3 e1 = mk(B.x, B.y, B.z), e2 = mk(C.x, C.y, C.z);
  const V3 pvec = cross(d, e2);
  const float det = dot(e1, pvec);
  if (det > -1e-6f && det < 1e-6f) return false;
#if EAR_FAST_TRIANGLE_TEST
  // fast kernels: the barycentric bounds are compared unscaled, u*det and
  // v*det against det, so only accepted candidates pay the division
  const V3 tvec = sub(o, mk(A.x, A.y, A.z));
  const float un = dot(tvec, pvec);
  const V3 qvec = cross(tvec, e1);
  const float vn = dot(d, qvec);
  if (det > 0.0f) {
    if (un < 0.0f || un > det || vn < 0.0f || un + vn > det) return false;
  } else {
    if (un > 0.0f || un < det || vn > 0.0f || un + vn < det) return false;
  }
  t = dot(e2, qvec) / det;
  return true;
#else
  const float inv_det = 1.0f / det;
  const V3 tvec = sub(o, mk(A.x, A.y, A.z));
  const float u = dot(tvec, pvec) * inv_det;
  if (u < 0.0f || u > 1.0f) return false;
  const V3 qvec = cross(tvec, e1);
  const float v = dot(d, qvec) * inv_det;
  if (v < 0.0f || u + v > 1.0f) return false;
  t = dot(e2, qvec) * inv_det;
  return true;
#endif
}

// 32-byte read-only load (sm_100+ `ld.global.nc.v8`): a 4-wide node is 4
// of them, a binary node 2, instead of 8 and 4 16-byte loads -- half the L1
// wavefronts for the scattered node fetches of a warp.  p is 32-byte aligned.
__device__ __forceinline__ void ldg256(const void* p, float4& a, float4& b) {
  asm("ld.global.nc.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
      : "=f"(a.x), "=f"(a.y), "=f"(a.z), "=f"(a.w), "=f"(b.x), "=f"(b.y), "=f"(b.z), "=f"(b.w)
      : "l"(p));
}

__device__ __forceinline__ int4 as_int4(const float4& v) {
  return make_int4(__float_as_int(v.x), __float_as_int(v.y), __float_as_int(v.z),
                   __float_as_int(v.w));
}

struct Hit {
  float t;
  int pos;   // leaf-order position, -1 = none
  int orig;  // original (file-order) index
};

struct LaneCounters {
  uint32_t segments, shadow, contrib, overflow, nodes, tris, bins, map;
};

// Indices read from device data (child and parent links, leaf ranges, hit
// positions, material ids) are range-checked before they address memory.
// A failed check sets kErrIndex in `err` and clamps the index to 0 -- no
// early exit, so the warp keeps its shape; the launch then fails with
// EAR_ERR_CUDA instead of touching memory outside the scene.
__device__ __forceinline__ int clamp_index(int idx, int n, int& err) {
  const bool b = (unsigned)idx >= (unsigned)n;
  if (b) err |= kErrIndex;
  return b ? 0 : idx;
}

// Returns true (ANY) when the segment is blocked.
template <bool ANY>
__device__ __forceinline__ bool leaf_test(const SceneRef& S, int code, V3 o, V3 d, Hit& h,
                                          LaneCounters& c, int& err) {
  int start = (~code) & kLeafStartMask;
  int cnt = ((~code) >> kLeafCountShift) + 1;
  if ((unsigned)(start + cnt - 1) >= (unsigned)S.num_tris) {
    err |= kErrIndex;
    start = 0;
    cnt = 1;
  }
  c.tris += (uint32_t)cnt;
  bool blocked = false;
  for (int k = 0; k < cnt; ++k) {
    const float4* T = S.tris + 4 * (start + k);
    float4 A, B, C, Nn;
    ldg256(T, A, B);
    ldg256(T + 2, C, Nn);
    float t;
    if (mt_intersect(A, B, C, o, d, t)) {
      if (ANY) {
        // Mesh::LineIntersection: 1e-5 < t < 1 (src/Mesh.cpp:65)
        blocked |= (t > 1e-5f && t < 1.0f);
      } else {
        // Mesh::RayIntersection: t > 0.001, strict t < d, lowest index on
        // ties (src/Mesh.cpp:40) == lexicographic min of (t, index).
        const int orig = __float_as_int(A.w);
        if (t > 0.001f && (t < h.t || (t == h.t && orig < h.orig))) {
          h.t = t;
          h.pos = start + k;
          h.orig = orig;
        }
      }
    }
  }
  return blocked;
}

__device__ __forceinline__ float lane4(const float4& v, int k) {
  return k == 0 ? v.x : (k == 1 ? v.y : (k == 2 ? v.z : v.w));
}
__device__ __forceinline__ int lane4(const int4& v, int k) {
  return k == 0 ? v.x : (k == 1 ? v.y : (k == 2 ? v.z : v.w));
}

// Stackless traversal of the binary tree.  Closest hit (ANY = false): h
// receives the hit.
// Any hit (ANY = true): returns true when blocked.  `slack` widens the
// t-range culling so rounding in the slab test never removes a candidate.
template <bool ANY>
__device__ bool traverse2(const SceneRef& S, V3 o, V3 d, float tlimit, float slack, Hit& h,
                          LaneCounters& c, int& err) {
  h.t = tlimit;
  h.pos = -1;
  h.orig = INT_MAX;
  if (S.num_tris == 0) return false;
  const Ray r = make_ray(o, d);
  // closest hit: only t > 0.001 counts (src/Mesh.cpp:40), so boxes the
  // ray leaves before 0.001 - slack hold no hit (slack = the boxes' padding
  // covers the rounding of the slab distances, as on the far side); the
  // boxes around the ray's origin on its surface are culled at once
  const int tmin_bits = ANY ? 0 : __float_as_int(fmaxf(0.001f - slack, 0.0f));
  int cur = 0;
  unsigned long long trail = 1ull;
  int iters = 0;
  const Node* __restrict__ nodes = S.nodes2;
  bool blocked = false;
  const int err0 = err;
  for (;;) {
    if (++iters > S.traverse_budget) {
      err |= kErrBudget;
      break;
    }
    cur = clamp_index(cur, S.num_nodes, err);
    const Node* nd = nodes + cur;
    float4 na, nb, nc, nd4;
    ldg256(&nd->a, na, nb);
    ldg256(&nd->c, nc, nd4);
    const int4 ch = as_int4(nd4);
    const float lim = ANY ? tlimit + slack : h.t + (h.t * kSlackRel + slack);
    float t0, t1;
    bool h0 = box_hit(na.x, na.y, na.z, na.w, nb.x, nb.y, r, lim, tmin_bits, t0);
    bool h1 = box_hit(nb.z, nb.w, nc.x, nc.y, nc.z, nc.w, r, lim, tmin_bits, t1);
    // the hit leaf children (0, 1 or 2) are tested by one loop, so lanes
    // with one leaf and lanes with two share the same instructions
    const bool l0 = h0 && ch.x < 0, l1 = h1 && ch.y < 0;
    const int nleaf = (int)l0 + (int)l1;
    for (int q = 0; q < nleaf; ++q) {
      const int code = (q == 0 && l0) ? ch.x : ch.y;
      blocked |= leaf_test<ANY>(S, code, o, d, h, c, err);
    }
    h0 = h0 && !l0;
    h1 = h1 && !l1;
    if (ANY && blocked) break;
    if (h0 || h1) {
      if (h0 && h1) {
        trail = (trail << 1) | 1ull;
        cur = ((t0 <= t1) != (ANY && S.any_far)) ? ch.x : ch.y;
      } else {
        trail <<= 1;
        cur = h0 ? ch.x : ch.y;
      }
      continue;
    }
    // backtrack to the deepest level whose far child is pending
    bool done = false;
    for (;;) {
      if (trail == 1ull) {
        done = true;
        break;
      }
      if (trail & 1ull) {
        trail ^= 1ull;
        const int par = clamp_index(__ldg(&nodes[cur].d.z), S.num_nodes, err);
        const int4 pc = __ldg(&nodes[par].d);
        cur = (pc.x == cur) ? pc.y : pc.x;
        break;
      }
      trail >>= 1;
      cur = clamp_index(__ldg(&nodes[cur].d.z), S.num_nodes, err);
    }
    if (done) break;
  }
  // node visits, counted once; the climbs need no budget: each drops a bit
  // of the trail (+0.9% on the 12-triangle shoebox, +3.3% on the small room)
  c.nodes += (uint32_t)iters;
  if (err != err0) {
    h.pos = -1;
    return false;
  }
  return blocked;
}

// Stackless traversal of the 4-wide tree.  Closest hit (ANY = false): h
// receives the hit.  Any hit (ANY = true): returns true when blocked.
// `slack` widens the t-range culling so rounding in the slab test never
// removes a candidate.
//
// The trail holds, per level of the current root path, a 4-bit mask of the
// node's hit children not yet visited (newest level in the low nibble,
// 64 bits for the 16 levels a kept 4-wide tree has at most; one register
// pair instead of two: +1.2% segments/s on the nave, +1.0% on the hall).
// An all-zero trail means nothing is pending on any level, so no level
// counter is kept; a lane's error flags are sticky, so no copy of them
// either: the two registers saved reduce the bounce kernel's spills, +5.2%
// segments/s on the nave and +6.6% on the hall.  (The same two changes in
// the binary traversal cost the small rooms 20-28%: not made there.)  The
// node visits are counted once, from the budget spent, at the end (+1.8%
// on the nave).
//
// A node visit tests its candidate slots' boxes,
// tests hit leaf children at once (one merged loop) and descends into the
// nearest hit internal child, pushing the others.  At a dead end the walk
// climbs parent links to the deepest level with pending children and
// re-enters that node, re-testing only the pending slots against the
// current limit (after Afra and Szirmay-Kalos, "Stackless multi-BVH
// traversal for CPU, MIC and GPU ray tracing", CGF 2014).  The closest hit
// is the lexicographic (t, index) minimum and the any-hit result a
// boolean, so neither depends on the visiting order.
template <bool ANY>
__device__ bool traverse4(const SceneRef& S, V3 o, V3 d, float tlimit, float slack, Hit& h,
                          LaneCounters& c, int& err) {
  h.t = tlimit;
  h.pos = -1;
  h.orig = INT_MAX;
  if (S.num_tris == 0) return false;
  const Ray r = make_ray(o, d);
  // closest hit: only t > 0.001 counts (src/Mesh.cpp:40), so boxes the
  // ray leaves before 0.001 - slack hold no hit (slack = the boxes' padding
  // covers the rounding of the slab distances, as on the far side); the
  // boxes around the ray's origin on its surface are culled at once
  const int tmin_bits = ANY ? 0 : __float_as_int(fmaxf(0.001f - slack, 0.0f));
  const Node4* __restrict__ nodes = S.nodes4;
  int cur = 0;
  unsigned long long tlo = 0ull;  // the trail (all zero: nothing pending)
  bool reentry = false;  // cur's own pending mask is the low nibble
  // node visits left; the climbs need no budget: each drops a nibble of
  // the trail, so a dead end climbs at most 16 levels
  int budget = S.traverse_budget;
  bool blocked = false;
  for (;;) {
    if (--budget < 0) {
      err |= kErrBudget;
      break;
    }
    cur = clamp_index(cur, S.num_nodes, err);
    const Node4* nd = nodes + cur;
    // the near and far planes of each axis, picked by the load address
    // (lox, hix, loy, hiy, loz, hiz are consecutive float4s)
    const float4* P = &nd->lox;
    const int sx = __float_as_int(r.ix) < 0, sy = __float_as_int(r.iy) < 0,
              sz = __float_as_int(r.iz) < 0;
    const float4 nx4 = __ldg(P + sx), fx4 = __ldg(P + 1 - sx);
    const float4 ny4 = __ldg(P + 2 + sy), fy4 = __ldg(P + 3 - sy);
    const float4 nz4 = __ldg(P + 4 + sz), fz4 = __ldg(P + 5 - sz);
    float4 chf, mtf;
    ldg256(&nd->child, chf, mtf);
    const int4 ch = as_int4(chf), meta = as_int4(mtf);
    const unsigned cand = (reentry ? (unsigned)(tlo & 0xFull) : 0xFu) & (unsigned)meta.y;
    const float lim = ANY ? tlimit + slack : h.t + (h.t * kSlackRel + slack);
    unsigned hit = 0u, leaf = 0u;
    float tk[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      float tn;
      const bool b = box_hit_nf(lane4(nx4, k), lane4(fx4, k), lane4(ny4, k), lane4(fy4, k),
                                lane4(nz4, k), lane4(fz4, k), r, lim, tmin_bits, tn);
      tk[k] = tn;
      if (((cand >> k) & 1u) && b) hit |= 1u << k;
      if (lane4(ch, k) < 0) leaf |= 1u << k;
    }
    // the next internal child is chosen before the leaf tests, so the
    // entry distances are dead while the triangles are tested: nearest hit
    // child first; visibility tests in scenes where most segments are
    // blocked go farthest first (occluders between the surface and the
    // listener are met sooner)
    const unsigned inner = hit & ~leaf;
    unsigned rest = 0u;
    int next = 0;
    if (inner) {
      int kb = -1;
      float best = 0.0f;
      const bool far = ANY && S.any_far;
#pragma unroll
      for (int k = 0; k < 4; ++k)
        if (((inner >> k) & 1u) && (kb < 0 || (far ? tk[k] > best : tk[k] < best))) {
          best = tk[k];
          kb = k;
        }
      rest = inner & ~(1u << kb);
      next = lane4(ch, kb);
    }
    // hit leaf children, one merged loop
    for (unsigned lm = hit & leaf; lm; lm &= lm - 1u) {
      const int k = __ffs(lm) - 1;
      blocked |= leaf_test<ANY>(S, lane4(ch, k), o, d, h, c, err);
    }
    if (ANY && blocked) break;
    if (inner) {
      if (reentry) {
        tlo = (tlo & ~0xFull) | rest;
      } else {
        tlo = (tlo << 4) | rest;
      }
      cur = next;
      reentry = false;
      continue;
    }
    // dead end: climb to the deepest level with pending children
    if (reentry) tlo >>= 4;  // cur's own pending mask is exhausted
    int par = meta.x;
    bool done = false;
    for (;;) {
      // an all-zero trail holds no pending child on any level
      if (tlo == 0ull) {
        done = true;
        break;
      }
      if (tlo & 0xFull) {
        cur = par;
        reentry = true;
        break;
      }
      tlo >>= 4;
      cur = clamp_index(par, S.num_nodes, err);
      if (tlo == 0ull) {
        done = true;
        break;
      }
      par = __ldg(&nodes[cur].meta.x);
    }
    if (done) break;
  }
  // node visits = budget spent (the climbs are bounded by the trail:
  // each step drops a nibble); two 64-byte halves each
  c.nodes += 2u * (uint32_t)(S.traverse_budget - budget);
  if (err) {  // any error of this lane invalidates its results
    h.pos = -1;
    return false;
  }
  return blocked;
}

// The scene's tree: 4-wide for large scenes (fewer dependent node loads
// per query), binary for small ones (cheaper visits).
template <bool ANY>
__device__ __forceinline__ bool traverse(const SceneRef& S, V3 o, V3 d, float tlimit, float slack,
                                         Hit& h, LaneCounters& c, int& err) {
  return S.wide ? traverse4<ANY>(S, o, d, tlimit, slack, h, c, err)
                : traverse2<ANY>(S, o, d, tlimit, slack, h, c, err);
}

// ------------------------------------------------------------- sampling
// Sample_Sphere / Sample_Hemi (src/Distributions.h:48-67): one Philox
// block per try; try 0's block is passed in (its 4th word also drives the
// material choice).
__device__ __forceinline__ bool sample_dir(const TraceArgs& a, uint32_t ctx, uint32_t band,
                                           uint64_t ray, uint32_t bounce, bool hemi, V3 n, U4 b,
                                           V3& out) {
  bool ok = false;
  out = mk(0.0f, 0.0f, 1.0f);
  for (int tr = 0; tr < kMaxTries; ++tr) {
    if (tr) b = rng_block(a.k0, a.k1, ctx, band, ray, 0, bounce, (uint32_t)tr);
    const float f1 = uniform24(b.x) * 2.0f - 1.0f;
    const float f2 = uniform24(b.y) * 2.0f - 1.0f;
    const float f3 = uniform24(b.z) * 2.0f - 1.0f;
    const float l = (f1 * f1 + f2 * f2) + f3 * f3;
    if (l < 0.001f || l > 1.0f) continue;
    const float sl = f_sqrt(l);
    const V3 v = mk(f1 / sl, f2 / sl, f3 / sl);
    if (hemi && dot(n, v) < 0.0f) continue;
    out = v;
    ok = true;
    break;
  }
  return ok;
}

// ---------------------------------------------------------------- splats
// Adds the triangular splat v_0 = ampl, v_{i+1} = v_i - step at positions
// s .. s+w-1 (src/MonoRecorder.cpp:90-93), skipping negative positions
// (src/StereoRecorder.cpp:93) and positions beyond the window, and updates
// the FloatBuffer bookkeeping (first_sample / real_length,
// src/Recorder.cpp:56-57) in shared memory.  The values follow the
// reference's float recurrence (one subtraction per position, skipped
// positions included); they are added four aligned bins at a time, one
// 16-byte vector reduction per group.
__device__ __forceinline__ void splat(float* row, int* first, int* last, int nb, long long s,
                                      int w, float ampl, float step, uint32_t& bins) {
  bins += (uint32_t)w;
  const long long lastpos = s + w - 1;
  if (lastpos < 0) return;
  const long long firstpos = s < 0 ? 0 : s;
  // first only decreases and last only increases, so a stale read can only
  // cause a redundant atomic, never a missed one
  const int fp = (int)(firstpos < nb ? firstpos : nb);
  const int lp = (int)(lastpos < nb ? lastpos : nb);
  if (fp < *(volatile int*)first) atomicMin(first, fp);
  if (lp > *(volatile int*)last) atomicMax(last, lp);
  if (firstpos >= nb) return;
  float v = ampl;
  for (long long q = s; q < 0; ++q) v -= step;  // positions before the track
  const int p0 = fp;                             // first and last position added
  const int p1 = lastpos < nb ? (int)lastpos : nb - 1;
  for (int g = p0 >> 2; g <= (p1 >> 2); ++g) {
    const int q = 4 * g;
    float4 acc;
    const bool i0 = q >= p0 && q <= p1, i1 = q + 1 >= p0 && q + 1 <= p1;
    const bool i2 = q + 2 >= p0 && q + 2 <= p1, i3 = q + 3 >= p0 && q + 3 <= p1;
    acc.x = i0 ? v : 0.0f;
    v = i0 ? v - step : v;
    acc.y = i1 ? v : 0.0f;
    v = i1 ? v - step : v;
    acc.z = i2 ? v : 0.0f;
    v = i2 ? v - step : v;
    acc.w = i3 ? v : 0.0f;
    v = i3 ? v - step : v;
    atomicAdd(reinterpret_cast<float4*>(row + q), acc);
  }
}

// Adjoint counterpart of splat(): the dot product of the upstream gradient
// with the splat values, over the same positions.
__device__ __forceinline__ float gather(const float* __restrict__ g, int nb, long long s, int w,
                                        float ampl, float step) {
  float v = ampl, acc = 0.0f;
  for (int i = 0; i < w; ++i) {
    const long long pos = s + i;
    if (pos >= nb) break;
    if (pos >= 0) acc += __ldg(g + pos) * v;
    v -= step;
  }
  return acc;
}

// Records one contribution (forward) or returns its gradient weight
// sum_i g[s+i] * v_i (adjoint).
template <int MODE>
__device__ __forceinline__ float record(const TraceArgs& a, const DevRecorder& R, int band, V3 dir,
                                        float amp, float t, float dist, int* s_first, int* s_last,
                                        uint32_t& bins) {
  const SplatPlan p = record_plan<kFastMath>(R, band, dir, amp, t, dist);
  float G = 0.0f;
  for (int k = 0; k < p.tracks; ++k) {
    const int tb = (R.track0 + k) * 3 + band;
    if (MODE == kModeAdjoint) {
      G += gather(a.adj_g + (size_t)tb * (size_t)a.stride, a.num_bins, p.s[k], p.w, p.ampl[k],
                  p.step[k]);
    } else {
      // single render: bookkeeping privatised in shared memory, merged once
      // per block; batch: straight to the global rows
      int* fp = MODE == kModeBatch ? reinterpret_cast<int*>(a.first_last + tb) : s_first + tb;
      int* lp = MODE == kModeBatch ? fp + 1 : s_last + tb;
      splat(a.hist + (size_t)tb * (size_t)a.stride, fp, lp, a.num_bins, p.s[k], p.w, p.ampl[k],
            p.step[k], bins);
    }
  }
  return G;
}

// --------------------------------------------------------------- paths
struct PathState {
  V3 o, d, prev;
  float I, L;
  int k;
  int band;
  uint64_t ray;
  float P, T;  // adjoint: gradient weights of the contributions so far / in total
  // batch mode: the lane's job
  int job, scene, rec_base, num_recs;
  uint32_t ctx;
};

template <int MODE>
__device__ __forceinline__ uint32_t ctx_of(const TraceArgs& a, const PathState& st) {
  return MODE == kModeBatch ? st.ctx : a.context;
}

template <int MODE>
__device__ __forceinline__ SceneRef scene_of(const TraceArgs& a, const SceneRef* s_scenes,
                                             const PathState& st) {
  if (MODE == kModeBatch) return s_scenes[st.scene];
  SceneRef S;
  S.nodes2 = a.nodes;
  S.nodes4 = a.nodes4;
  S.wide = a.wide;
  S.any_far = a.any_far;
  S.tris = a.tris;
  S.shade = a.tris + 3;
  S.num_tris = a.num_tris;
  S.num_nodes = a.num_nodes;
  S.box_pad = a.box_pad;
  S.mat_base = 0;
  S.num_mats = a.num_mats;
  S.traverse_budget = a.traverse_budget;
  S.vis_cells = a.vis_cells;
  S.vis_entries = a.vis_entries;
  S.vis_res = a.vis_res;
  S.vis_cap = a.vis_cap;
  return S;
}

// Adjoint bookkeeping in shared memory: per thread, the per-material sums
// A[m] of v_j = grad log(weight of the choice at bounce j) -- the weight of
// a REFLECT is refl, of a REFRACT refr (survival times choice probability);
// per block, the gradient accumulators [material][band][2].
struct AdjShared {
  float* A;       // this thread's A[num_mats][2]
  double* grad;   // block accumulators
};

// The state a vertex hands to the recorder phase.
struct Vertex {
  V3 n;          // oriented (and, for REFRACT, flipped) surface normal
  int bt;        // 0 REFLECT, 1 REFRACT (src/Material.h:27)
  float spec;    // specularity of the hit material in this band
  bool conn;     // connect the recorders at this vertex
};

// Cell of the direction o - location (sdir = location - o) in list set mi
// of the scene's maps; false for a degenerate direction.
__device__ __forceinline__ bool vis_cell_of(const SceneRef& S, int mi, V3 sdir, uint32_t& cell) {
  int f, iu, iv;
  const int res = S.vis_res;
  if (!vis_query_cell(sdir.x, sdir.y, sdir.z, res, f, iu, iv)) return false;
  cell = ((uint32_t)(mi * 6 + f) * (uint32_t)res + (uint32_t)iv) * (uint32_t)res + (uint32_t)iu;
  return true;
}

// Visibility test of the segment from `o` to the recorder with list set
// `ri` in the scene's maps (sdir = its location - o, len = |sdir|): the
// entries of the cell of direction o - location nearer than the vertex, each
// by the tree's own triangle test.  Returns 1 blocked, 0 clear, -1 when the
// map leaves the test to the tree (degenerate direction, or a cell longer
// than vis_cap).  The result equals the tree traversal's: the entries are
// every triangle whose padded box meets the segment.
__device__ __forceinline__ int vis_map_test(const SceneRef& S, int ri, V3 o, V3 sdir, float len,
                                            LaneCounters& c, int& err) {
  uint32_t cell;
  if (!vis_cell_of(S, ri, sdir, cell)) return -1;
  const float4* Cp = S.vis_cells + 4 * (size_t)cell;
  float4 H, A0, B0, C0;
  ldg256(Cp, H, A0);
  ldg256(Cp + 2, B0, C0);
  const uint32_t b = __float_as_uint(H.x), e = __float_as_uint(H.y);
  if (e - b > (uint32_t)S.vis_cap) return -1;
  // entries are ordered by their boxes' distance from the recorder; a hit
  // point of the segment lies nearer than len (t > 1e-5).  The cell holds
  // the first three distances (+inf past the end) and the first entry: the
  // entries to test among the first three are counted here, and the first
  // is tested from the cell while the next ones load.
  const float cut = vis_cut(len);
  const uint32_t known = (uint32_t)(A0.w <= cut) + (uint32_t)(H.z <= cut) + (uint32_t)(H.w <= cut);
  if (known == 0) return 0;
  // all three nearer: later entries may be too, and carry their distances
  const uint32_t end = known == kVisCellDists ? e : b + known;
  const bool check = known == kVisCellDists;
  float t;
  ++c.tris;
  uint32_t i = b + 1;
  bool blocked = mt_intersect(A0, B0, C0, o, sdir, t) && t > 1e-5f && t < 1.0f;
  // the rest two entries per step, both loaded before the first test; each
  // carries its triangle's test data (Mesh::LineIntersection: 1e-5 < t <
  // 1, src/Mesh.cpp:65)
  while (!blocked && i < end) {
    const float4* E0 = S.vis_entries + (size_t)kVisEntryVecs * i;
    const bool has1 = i + 1 < end;
    const float4* E1 = has1 ? E0 + kVisEntryVecs : E0;
    const float4 A1 = __ldg(E0), B1 = __ldg(E0 + 1), C1 = __ldg(E0 + 2);
    const float4 A2 = __ldg(E1), B2 = __ldg(E1 + 1), C2 = __ldg(E1 + 2);
    if (check && A1.w > cut) break;
    const bool use2 = has1 && !(check && A2.w > cut);
    ++c.tris;
    ++i;
    if (mt_intersect(A1, B1, C1, o, sdir, t) && t > 1e-5f && t < 1.0f) {
      blocked = true;
      break;
    }
    if (!use2) break;
    ++c.tris;
    ++i;
    if (mt_intersect(A2, B2, C2, o, sdir, t) && t > 1e-5f && t < 1.0f) blocked = true;
  }
  c.map += i - b;
  return blocked ? 1 : 0;
}

// Visibility + contribution of recorder `ri` at the current vertex
// (src/Scene.cpp:188-268).  Returns kNotTested, kBlockedSeg or kVisible.
enum { kNotTested = 0, kBlockedSeg = 1, kVisible = 2 };
template <int MODE>
__device__ __forceinline__ int connect_one(const TraceArgs& a, const SceneRef* s_scenes,
                                            PathState& st, const Vertex& vx, int ri,
                                            LaneCounters& c, int& err, int* s_first,
                                            int* s_last) {
  const DevRecorder& R = a.recs[(MODE == kModeBatch ? st.rec_base : 0) + ri];
  const V3 sdir = sub(mk(R.loc[0], R.loc[1], R.loc[2]), st.o);
  const int k = st.k;
  const V3 lsdir = normalized(sdir);
  const float dt = k ? dot(lsdir, vx.n) : 1.0f;
  // The reference tests the orientation after the visibility
  // (src/Scene.cpp:194-208); a recorder behind the surface contributes
  // nothing either way, so its visibility test is skipped -- except for the
  // debug record, whose mask reports every recorder's visibility.
  if (MODE != kModeDebug && !(dt > 0)) return kNotTested;
  c.shadow++;
  const float len = length(sdir);
  Hit hh;
  const SceneRef S = scene_of<MODE>(a, s_scenes, st);
  const float slack = kSlackRel + S.box_pad / len;
  int vm = -1;
  const int mi = MODE == kModeBatch ? R.vis_index : ri;
  if (S.vis_res > 0 && mi >= 0) vm = vis_map_test(S, mi, st.o, sdir, len, c, err);
  if (vm < 0) vm = traverse<true>(S, st.o, sdir, 1.0f, slack, hh, c, err) ? 1 : 0;
  if (vm) return kBlockedSeg;
  if (!(dt > 0)) return kVisible;
  // sample_intensity_before_bounce (src/Scene.cpp:173): the path's
  // intensity, unchanged between the vertex and its connections
  float I = st.I;
  if (k) {
    const V3 n = vx.n;
    float factor;
    if (vx.bt == 0) {
      const V3 refl_vector = reflect(st.prev, n);
      const float diff_factor = -dot(n, st.prev);
      const float rv = dot(refl_vector, lsdir);
      const float spec_factor = (0.0f < rv) ? rv : 0.0f;
      factor = vx.spec * 1001.0f * pow_sel<kFastMath>(spec_factor, 1000.0f) +
               (1.0f - vx.spec) * diff_factor;
    } else {
      const float diff_factor = dot(n, st.prev);
      const float rv = dot(st.prev, lsdir);
      const float spec_factor = (0.0f < rv) ? rv : 0.0f;
      factor = vx.spec * 1001.0f * pow_sel<kFastMath>(spec_factor, 1000.0f) +
               (1.0f - vx.spec) * diff_factor;
    }
    I *= factor;
  }
  I *= pow_sel<kFastMath>(a.air[st.band], len);
  I *= inv_hemi_2(len);
  if (!invalid_float(I)) {
    if (k & 1) I *= -1.0f;
    c.contrib++;
    const float total = st.L + len;
    const float G = record<MODE>(a, R, st.band, lsdir, I, total / 343.0f, total, s_first, s_last,
                                 c.bins);
    if (MODE == kModeAdjoint) {
      st.P += G;
      st.T += G;
    }
  }
  return kVisible;
}

template <int MODE>
__device__ __forceinline__ void debug_put(const TraceArgs& a, const PathState& st, int k, int hit,
                                          int bt, uint32_t vis, int what) {
  if (MODE != kModeDebug) return;
  const uint64_t local = st.ray - a.ray0;
  if (st.band != a.dbg_band || local >= (uint64_t)a.dbg_rays || k < 1 || k > a.dbg_max_record)
    return;
  const size_t i = (size_t)local * a.dbg_max_record + (k - 1);
  if (what == 0) a.dbg_hit[i] = hit;
  if (what == 1) a.dbg_bt[i] = (uint8_t)bt;
  if (what == 2) a.dbg_vis[i] = vis;
}

// Bounce 0: AbstractSoundFile::SoundRay (src/SoundFile.cpp:215-228).  Area
// emitters connect the recorders at bounce 0 (src/Scene.cpp:185).
template <int MODE>
__device__ void emit_vertex(const TraceArgs& a, PathState& st, LaneCounters& c, Vertex& vx,
                            const AdjShared& adj) {
  st.I = 1.0f;
  st.L = 0.0f;
  st.k = 0;
  if (MODE == kModeAdjoint) {
    st.P = 0.0f;
    st.T = 0.0f;
    for (int m = 0; m < 2 * a.num_mats; ++m) adj.A[m] = 0.0f;
  }
  const uint32_t band = (uint32_t)st.band;
  const uint32_t ctx = ctx_of<MODE>(a, st);
  const U4 b0 = rng_block(a.k0, a.k1, ctx, band, st.ray, 0, 0, 0);
  if (MODE != kModeBatch && a.num_emitter > 0) {
    // Mesh::SamplePoint (src/Mesh.cpp:143-154): linear walk of the area CDF
    const U4 e = rng_block(a.k0, a.k1, ctx, band, st.ray, 1, 0, 0);
    float x = uniform24(e.x) * a.emitter_total_area;
    V3 p = mk(0, 0, 0), en = mk(0, 0, 0);
    for (int i = 0; i < a.num_emitter; ++i) {
      const float4 A = __ldg(a.emitter + 4 * i);
      x -= A.w;
      if (x < 0) {
        const float4 B = __ldg(a.emitter + 4 * i + 1), C = __ldg(a.emitter + 4 * i + 2),
                     N = __ldg(a.emitter + 4 * i + 3);
        const float r1 = uniform24(e.y), r2 = uniform24(e.z);
        const float sr1 = f_sqrt(r1);
        const float wa = 1.0f - sr1, wb = sr1 * (1.0f - r2), wc = sr1 * r2;
        p = mk((wa * A.x + wb * B.x) + wc * C.x, (wa * A.y + wb * B.y) + wc * C.y,
               (wa * A.z + wb * B.z) + wc * C.z);
        en = mk(N.x, N.y, N.z);
        break;
      }
    }
    st.o = p;
    if (!sample_dir(a, ctx, band, st.ray, 0, true, en, b0, st.d)) c.overflow++;
  } else {
    if (MODE == kModeBatch) {
      const float* js = a.jobs[st.job].src;
      st.o = mk(js[0], js[1], js[2]);
    } else {
      st.o = mk(a.src[0], a.src[1], a.src[2]);
    }
    if (!sample_dir(a, ctx, band, st.ray, 0, false, mk(0, 0, 0), b0, st.d)) c.overflow++;
  }
  vx.n = mk(0, 0, 0);
  vx.bt = 0;
  vx.spec = 0.0f;
  vx.conn = MODE != kModeBatch && a.num_emitter > 0;
}

// Reflection k = st.k + 1 up to the recorder connections
// (src/Scene.cpp:150-177): closest hit, Material::Bounce, Sample_Hemi,
// air and surface losses.  Returns whether the path continues.
template <int MODE>
__device__ bool bounce_vertex(const TraceArgs& a, const DevMaterial* __restrict__ mats,
                              const SceneRef* s_scenes, PathState& st, LaneCounters& c, int& err,
                              Vertex& vx, const AdjShared& adj) {
  const int k = st.k + 1;
  const uint32_t band = (uint32_t)st.band;
  c.segments++;
  Hit h;
  const SceneRef S = scene_of<MODE>(a, s_scenes, st);
  traverse<false>(S, st.o, st.d, 1000000.0f, S.box_pad, h, c, err);
  debug_put<MODE>(a, st, k, h.pos >= 0 ? h.orig : -1, 0, 0, 0);
  if (h.pos < 0) return false;
  const float4 nm = __ldg(S.shade + 4 * h.pos);
  const float t = h.t;
  const V3 p = mk(st.o.x + st.d.x * t, st.o.y + st.d.y * t, st.o.z + st.d.z * t);
  const V3 N = mk(nm.x, nm.y, nm.z);
  V3 n = (dot(N, st.d) > 0.0f) ? neg(N) : N;
  const int mid = clamp_index(__float_as_int(nm.w), S.num_mats, err) + S.mat_base;
  const DevMaterial& M = mats[mid];
  // Material::Bounce (src/Material.cpp:76-83)
  const uint32_t ctx = ctx_of<MODE>(a, st);
  const U4 b0 = rng_block(a.k0, a.k1, ctx, band, st.ray, 0, (uint32_t)k, 0);
  int bt = 0;
  if (!((M.always_reflect >> band) & 1u)) bt = (uniform24(b0.w) <= M.p_reflect[band]) ? 0 : 1;
  debug_put<MODE>(a, st, k, 0, bt, 0, 1);
  if (MODE == kModeAdjoint) {
    // v = grad log(s P(choice)) w.r.t. (absorption, refraction), with
    // refl = 1 - absorption - refraction: -1/s from the survival plus the
    // score of the choice; the sum is -1/refl (REFLECT) or (0, 1/refr)
    // (REFRACT), and -1/s alone when the choice is forced.
    float va, vr;
    if ((M.always_reflect >> band) & 1u) {
      va = -1.0f / M.survival[band];
      vr = 0.0f;
    } else if (bt == 0) {
      va = -1.0f / M.survival[band] - M.refr[band] / ((M.refl[band] + M.refr[band]) * M.refl[band]);
      vr = -1.0f / M.refl[band];
    } else {
      va = -1.0f / M.survival[band] + 1.0f / (M.refl[band] + M.refr[band]);
      vr = 1.0f / M.refr[band];
    }
    adj.A[2 * mid] += va;
    adj.A[2 * mid + 1] += vr;
    if (st.P != 0.0f) {
      double* gm = adj.grad + ((size_t)mid * 3 + band) * 2;
      atomicAdd(gm, -(double)va * (double)st.P);
      atomicAdd(gm + 1, -(double)vr * (double)st.P);
    }
  }
  const float spec = M.spec[band];
  V3 base;
  if (bt == 1) {
    n = neg(n);
    base = st.d;
  } else {
    base = reflect(st.d, n);
  }
  V3 v;
  if (!sample_dir(a, ctx, band, st.ray, (uint32_t)k, true, n, b0, v)) c.overflow++;
  const float om = 1.0f - spec;
  v = normalized(mk(v.x * om + base.x * spec, v.y * om + base.y * spec, v.z * om + base.z * spec));
  const float l = length(sub(p, st.o));
  st.I *= pow_sel<kFastMath>(a.air[band], l);
  st.L += l;
  st.o = p;
  st.d = v;
  st.k = k;
  st.I *= M.survival[band];
  vx.n = n;
  vx.bt = bt;
  vx.spec = spec;
  vx.conn = true;
  return !invalid_float(st.I);
}

// End of an adjoint path: grad[m][band] += T * A[m].
__device__ __forceinline__ void adjoint_flush(const TraceArgs& a, const PathState& st,
                                              const AdjShared& adj) {
  if (st.T == 0.0f) return;
  for (int m = 0; m < a.num_mats; ++m) {
    const float va = adj.A[2 * m], vr = adj.A[2 * m + 1];
    if (va == 0.0f && vr == 0.0f) continue;
    double* gm = adj.grad + ((size_t)m * 3 + st.band) * 2;
    atomicAdd(gm, (double)st.T * (double)va);
    atomicAdd(gm + 1, (double)st.T * (double)vr);
  }
}

// Direct-sound visibility (src/Scene.cpp:299-304): Connect(listener,
// source) for every recorder, computed by the first threads of block 0
// with the same any-hit traversal as the path connections.  The lobe
// itself is added by the finalize kernel between the two scaling passes.
// A batch spreads its (job, recorder) pairs over every thread of the grid.
template <int MODE>
__device__ void direct_visibility(const TraceArgs& a, const SceneRef* s_scenes, int& err) {
  if (a.direct_vis == nullptr) return;
  int r = (int)threadIdx.x;
  int step = a.num_recs;
  if (MODE == kModeBatch) {
    r += (int)(blockIdx.x * blockDim.x);
    step = (int)(gridDim.x * blockDim.x);
  } else if (blockIdx.x != 0) {
    return;
  }
  for (; r < a.num_recs; r += step) {
    const DevRecorder& R = a.recs[r];
    const float* src = a.src;
    PathState st;
    st.scene = 0;
    if (MODE == kModeBatch) {
      const BatchJob& J = a.jobs[R.job];
      src = J.src;
      st.scene = J.scene;
    }
    const SceneRef S = scene_of<MODE>(a, s_scenes, st);
    const V3 loc = mk(R.loc[0], R.loc[1], R.loc[2]);
    const V3 seg = sub(mk(src[0], src[1], src[2]), loc);
    const float seglen = length(seg);
    const float slack = kSlackRel + (seglen > 0.0f ? S.box_pad / seglen : 0.0f);
    LaneCounters c = {0, 0, 0, 0, 0, 0, 0, 0};
    Hit hh;
    const bool blocked = traverse<true>(S, loc, seg, 1.0f, slack, hh, c, err);
    a.direct_vis[r] = blocked ? 0 : 1;
  }
}

// Four resident blocks per SM (64 registers): the traversal is bound by
// the latency of dependent node loads, and 32 warps per SM hide it better
// than 16 warps without register spills (measured: +44% segments/s on the
// 20,000-triangle hall, +59% on the 2,000,000-triangle nave).
template <int MODE>
__global__ void __launch_bounds__(kTraceMaxBlock, 4) trace_kernel(const TraceArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  DevMaterial* s_mats = reinterpret_cast<DevMaterial*>(smem_raw);
  const size_t mat_bytes = (sizeof(DevMaterial) * (size_t)a.num_mats + 15) & ~(size_t)15;
  // single render: first/last bookkeeping per (track, band); batch: the
  // scene table
  int* s_first = reinterpret_cast<int*>(smem_raw + mat_bytes);
  int* s_last = s_first + a.num_tracks * 3;
  SceneRef* s_scenes = reinterpret_cast<SceneRef*>(smem_raw + mat_bytes);
  AdjShared adj = {nullptr, nullptr};
  if (MODE == kModeAdjoint) {
    size_t off = mat_bytes + sizeof(int) * 6 * a.num_tracks;
    off = (off + 7) & ~(size_t)7;
    adj.grad = reinterpret_cast<double*>(smem_raw + off);
    float* all_A = reinterpret_cast<float*>(adj.grad + 6 * a.num_mats);
    adj.A = all_A + (size_t)threadIdx.x * 2 * a.num_mats;
    for (int i = threadIdx.x; i < 6 * a.num_mats; i += blockDim.x) adj.grad[i] = 0.0;
  }
  {
    const uint32_t* src = reinterpret_cast<const uint32_t*>(a.mats);
    uint32_t* dst = reinterpret_cast<uint32_t*>(s_mats);
    const int words = (int)(sizeof(DevMaterial) / 4) * a.num_mats;
    for (int i = threadIdx.x; i < words; i += blockDim.x) dst[i] = __ldg(src + i);
    if (MODE == kModeBatch) {
      const uint32_t* ssrc = reinterpret_cast<const uint32_t*>(a.scenes);
      uint32_t* sdst = reinterpret_cast<uint32_t*>(s_scenes);
      const int swords = (int)(sizeof(SceneRef) / 4) * a.num_scenes;
      for (int i = threadIdx.x; i < swords; i += blockDim.x) sdst[i] = __ldg(ssrc + i);
    } else {
      for (int i = threadIdx.x; i < a.num_tracks * 3; i += blockDim.x) {
        s_first[i] = kInitialFirstSample;
        s_last[i] = 0;
      }
    }
  }
  int err = 0;
  if (MODE != kModeBatch) direct_visibility<MODE>(a, s_scenes, err);
  __syncthreads();
  if (MODE == kModeBatch) direct_visibility<MODE>(a, s_scenes, err);
  const int lane = threadIdx.x & 31;
  LaneCounters c = {0, 0, 0, 0, 0, 0, 0, 0};
  bool alive = false, exhausted = false;
  PathState st;
  st.k = 0;
  st.band = 0;
  st.ray = 0;
  st.P = 0.0f;
  st.T = 0.0f;
  st.job = 0;
  st.scene = 0;
  st.rec_base = 0;
  st.num_recs = 0;
  st.ctx = 0;
  // Every lane, live or not, passes the same __syncwarp() points below;
  // per-lane work between them is predicated, so divergent loops
  // (traversal, rejection sampling) reconverge at each phase boundary.
  for (;;) {
    // phase 1: refill lanes whose path ended (one atomic per warp)
    const unsigned need = __ballot_sync(kFull, !alive && !exhausted);
    bool fresh = false;
    if (need) {
      const int leader = __ffs(need) - 1;
      unsigned long long base = 0;
      if (lane == leader) base = atomicAdd(a.counters + kWork, (unsigned long long)__popc(need));
      base = __shfl_sync(kFull, base, leader);
      if (!alive && !exhausted) {
        const unsigned long long w = base + (unsigned long long)__popc(need & ((1u << lane) - 1u));
        if (w < a.num_items) {
          if (MODE == kModeBatch) {
            // the job whose item range holds w: first job with w < end
            int lo = 0, hi = a.num_jobs - 1;
            while (lo < hi) {
              const int mid = (lo + hi) >> 1;
              if (w < __ldg(a.job_end + mid)) {
                hi = mid;
              } else {
                lo = mid + 1;
              }
            }
            const uint64_t begin = lo ? __ldg(a.job_end + lo - 1) : 0ull;
            const BatchJob& J = a.jobs[lo];
            const uint64_t nr = J.num_rays;
            const uint64_t local = w - begin;
            const uint64_t bi = local / nr;
            st.band = a.bands[bi < 3 ? bi : 0];
            st.ray = local - bi * nr;
            st.job = lo;
            st.scene = J.scene;
            st.rec_base = J.rec_base;
            st.num_recs = J.num_recs;
            st.ctx = J.context;
          } else {
            const uint64_t bi = w / a.num_rays;
            st.band = a.bands[bi < 3 ? bi : 0];
            st.ray = a.ray0 + (w - bi * a.num_rays);
          }
          fresh = true;
        } else {
          exhausted = true;
        }
      }
    }
    if (__all_sync(kFull, exhausted)) break;
    // phase 2: one path vertex -- the emission of a fresh ray or the next
    // reflection of a live one
    Vertex vx;
    vx.conn = false;
    if (fresh) {
      emit_vertex<MODE>(a, st, c, vx, adj);
      alive = true;
    } else if (alive) {
      alive = bounce_vertex<MODE>(a, s_mats, s_scenes, st, c, err, vx, adj);
      vx.conn = alive;
      if (MODE == kModeAdjoint && !alive) adjoint_flush(a, st, adj);
    }
    __syncwarp();
    // phase 3: recorder connections (src/Scene.cpp:185-270)
    uint32_t vis = 0;
    const int nrec = MODE == kModeBatch
                         ? (int)__reduce_max_sync(kFull, vx.conn ? (unsigned)st.num_recs : 0u)
                         : a.num_recs;
    for (int ri = 0; ri < nrec; ++ri) {
      int res = kNotTested;
      if (vx.conn && (MODE != kModeBatch || ri < st.num_recs))
        res = connect_one<MODE>(a, s_scenes, st, vx, ri, c, err, s_first, s_last);
      if (res == kVisible) vis |= 1u << (ri & 31);
      __syncwarp();
    }
    // phase 4: cut-off, next direction, bounce limit (src/Scene.cpp:275-277)
    if (alive) {
      if (st.k > 0) debug_put<MODE>(a, st, st.k, 0, 0, vis, 2);
      if ((double)st.I < a.cutoff || st.k >= a.max_bounces) {
        alive = false;
        if (MODE == kModeAdjoint) adjoint_flush(a, st, adj);
      } else {
        st.prev = normalized(st.d);
      }
    }
  }
  __syncwarp();
  // flush statistics: one atomic per warp and counter
  {
    const uint32_t seg = __reduce_add_sync(kFull, c.segments);
    const uint32_t sh = __reduce_add_sync(kFull, c.shadow);
    const uint32_t co = __reduce_add_sync(kFull, c.contrib);
    const uint32_t ov = __reduce_add_sync(kFull, c.overflow);
    const unsigned long long nv = __reduce_add_sync(kFull, c.nodes);
    const unsigned long long tt = __reduce_add_sync(kFull, c.tris);
    const unsigned long long bn = __reduce_add_sync(kFull, c.bins);
    const unsigned long long me = __reduce_add_sync(kFull, c.map);
    const int werr = (int)__reduce_or_sync(kFull, (unsigned)err);
    if (lane == 0) {
      atomicAdd(a.counters + kNodeVisits, nv);
      atomicAdd(a.counters + kTriTests, tt);
      atomicAdd(a.counters + kSplatBins, bn);
      if (me) atomicAdd(a.counters + kMapEntries, me);
      atomicAdd(a.counters + kSegments, (unsigned long long)seg);
      atomicAdd(a.counters + kShadow, (unsigned long long)sh);
      atomicAdd(a.counters + kContrib, (unsigned long long)co);
      if (ov) atomicAdd(a.counters + kOverflow, (unsigned long long)ov);
      if (werr) atomicOr(a.error_flag, werr);
    }
  }
  if (MODE == kModeBatch) return;
  __syncthreads();
  if (MODE == kModeAdjoint) {
    for (int i = threadIdx.x; i < 6 * a.num_mats; i += blockDim.x)
      if (adj.grad[i] != 0.0) atomicAdd(a.adj_grad + i, adj.grad[i]);
    return;
  }
  for (int i = threadIdx.x; i < a.num_tracks * 3; i += blockDim.x) {
    if (s_last[i] > 0) atomicMax(&a.first_last[i].y, s_last[i]);
    if (s_first[i] < kInitialFirstSample) atomicMin(&a.first_last[i].x, s_first[i]);
  }
}

// Occlusion probe for the visibility order: n seeded segments from
// triangle centroids, moved 1 mm off the surface on the side facing the
// listener, to the render's recorders; counts the blocked ones.  Only the
// traversal order of later visibility tests depends on the result.
__global__ void occlusion_probe_kernel(const TraceArgs a, int n, unsigned* blocked) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n || a.num_tris < 1 || a.num_recs < 1) return;
  const U4 r = philox4x32_10((uint32_t)k, 0x9e3779b9u, 0u, 0u, 0x85ebca6bu, 0xc2b2ae35u);
  const int i = (int)(r.x % (uint32_t)a.num_tris);
  const DevRecorder& R = a.recs[r.y % (uint32_t)a.num_recs];
  const float4* T = a.tris + 4 * i;
  const float4 A = __ldg(T), B = __ldg(T + 1), C = __ldg(T + 2), Nn = __ldg(T + 3);
  const V3 c = mk(A.x + (B.x + C.x) / 3.0f, A.y + (B.y + C.y) / 3.0f, A.z + (B.z + C.z) / 3.0f);
  const V3 rl = mk(R.loc[0], R.loc[1], R.loc[2]);
  V3 nn = mk(Nn.x, Nn.y, Nn.z);
  if (dot(nn, sub(rl, c)) < 0.0f) nn = neg(nn);
  const V3 o = mk(c.x + nn.x * 1e-3f, c.y + nn.y * 1e-3f, c.z + nn.z * 1e-3f);
  const V3 seg = sub(rl, o);
  const float len = length(seg);
  if (!(len > 0.0f)) return;
  PathState st;
  st.scene = 0;
  const SceneRef S = scene_of<kModeForward>(a, nullptr, st);
  LaneCounters cnt = {0, 0, 0, 0, 0, 0, 0};
  int err = 0;
  Hit h;
  if (traverse<true>(S, o, seg, 1.0f, kSlackRel + S.box_pad / len, h, cnt, err)) atomicAdd(blocked, 1u);
}

}  // namespace EAR_NS
}  // namespace ear
