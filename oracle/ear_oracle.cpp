// ear_oracle.cpp -- CPU restatement of E.A.R's ray-tracing path.
//
// TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and the
// cpu_baseline / --impl reference legs of bench.py may load this library,
// and only as the checker or the timed CPU baseline; the product path never
// calls it.
//
// PINNED to the reference itself.  The reference's shipped build cannot
// run here (GMTL 0.6.1 and Boost.Thread are neither vendored nor
// installed, and it ships no tests, golden vectors or .EAR fixtures), so
// oracle/build_ref.py compiles its own ray-tracing sources (src/Scene,
// Mesh, Triangle, Material, Mono/StereoRecorder, Recorder, Datatype, ...)
// against a project-written GMTL / Boost interface shim (oracle/refshim/)
// into oracle/_ref, and tests/test_ref_pin.py checks that its
// Scene::Render, fed this oracle's random numbers in its own call order
// (oracle_random_tape), writes FloatBuffer tracks bit-identical to this
// file's float accumulation.  This file restates the reference's algorithm
// step by step from its sources (citations are path:line inside
// aothms/ear) with three documented substitutions that this oracle, the
// CUDA path and the shim share by specification:
//   1. gmtl::Math::unitRandom (a global, time-seeded PRNG) is replaced by a
//      counter-based Philox-4x32-10 stream (Salmon et al., SC'11) indexed by
//      (seed, context, band, ray, bounce, try), so every draw is addressable.
//   2. gmtl::intersectDoubleSided is restated from Moller & Trumbore (1997),
//      non-culling variant, epsilon 1e-6, in a fixed operation order.  GMTL
//      is not vendored, so this one function is not pinned to it.
//   3. pow() is the project-defined portable_powf() below (exp2(y*log2 x)
//      with an atanh series for the log and a Taylor polynomial for exp2),
//      so the cut-off decision at src/Scene.cpp:275 cannot diverge between
//      CPU and GPU through libm differences.  pow_mode = 1 selects libm
//      powf() instead, for the statistical comparison.
// Everything else (FloatBuffer bookkeeping, the 1/N and gain^2 scaling
// quirks, the float-accumulated ray count) follows the reference verbatim.
// The auralisation restatement at the end of this file (equalizer band
// split, RecorderTrack::Process) is pinned: the band split equals the
// reference's own lib/equalizer/Equalizer.cpp bit for bit, compiled into
// oracle/_ref by oracle/build_ref.py where the reference tree exists.
// Compile with -ffp-contract=off: the restatement relies on IEEE single
// precision with no fused multiply-adds.

#include "../include/ear_gb300.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <limits>
#include <thread>
#include <vector>

namespace {

// ------------------------------------------------------------ vector math
// Written for this project; gmtl (not vendored) is only known through its
// call sites.  dot = (x*x' + y*y') + z*z', cross in the usual component
// order, normalize divides each component by the Euclidean length when it
// is non-zero.
struct V3 {
  float x, y, z;
};
inline V3 sub(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 neg(V3 a) { return {a.x * -1.0f, a.y * -1.0f, a.z * -1.0f}; }
inline float dot(V3 a, V3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
inline V3 cross(V3 a, V3 b) {
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
inline float length(V3 a) { return std::sqrt(dot(a, a)); }
inline V3 normalized(V3 a) {
  const float l = length(a);
  if (l != 0.0f) return {a.x / l, a.y / l, a.z / l};
  return a;
}
// reflect(v, n) = v - 2 (v.n) n
inline V3 reflect(V3 v, V3 n) {
  const float d = dot(v, n);
  return {v.x - 2.0f * (d * n.x), v.y - 2.0f * (d * n.y), v.z - 2.0f * (d * n.z)};
}
inline V3 load3(const float* p) { return {p[0], p[1], p[2]}; }

inline uint32_t f2u(float f) {
  uint32_t u;
  std::memcpy(&u, &f, 4);
  return u;
}
inline float u2f(uint32_t u) {
  float f;
  std::memcpy(&f, &u, 4);
  return f;
}

// fpclassify(x) != FP_NORMAL (src/Scene.cpp:35-41)
inline bool invalid_float(float x) {
  const uint32_t e = (f2u(x) >> 23) & 0xffu;
  return e == 0u || e == 0xffu;
}

// ------------------------------------------------------------------- pow
float portable_powf(float x, float y) {
  if (x == 1.0f || y == 0.0f) return 1.0f;
  if (x != x || y != y) return std::numeric_limits<float>::quiet_NaN();
  if (x < 0.0f) return std::numeric_limits<float>::quiet_NaN();
  if (x == 0.0f) return y > 0.0f ? 0.0f : std::numeric_limits<float>::infinity();
  if (x == std::numeric_limits<float>::infinity())
    return y > 0.0f ? x : 0.0f;
  uint32_t b = f2u(x);
  int e = (int)(b >> 23);
  if (e == 0) {  // subnormal input: scale by 2^24 (exact)
    b = f2u(x * 16777216.0f);
    e = (int)(b >> 23) - 24;
  }
  e -= 127;
  float m = u2f((b & 0x007fffffu) | 0x3f800000u);
  if (m > 1.41421354f) {
    m = m * 0.5f;
    e += 1;
  }
  // ln m = 2 atanh(s), s = (m-1)/(m+1), |s| <= 0.1716
  const float s = (m - 1.0f) / (m + 1.0f);
  const float s2 = s * s;
  float p = 0.0909090936f;      // 1/11
  p = p * s2 + 0.111111112f;    // 1/9
  p = p * s2 + 0.142857149f;    // 1/7
  p = p * s2 + 0.200000003f;    // 1/5
  p = p * s2 + 0.333333343f;    // 1/3
  const float two_s = s + s;
  const float ln_m = two_s + two_s * (s2 * p);
  const float log2x = (float)e + ln_m * 1.44269502f;  // log2(e)
  const float z = y * log2x;
  if (z > 128.0f) return std::numeric_limits<float>::infinity();
  if (z < -150.0f) return 0.0f;
  const float n = std::rint(z);
  const float f = z - n;  // exact, |f| <= 0.5
  const float g = f * 0.693147182f;  // ln 2
  // e^g by its Taylor polynomial of degree 7 (|g| <= 0.347)
  float q = 1.98412698e-4f;     // 1/7!
  q = q * g + 1.38888889e-3f;   // 1/6!
  q = q * g + 8.33333377e-3f;   // 1/5!
  q = q * g + 4.16666679e-2f;   // 1/4!
  q = q * g + 0.166666672f;     // 1/3!
  q = q * g + 0.5f;
  q = q * g + 1.0f;
  q = q * g + 1.0f;
  int ni = (int)n;
  if (ni > 127) return (q * u2f(0x7f000000u)) * 2.0f;  // 2^127 * 2
  if (ni >= -126) return q * u2f((uint32_t)(ni + 127) << 23);
  return (q * u2f((uint32_t)(ni + 64 + 127) << 23)) * 5.42101086e-20f;  // 2^-64
}

// ---------------------------------------------------------------- Philox
// Philox-4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11).
struct U4 {
  uint32_t v[4];
};
inline U4 philox4x32_10(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3,
                        uint32_t k0, uint32_t k1) {
  for (int r = 0; r < 10; ++r) {
    if (r) {
      k0 += 0x9E3779B9u;
      k1 += 0xBB67AE85u;
    }
    const uint64_t p0 = (uint64_t)0xD2511F53u * c0;
    const uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
    const uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0;
    const uint32_t n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1;
    c0 = n0;
    c1 = (uint32_t)p1;
    c2 = n2;
    c3 = (uint32_t)p0;
  }
  return {{c0, c1, c2, c3}};
}
inline float uniform24(uint32_t x) { return (float)(x >> 8) * 5.9604644775390625e-8f; }

// Counter layout (shared by specification with the CUDA path):
//   c0 = ray index bits 0..31
//   c1 = ray index bits 32..47 | band << 16 | stream << 24
//   c2 = bounce | try << 16
//   c3 = context
//   key = (seed bits 0..31, seed bits 32..63)
// stream 0: direction sampling (u0..u2 per try) and the material choice
//           (u3 of try 0); stream 1: emitter point sampling (try 0).
struct Rng {
  uint32_t k0, k1, context, band;
  U4 block(uint64_t ray, uint32_t stream, uint32_t bounce, uint32_t tr) const {
    const uint32_t c1 = (uint32_t)((ray >> 32) & 0xffffu) | (band << 16) | (stream << 24);
    return philox4x32_10((uint32_t)ray, c1, bounce | (tr << 16), context, k0, k1);
  }
};

constexpr int kMaxTries = 256;

// Random tape (oracle_random_tape): when set, every uniform a trace
// consumes is appended in the order the reference's single global
// generator would be called for the same path -- per reflection the
// material choice (src/Material.cpp:82) before the direction tries
// (src/Scene.cpp:59-71), each try's three draws in Sample_Sphere's order
// (src/Distributions.h:49-51).  Single-threaded renders only.
thread_local std::vector<float>* g_tape = nullptr;

// Sample_Sphere (src/Distributions.h:48-58) and Sample_Hemi
// (src/Distributions.h:62-67): rejection in the cube, reject l<0.001 or
// l>1, then (hemisphere) reject dot(n,v) < 0.  One Philox block per try.
// Returns false when kMaxTries candidates were all rejected; the direction
// is then the deterministic fall-back (0,0,1).
bool sample_dir(const Rng& rng, uint64_t ray, uint32_t bounce, const V3* n, V3* out) {
  for (int tr = 0; tr < kMaxTries; ++tr) {
    const U4 b = rng.block(ray, 0, bounce, (uint32_t)tr);
    if (g_tape)
      for (int q = 0; q < 3; ++q) g_tape->push_back(uniform24(b.v[q]));
    const float f1 = uniform24(b.v[0]) * 2.0f - 1.0f;
    const float f2 = uniform24(b.v[1]) * 2.0f - 1.0f;
    const float f3 = uniform24(b.v[2]) * 2.0f - 1.0f;
    const float l = (f1 * f1 + f2 * f2) + f3 * f3;
    if (l < 0.001f || l > 1.0f) continue;
    const float sl = std::sqrt(l);
    const V3 v = {f1 / sl, f2 / sl, f3 / sl};
    if (n && dot(*n, v) < 0.0f) continue;
    *out = v;
    return true;
  }
  *out = {0.0f, 0.0f, 1.0f};
  return false;
}

// ------------------------------------------------------------- materials
struct OMat {
  float survival[3];  // Material::absorption_coefficient (src/Material.cpp:33-60)
  float p_reflect[3]; // fl2 of Material::Bounce (src/Material.cpp:81)
  bool always_reflect[3];  // src/Material.cpp:79
  float spec[3];
  float refl[3], refr[3];  // the MAT values (refr = 0 when opaque)
};

bool derive_material(const ear_material& m, OMat* o) {
  for (int i = 0; i < 3; ++i) {
    float a = 1.0f;
    a -= m.reflection[i] - 1e-9f;
    if (m.has_refraction) a -= m.refraction[i] - 1e-9f;
    if (a < 0.0f) return false;  // "Invalid material settings"
    o->survival[i] = 1.0f - a;
    const float fl = m.reflection[i];
    const float fr = m.has_refraction ? m.refraction[i] : 0.0f;
    o->always_reflect[i] = ((double)fl < 0.0001 && (double)fr < 0.0001);
    o->p_reflect[i] = fl / (fl + fr);
    o->spec[i] = m.has_specularity ? m.specularity[i] : 0.0f;
    o->refl[i] = fl;
    o->refr[i] = fr;
  }
  return true;
}

// -------------------------------------------------------------- geometry
struct OTri {
  V3 v0, e1, e2;  // e1 = v1 - v0, e2 = v2 - v0
  V3 normal;      // gmtl::normal: normalize(cross(v1 - v0, v2 - v0))
  int mat;
};

// Moller & Trumbore 1997, non-culling branch.
inline bool mt_intersect(const OTri& tr, V3 o, V3 d, float* t_out) {
  const V3 pvec = cross(d, tr.e2);
  const float det = dot(tr.e1, pvec);
  if (det > -1e-6f && det < 1e-6f) return false;
  const float inv_det = 1.0f / det;
  const V3 tvec = sub(o, tr.v0);
  const float u = dot(tvec, pvec) * inv_det;
  if (u < 0.0f || u > 1.0f) return false;
  const V3 qvec = cross(tvec, tr.e1);
  const float v = dot(d, qvec) * inv_det;
  if (v < 0.0f || u + v > 1.0f) return false;
  *t_out = dot(tr.e2, qvec) * inv_det;
  return true;
}

struct OScene {
  std::vector<OTri> tris;
  std::vector<OMat> mats;
};

// Mesh::RayIntersection (src/Mesh.cpp:33-56): brute force, t > 0.001,
// strict t < d so the lowest index wins ties.
inline int closest_hit(const OScene& s, V3 o, V3 d, float* t_best) {
  float best = 1000000.0f;
  int idx = -1;
  const int n = (int)s.tris.size();
  for (int i = 0; i < n; ++i) {
    float t;
    if (mt_intersect(s.tris[i], o, d, &t) && t > 0.001f && t < best) {
      best = t;
      idx = i;
    }
  }
  *t_best = best;
  return idx;
}

// Mesh::LineIntersection (src/Mesh.cpp:58-71): any hit with 1e-5 < t < 1
// on the un-normalised segment direction.
inline bool segment_blocked(const OScene& s, V3 p, V3 dir) {
  for (const OTri& tr : s.tris) {
    float t;
    if (mt_intersect(tr, p, dir, &t) && t > 1e-5f && t < 1.0f) return true;
  }
  return false;
}

// --------------------------------------------------------------- tracks
constexpr int64_t kInitialFirstSample = 3 * 44100 - 1;  // src/Recorder.cpp:46

struct OTrack {  // one FloatBuffer (src/Recorder.h:55-92) restricted to a window
  std::vector<double> h64;
  std::vector<float> h32;
  int64_t first = kInitialFirstSample;
  int64_t last = 0;  // real_length
};

// Adjoint (path-replay) state.  With absorption a = 1 - refl - refr and
// refraction r = refr as parameters, a contribution recorded at bounce k
// carries the survival product of the materials hit (pathwise term) and the
// probabilities of the REFLECT/REFRACT choices (score term); its gradient
// in expectation is C * sum_{j<=k} v_j with v_j = grad log(s P(choice)) of
// the material hit at bounce j.  Summed over contributions this is
// T * sum_j v_j - sum_j v_j P_j, P_j = sum of contribution gradients before
// bounce j, T = their total -- accumulated in one forward replay.
struct Adjoint {
  const double* g = nullptr;  // dL/d(raw splat sum) [track][band][bin]
  int nb = 0;
  int num_mats = 0;
  std::vector<double> A;      // per ray: sum of v per material, (a, r)
  double P = 0.0, T = 0.0, G = 0.0;
  std::vector<double>* grad;  // [material][band][2]
};

struct Sink {
  int num_bins;
  std::vector<OTrack>* tracks;  // [track][band]
  uint64_t contributions = 0;
  Adjoint* adj = nullptr;
  // FloatBuffer::operator[] bookkeeping + accumulation (src/Recorder.cpp:52-59)
  inline void sample(int track, int band, int64_t i, float v) {
    if (adj) {
      if (i >= 0 && i < num_bins) adj->G += adj->g[((size_t)track * 3 + band) * (size_t)num_bins + i] * (double)v;
      return;
    }
    OTrack& tr = (*tracks)[(size_t)track * 3 + band];
    if (i > tr.last) tr.last = i;
    if (i < tr.first) tr.first = i;
    if (i < num_bins) {
      tr.h64[(size_t)i] += (double)v;
      tr.h32[(size_t)i] += v;
    }
  }
};

struct ORec {
  int channels;
  V3 loc, right;
  float head_size;
  float habs[3];  // max(0, pow(1 - h, 4)), src/StereoRecorder.cpp:55-57
  int track0;
};

typedef float (*PowFn)(float, float);
float libm_powf(float x, float y) { return std::pow(x, y); }

// (int)(t * 44100.0) evaluated in double (src/MonoRecorder.cpp:84).  A
// value outside the int range (undefined behaviour in the reference) is
// mapped beyond any window.
inline int64_t sample_index(float t) {
  const double ts = (double)t * 44100.0;
  if (!(ts < 2147483647.0) || !(ts > -2147483648.0)) return (int64_t)1 << 40;
  return (int64_t)(int)ts;
}

// MonoRecorder::Record (src/MonoRecorder.cpp:83-97)
void record_mono(Sink& sk, const ORec& r, int band, float a, float t, float dist) {
  const int64_t s = sample_index(t);
  const float width = std::sqrt(dist);
  float ampl = 2.0f * a / width;
  const int w = (int)std::ceil(width);
  const float step = ampl / (float)w;
  for (int i = 0; i < w; ++i) {
    sk.sample(r.track0, band, i + s, ampl);
    ampl -= step;
  }
}

// StereoRecorder::Record (src/StereoRecorder.cpp:97-130)
void record_stereo(Sink& sk, const ORec& r, int band, V3 dir, float a, float t,
                   float dist, PowFn pw) {
  const float d = dot(dir, r.right);
  const float time_difference = r.head_size / 343.0f;
  const int64_t s_right = sample_index(t - (d * time_difference));
  const int64_t s_left = sample_index(t + (d * time_difference));
  const float width = std::sqrt(dist);
  const float ampl = 2.0f * a / width;
  float al = ampl, ar = ampl;
  const float intensity_difference = std::fabs(d);
  const float factor = pw(r.habs[band], intensity_difference * r.head_size);
  if (d < 0) {
    ar *= factor * factor;
  } else {
    al *= factor * factor;
  }
  const int w = (int)std::ceil(width);
  const float sl = al / (float)w;
  const float sr = ar / (float)w;
  for (int i = 0; i < w; ++i) {
    if (i + s_left >= 0) sk.sample(r.track0, band, i + s_left, al);
    al -= sl;
    if (i + s_right >= 0) sk.sample(r.track0 + 1, band, i + s_right, ar);
    ar -= sr;
  }
}

inline void record(Sink& sk, const ORec& r, int band, V3 dir, float a, float t, float dist,
                   PowFn pw) {
  if (r.channels == 2)
    record_stereo(sk, r, band, dir, a, t, dist, pw);
  else
    record_mono(sk, r, band, a, t, dist);
}

// INV_HEMI_2 / INV_SPHERE_2 (src/Distributions.h:37-43), PI = 3.14159265f
constexpr float kFourPi = 4.0f * 3.14159265f;
inline float inv_hemi_2(float r) { return 2.0f / (kFourPi * r * r); }
inline float inv_sphere_2(float r) { return 1.0f / (kFourPi * r * r); }

struct Emitter {
  std::vector<V3> a, b, c, normal;
  std::vector<float> area;
  float total_area = 0.0f;
};

struct Debug {
  int band = -1;
  uint64_t first = 0;  // the call's first ray (ear_render_params.first_ray)
  int64_t rays = 0;
  int max_record = 0;
  int32_t* hit_tri = nullptr;
  uint8_t* bounce_type = nullptr;
  uint32_t* visible = nullptr;
};

struct Counters {
  uint64_t rays = 0, segments = 0, shadow = 0, contributions = 0, overflows = 0;
};

// One ray of Scene::Render (src/Scene.cpp:124-284).
void trace_ray(const OScene& sc, const Emitter* em, V3 src, const std::vector<ORec>& recs,
               const Rng& rng, uint64_t ray, int band, float air, double cutoff,
               int max_bounces, PowFn pw, Sink& sk, Counters& cnt, const Debug& dbg) {
  const bool mesh_source = em != nullptr;
  const uint64_t local = ray - dbg.first;  // debug records are per call
  const bool dbg_on = dbg.band == band && local < (uint64_t)dbg.rays;
  float intensity = 1.0f;
  float total_path_length = 0.0f;
  V3 prev_ray_dir = {0.0f, 0.0f, 0.0f};
  V3 o = {0, 0, 0}, d = {0, 0, 0};
  cnt.rays++;
  Adjoint* adj = sk.adj;
  if (adj) {
    std::fill(adj->A.begin(), adj->A.end(), 0.0);
    adj->P = adj->T = 0.0;
  }
  struct Flush {  // at the end of the path: grad += T * A
    Adjoint* adj;
    int band;
    ~Flush() {
      if (!adj) return;
      for (int m = 0; m < adj->num_mats; ++m)
        for (int q = 0; q < 2; ++q)
          (*adj->grad)[((size_t)m * 3 + band) * 2 + q] += adj->T * adj->A[(size_t)m * 2 + q];
    }
  } flush{adj, band};
  for (int k = 0; k <= max_bounces; ++k) {
    V3 n = {0, 0, 0};
    int mat = -1;
    int bt = 0;  // 0 REFLECT, 1 REFRACT
    if (k == 0) {
      // AbstractSoundFile::SoundRay (src/SoundFile.cpp:215-228)
      if (mesh_source) {
        // Mesh::SamplePoint (src/Mesh.cpp:143-154) + Triangle::SamplePoint
        // (src/Triangle.cpp:44-53)
        const U4 b = rng.block(ray, 1, 0, 0);
        float x = uniform24(b.v[0]) * em->total_area;
        if (g_tape) g_tape->push_back(uniform24(b.v[0]));
        V3 p = {0, 0, 0}, en = {0, 0, 0};
        for (size_t i = 0; i < em->area.size(); ++i) {
          x -= em->area[i];
          if (x < 0) {
            if (g_tape) {
              g_tape->push_back(uniform24(b.v[1]));
              g_tape->push_back(uniform24(b.v[2]));
            }
            const float r1 = uniform24(b.v[1]);
            const float r2 = uniform24(b.v[2]);
            const float sr1 = std::sqrt(r1);
            const float wa = 1.0f - sr1, wb = sr1 * (1.0f - r2), wc = sr1 * r2;
            const V3 A = em->a[i], B = em->b[i], C = em->c[i];
            p = {(wa * A.x + wb * B.x) + wc * C.x, (wa * A.y + wb * B.y) + wc * C.y,
                 (wa * A.z + wb * B.z) + wc * C.z};
            en = em->normal[i];
            break;
          }
        }
        o = p;
        if (!sample_dir(rng, ray, 0, &en, &d)) cnt.overflows++;
      } else {
        o = src;
        if (!sample_dir(rng, ray, 0, nullptr, &d)) cnt.overflows++;
      }
    } else {
      // Scene::Bounce (src/Scene.cpp:49-82)
      cnt.segments++;
      float t;
      const int hit = closest_hit(sc, o, d, &t);
      if (dbg_on && k <= dbg.max_record) dbg.hit_tri[local * dbg.max_record + (k - 1)] = hit;
      if (hit < 0) break;
      const OTri& tr = sc.tris[(size_t)hit];
      const V3 p = {o.x + d.x * t, o.y + d.y * t, o.z + d.z * t};
      n = (dot(tr.normal, d) > 0.0f) ? neg(tr.normal) : tr.normal;
      mat = tr.mat;
      const OMat& M = sc.mats[(size_t)mat];
      // Material::Bounce (src/Material.cpp:76-83)
      if (!M.always_reflect[band]) {
        const U4 b = rng.block(ray, 0, (uint32_t)k, 0);
        if (g_tape) g_tape->push_back(uniform24(b.v[3]));
        bt = (uniform24(b.v[3]) <= M.p_reflect[band]) ? 0 : 1;
      }
      if (adj) {
        const double fl = M.refl[band], fr = M.refr[band];
        double va = -1.0 / (double)M.survival[band], vr = 0.0;
        if (!M.always_reflect[band]) {
          if (bt == 0) {
            va += -fr / ((fl + fr) * fl);
            vr += -1.0 / fl;
          } else {
            va += 1.0 / (fl + fr);
            vr += 1.0 / fr;
          }
        }
        adj->A[(size_t)mat * 2 + 0] += va;
        adj->A[(size_t)mat * 2 + 1] += vr;
        (*adj->grad)[((size_t)mat * 3 + band) * 2 + 0] -= va * adj->P;
        (*adj->grad)[((size_t)mat * 3 + band) * 2 + 1] -= vr * adj->P;
      }
      const float spec = M.spec[band];
      V3 base;
      if (bt == 1) {
        n = neg(n);
        base = d;
      } else {
        base = reflect(d, n);
      }
      // Sample_Hemi(v, n, refl, factor) (src/Distributions.h:71-75)
      V3 v;
      if (!sample_dir(rng, ray, (uint32_t)k, &n, &v)) cnt.overflows++;
      const float om = 1.0f - spec;
      v = {v.x * om + base.x * spec, v.y * om + base.y * spec, v.z * om + base.z * spec};
      v = normalized(v);
      const V3 dist = sub(p, o);
      const float l = length(dist);
      intensity *= pw(air, l);
      total_path_length += l;
      o = p;
      d = v;
      if (dbg_on && k <= dbg.max_record) dbg.bounce_type[local * dbg.max_record + (k - 1)] = (uint8_t)bt;
    }
    if (k > 0) intensity *= sc.mats[(size_t)mat].survival[band];
    const float before = intensity;
    if (invalid_float(intensity)) break;
    if (k > 0 || mesh_source) {
      const float spec_coef = (mat >= 0) ? sc.mats[(size_t)mat].spec[band] : 0.0f;
      uint32_t vis = 0;
      for (size_t ri = 0; ri < recs.size(); ++ri) {
        const ORec& rec = recs[ri];
        // Scene::Connect (src/Scene.cpp:84-96).  The reference tests the
        // orientation dot > 0 after the visibility; a recorder behind the
        // surface contributes nothing either way, so its visibility test is
        // skipped (and not counted) unless the debug record needs the mask.
        const V3 sdir = sub(rec.loc, o);
        const V3 lsdir = normalized(sdir);
        const float dt = k ? dot(lsdir, n) : 1.0f;
        const bool record_vis = dbg_on && k >= 1 && k <= dbg.max_record;
        if (!(dt > 0) && !record_vis) continue;
        cnt.shadow++;
        if (segment_blocked(sc, o, sdir)) continue;
        vis |= 1u << (ri & 31);
        if (!(dt > 0)) continue;
        float I = before;
        if (k) {
          float factor;
          if (bt == 0) {
            const V3 refl_vector = reflect(prev_ray_dir, n);
            const float diff_factor = -dot(n, prev_ray_dir);
            const float rv = dot(refl_vector, lsdir);
            const float spec_factor = (0.0f < rv) ? rv : 0.0f;
            factor = spec_coef * 1001.0f * pw(spec_factor, 1000.0f) + (1.0f - spec_coef) * diff_factor;
          } else {
            const float diff_factor = dot(n, prev_ray_dir);
            const float rv = dot(prev_ray_dir, lsdir);
            const float spec_factor = (0.0f < rv) ? rv : 0.0f;
            factor = spec_coef * 1001.0f * pw(spec_factor, 1000.0f) + (1.0f - spec_coef) * diff_factor;
          }
          I *= factor;
        }
        const float l = length(sdir);
        I *= pw(air, l);
        I *= inv_hemi_2(l);
        if (!invalid_float(I)) {
          if (k % 2) I *= -1.0f;
          cnt.contributions++;
          if (adj) adj->G = 0.0;
          record(sk, rec, band, lsdir, I, (total_path_length + l) / 343.0f, total_path_length + l, pw);
          if (adj) {
            adj->P += adj->G;
            adj->T += adj->G;
          }
        }
      }
      if (dbg_on && k >= 1 && k <= dbg.max_record) dbg.visible[local * dbg.max_record + (k - 1)] = vis;
    }
    if ((double)intensity < cutoff) break;
    prev_ray_dir = normalized(d);
  }
}

thread_local char g_err[256];

}  // namespace

extern "C" {

// ----------------------------------------------------------------- API
typedef struct oracle_output {
  double* hist64;          // [tracks][3][bins], FP64 re-accumulation
  float* hist32;           // [tracks][3][bins], float accumulation (may be NULL)
  int32_t* first_sample;   // [tracks][3] (may be NULL)
  int32_t* last_sample;    // [tracks][3] (may be NULL)
  uint64_t* counters;      // [5]: rays, segments, shadow, contributions, overflows
  // debug recording (band debug_band, rays < debug_rays)
  int32_t debug_band;
  int32_t debug_max_record;
  int64_t debug_rays;
  int32_t* hit_tri;
  uint8_t* bounce_type;
  uint32_t* visible;
} oracle_output;

const char* oracle_last_error(void) { return g_err; }

int ear_num_tracks_oracle(const ear_recorder* r, int32_t n) {
  int t = 0;
  for (int i = 0; i < n; ++i) t += r[i].channels == 2 ? 2 : 1;
  return t;
}

float oracle_powf(float x, float y) { return portable_powf(x, y); }

void oracle_philox(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0, uint32_t k1,
                   uint32_t* out) {
  const U4 r = philox4x32_10(c0, c1, c2, c3, k0, k1);
  for (int i = 0; i < 4; ++i) out[i] = r.v[i];
}

int oracle_material(const ear_material* m, float* survival, float* p_reflect,
                    int32_t* always_reflect, float* spec) {
  OMat o;
  if (!derive_material(*m, &o)) return 1;
  for (int i = 0; i < 3; ++i) {
    survival[i] = o.survival[i];
    p_reflect[i] = o.p_reflect[i];
    always_reflect[i] = o.always_reflect[i];
    spec[i] = o.spec[i];
  }
  return 0;
}

}  // extern "C"

namespace {

// Scene::Render for every band in params->bands_mask (rays of a band are
// split over num_threads threads in contiguous chunks).  pow_mode 0 =
// portable_powf, 1 = libm powf.  With adj_g set, the same rays are replayed
// in adjoint mode instead: nothing is recorded, adj_grad[material][band][2]
// receives the gradient of sum(adj_g * raw splat sums).
int render_impl(const ear_scene_desc* desc, const ear_source* source,
                const ear_recorder* recorders, int32_t num_recorders,
                const ear_render_params* params, int32_t num_threads, int32_t pow_mode,
                oracle_output* out, const double* adj_g, double* adj_grad) {
  g_err[0] = 0;
  if (!desc || !source || !params || !out || !out->hist64 || num_recorders < 0 ||
      (num_recorders > 0 && !recorders) || params->num_bins <= 0) {
    std::snprintf(g_err, sizeof g_err, "invalid argument");
    return 1;
  }
  const PowFn pw = pow_mode == 1 ? libm_powf : portable_powf;
  OScene sc;
  sc.mats.resize((size_t)desc->num_materials);
  for (int i = 0; i < desc->num_materials; ++i)
    if (!derive_material(desc->materials[i], &sc.mats[(size_t)i])) {
      std::snprintf(g_err, sizeof g_err, "Invalid material settings (material %d)", i);
      return 1;
    }
  sc.tris.resize((size_t)desc->num_triangles);
  for (int64_t i = 0; i < desc->num_triangles; ++i) {
    const float* v = desc->vertices + 9 * i;
    OTri& t = sc.tris[(size_t)i];
    const V3 a = load3(v), b = load3(v + 3), c = load3(v + 6);
    t.v0 = a;
    t.e1 = sub(b, a);
    t.e2 = sub(c, a);
    t.normal = normalized(cross(t.e1, t.e2));
    t.mat = desc->material_ids[i];
    if (t.mat < 0 || t.mat >= desc->num_materials) {
      std::snprintf(g_err, sizeof g_err, "material id out of range at triangle %lld", (long long)i);
      return 1;
    }
  }
  Emitter em;
  const bool mesh_source = source->num_emitter_triangles > 0;
  if (mesh_source) {
    for (int64_t i = 0; i < source->num_emitter_triangles; ++i) {
      const float* v = source->emitter_vertices + 9 * i;
      const V3 a = load3(v), b = load3(v + 3), c = load3(v + 6);
      em.a.push_back(a);
      em.b.push_back(b);
      em.c.push_back(c);
      em.normal.push_back(normalized(cross(sub(b, a), sub(c, a))));
      // Triangle::calcArea: |edge(0) x edge(1)| / 2 (src/Triangle.cpp:26-30)
      const float ar = length(cross(sub(b, a), sub(c, b))) / 2.0f;
      em.area.push_back(ar);
      em.total_area += ar;  // Mesh::Mesh (src/Mesh.cpp:90)
    }
  }
  std::vector<ORec> recs((size_t)num_recorders);
  int num_tracks = 0;
  for (int i = 0; i < num_recorders; ++i) {
    const ear_recorder& r = recorders[i];
    ORec& o = recs[(size_t)i];
    o.channels = r.channels == 2 ? 2 : 1;
    o.loc = load3(r.location);
    o.right = load3(r.right_ear);
    o.head_size = r.head_size;
    for (int b = 0; b < 3; ++b) {
      const float h = portable_powf(1.0f - r.head_absorption[b], 4.0f);
      o.habs[b] = (0.0f < h) ? h : 0.0f;  // std::max(0.0f, ...)
    }
    o.track0 = num_tracks;
    num_tracks += o.channels;
  }
  const int nb = params->num_bins;
  const int nthreads = std::max(1, (int)num_threads);
  const Rng rng0 = {(uint32_t)params->seed, (uint32_t)(params->seed >> 32), params->context, 0};
  const V3 src = load3(source->location);
  Debug dbg;
  dbg.first = params->first_ray;
  if (out->hit_tri && out->bounce_type && out->visible && out->debug_max_record > 0) {
    dbg.band = out->debug_band;
    dbg.rays = out->debug_rays;
    dbg.max_record = out->debug_max_record;
    dbg.hit_tri = out->hit_tri;
    dbg.bounce_type = out->bounce_type;
    dbg.visible = out->visible;
    for (int64_t i = 0; i < dbg.rays * dbg.max_record; ++i) {
      dbg.hit_tri[i] = -2;
      dbg.bounce_type[i] = 0;
      dbg.visible[i] = 0;
    }
  }
  std::vector<OTrack> tracks((size_t)num_tracks * 3);
  for (auto& t : tracks) {
    t.h64.assign((size_t)nb, 0.0);
    t.h32.assign((size_t)nb, 0.0f);
  }
  Counters total;
  for (int band = 0; band < 3; ++band) {
    if (!(params->bands_mask & (1u << band))) continue;
    Rng rng = rng0;
    rng.band = (uint32_t)band;
    const float air = 1.0f - params->air_absorption[band];
    const uint64_t N = params->num_rays;
    std::vector<std::vector<OTrack>> priv((size_t)nthreads);
    std::vector<Counters> cnts((size_t)nthreads);
    std::vector<std::vector<double>> tgrad((size_t)nthreads);
    auto work = [&](int tid) {
      std::vector<OTrack>& pt = priv[(size_t)tid];
      pt.assign(tracks.size(), OTrack());
      for (int tr = 0; tr < num_tracks; ++tr) {
        pt[(size_t)tr * 3 + band].h64.assign((size_t)nb, 0.0);
        pt[(size_t)tr * 3 + band].h32.assign((size_t)nb, 0.0f);
      }
      Sink sk;
      sk.num_bins = nb;
      sk.tracks = &pt;
      Adjoint adj;
      if (adj_g) {
        adj.g = adj_g;
        adj.nb = nb;
        adj.num_mats = (int)sc.mats.size();
        adj.A.assign(sc.mats.size() * 2, 0.0);
        adj.grad = &tgrad[(size_t)tid];
        adj.grad->assign(sc.mats.size() * 3 * 2, 0.0);
        sk.adj = &adj;
      }
      const uint64_t lo = N * (uint64_t)tid / (uint64_t)nthreads;
      const uint64_t hi = N * (uint64_t)(tid + 1) / (uint64_t)nthreads;
      for (uint64_t r = lo; r < hi; ++r)
        trace_ray(sc, mesh_source ? &em : nullptr, src, recs, rng, params->first_ray + r, band, air,
                  params->cutoff, params->max_bounces, pw, sk, cnts[(size_t)tid], dbg);
    };
    if (nthreads == 1) {
      work(0);
    } else {
      std::vector<std::thread> th;
      for (int t = 0; t < nthreads; ++t) th.emplace_back(work, t);
      for (auto& t : th) t.join();
    }
    if (adj_g)
      for (int t = 0; t < nthreads; ++t)
        for (size_t i = 0; i < tgrad[(size_t)t].size(); ++i) adj_grad[i] += tgrad[(size_t)t][i];
    for (int t = 0; t < nthreads; ++t) {
      for (int tr = 0; tr < num_tracks; ++tr) {
        OTrack& dst = tracks[(size_t)tr * 3 + band];
        const OTrack& s = priv[(size_t)t][(size_t)tr * 3 + band];
        for (int i = 0; i < nb; ++i) {
          dst.h64[(size_t)i] += s.h64[(size_t)i];
          dst.h32[(size_t)i] += s.h32[(size_t)i];
        }
        dst.first = std::min(dst.first, s.first);
        dst.last = std::max(dst.last, s.last);
      }
      total.rays += cnts[(size_t)t].rays;
      total.segments += cnts[(size_t)t].segments;
      total.shadow += cnts[(size_t)t].shadow;
      total.contributions += cnts[(size_t)t].contributions;
      total.overflows += cnts[(size_t)t].overflows;
    }
    // End of Scene::Render (src/Scene.cpp:286-316)
    if (params->flags & EAR_FLAG_RAW) continue;
    // float amount accumulated one ray at a time (src/Scene.cpp:122,127):
    // exact up to 2^24, then stuck.
    const float amount = N <= 16777216ull ? (float)N : 16777216.0f;
    const float inv_amount = 1.0f / amount;
    const float gain2 = source->gain * source->gain;
    Sink sk;
    sk.num_bins = nb;
    sk.tracks = &tracks;
    for (int ri = 0; ri < num_recorders; ++ri) {
      const ORec& rec = recs[(size_t)ri];
      // Recorder::Multiply -> FloatBuffer::Multiply over [first, real_length)
      for (int c = 0; c < rec.channels; ++c) {
        OTrack& t = tracks[(size_t)(rec.track0 + c) * 3 + band];
        for (int64_t i = t.first; i < t.last && i < nb; ++i) {
          t.h64[(size_t)i] *= (double)inv_amount;
          t.h32[(size_t)i] *= inv_amount;
        }
      }
      if (!mesh_source && !(params->flags & EAR_FLAG_NO_DIRECT)) {
        const V3 seg = sub(src, rec.loc);
        if (!segment_blocked(sc, rec.loc, seg)) {
          const V3 dist = sub(rec.loc, src);
          const float len = length(dist);
          const V3 dir = normalized(dist);
          record(sk, rec, band, dir, inv_sphere_2(len) * pw(air, len) * params->dry_level,
                 len / 343.0f, len, pw);
        }
      }
      for (int c = 0; c < rec.channels; ++c) {
        OTrack& t = tracks[(size_t)(rec.track0 + c) * 3 + band];
        for (int64_t i = t.first; i < t.last && i < nb; ++i) {
          t.h64[(size_t)i] *= (double)gain2;
          t.h32[(size_t)i] *= gain2;
        }
      }
    }
  }
  for (int tr = 0; tr < num_tracks; ++tr)
    for (int b = 0; b < 3; ++b) {
      const OTrack& t = tracks[(size_t)tr * 3 + b];
      const size_t off = ((size_t)tr * 3 + b) * (size_t)nb;
      std::memcpy(out->hist64 + off, t.h64.data(), sizeof(double) * (size_t)nb);
      if (out->hist32) std::memcpy(out->hist32 + off, t.h32.data(), sizeof(float) * (size_t)nb);
      if (out->first_sample) out->first_sample[tr * 3 + b] = (int32_t)std::min<int64_t>(t.first, nb);
      if (out->last_sample) out->last_sample[tr * 3 + b] = (int32_t)std::min<int64_t>(t.last, nb);
    }
  if (out->counters) {
    out->counters[0] = total.rays;
    out->counters[1] = total.segments;
    out->counters[2] = total.shadow;
    out->counters[3] = total.contributions;
    out->counters[4] = total.overflows;
  }
  return 0;
}

}  // namespace

extern "C" {

int oracle_render(const ear_scene_desc* desc, const ear_source* source,
                  const ear_recorder* recorders, int32_t num_recorders,
                  const ear_render_params* params, int32_t num_threads, int32_t pow_mode,
                  oracle_output* out) {
  return render_impl(desc, source, recorders, num_recorders, params, num_threads, pow_mode, out,
                     nullptr, nullptr);
}

// The uniforms a single-threaded render of one band consumes, in the order
// the reference's global generator is called (see g_tape): up to `cap`
// values into `tape`, the full count in *used.  Same arguments as
// oracle_render; bands_mask must select exactly one band.
int oracle_random_tape(const ear_scene_desc* desc, const ear_source* source,
                       const ear_recorder* recorders, int32_t num_recorders,
                       const ear_render_params* params, float* tape, int64_t cap,
                       int64_t* used) {
  if (!params || (params->bands_mask != 1u && params->bands_mask != 2u && params->bands_mask != 4u) ||
      !used || (cap > 0 && !tape)) {
    std::snprintf(g_err, sizeof g_err, "invalid argument");
    return 1;
  }
  std::vector<float> t;
  g_tape = &t;
  const int nb = params->num_bins > 0 ? params->num_bins : 1;
  int ntr = 0;
  for (int i = 0; i < num_recorders; ++i) ntr += recorders[i].channels == 2 ? 2 : 1;
  std::vector<double> h64((size_t)std::max(1, ntr) * 3 * (size_t)nb);
  oracle_output out;
  std::memset(&out, 0, sizeof out);
  out.hist64 = h64.data();
  const int rc = render_impl(desc, source, recorders, num_recorders, params, 1, 0, &out, nullptr,
                             nullptr);
  g_tape = nullptr;
  *used = (int64_t)t.size();
  if (cap > 0) std::memcpy(tape, t.data(), sizeof(float) * (size_t)std::min<int64_t>(cap, *used));
  return rc;
}

// FP64 reference gradient of L = sum(g * h) with respect to each material's
// per-band absorption and refraction (refl = 1 - absorption - refraction),
// h being the finalized histogram of oracle_render with the same
// arguments; grad[material][band][0 = absorption, 1 = refraction].  The
// finalize steps scale each bin by 1/N when it lies in the pre-direct
// [first_sample, real_length) and by gain^2 when it lies in the final one
// (src/Scene.cpp:291,314): the upstream gradient is scaled the same way.
int oracle_render_adjoint(const ear_scene_desc* desc, const ear_source* source,
                          const ear_recorder* recorders, int32_t num_recorders,
                          const ear_render_params* params, int32_t num_threads, int32_t pow_mode,
                          const double* g, double* grad) {
  const int nb = params->num_bins;
  const int tracks = ear_num_tracks_oracle(recorders, num_recorders);
  const size_t rows = (size_t)tracks * 3;
  std::vector<double> h64(rows * (size_t)nb), gs(rows * (size_t)nb, 0.0);
  std::vector<int32_t> f_raw(rows), l_raw(rows), f_fin(rows), l_fin(rows);
  oracle_output o = {};
  o.hist64 = h64.data();
  o.first_sample = f_raw.data();
  o.last_sample = l_raw.data();
  ear_render_params raw = *params;
  raw.flags |= EAR_FLAG_RAW;
  int rc = render_impl(desc, source, recorders, num_recorders, &raw, num_threads, pow_mode, &o,
                       nullptr, nullptr);
  if (rc) return rc;
  const bool scaled = !(params->flags & EAR_FLAG_RAW);
  if (scaled) {
    o.first_sample = f_fin.data();
    o.last_sample = l_fin.data();
    rc = render_impl(desc, source, recorders, num_recorders, params, num_threads, pow_mode, &o,
                     nullptr, nullptr);
    if (rc) return rc;
  }
  const uint64_t N = params->num_rays;
  const float amount = N <= 16777216ull ? (float)N : 16777216.0f;
  const double inv = (double)(1.0f / amount);
  const double gain2 = (double)(source->gain * source->gain);
  for (size_t r = 0; r < rows; ++r)
    for (int i = 0; i < nb; ++i) {
      double sc = 1.0;
      if (scaled) {
        if (i >= f_raw[r] && i < l_raw[r]) sc *= inv;
        if (i >= f_fin[r] && i < l_fin[r]) sc *= gain2;
      }
      gs[r * (size_t)nb + i] = g[r * (size_t)nb + i] * sc;
    }
  for (int i = 0; i < desc->num_materials * 3 * 2; ++i) grad[i] = 0.0;
  o = {};
  o.hist64 = h64.data();
  return render_impl(desc, source, recorders, num_recorders, params, num_threads, pow_mode, &o,
                     gs.data(), grad);
}

// Brute-force query probes (for the traversal parity tests).
int oracle_closest_hit(const ear_scene_desc* desc, int64_t num_rays, const float* origins,
                       const float* dirs, int32_t* hit, float* t_out) {
  OScene sc;
  sc.tris.resize((size_t)desc->num_triangles);
  for (int64_t i = 0; i < desc->num_triangles; ++i) {
    const float* v = desc->vertices + 9 * i;
    OTri& t = sc.tris[(size_t)i];
    t.v0 = load3(v);
    t.e1 = sub(load3(v + 3), t.v0);
    t.e2 = sub(load3(v + 6), t.v0);
  }
  for (int64_t r = 0; r < num_rays; ++r) {
    float t;
    hit[r] = closest_hit(sc, load3(origins + 3 * r), load3(dirs + 3 * r), &t);
    if (t_out) t_out[r] = t;
  }
  return 0;
}

int oracle_segment_blocked(const ear_scene_desc* desc, int64_t num_rays, const float* origins,
                           const float* dirs, uint8_t* blocked) {
  OScene sc;
  sc.tris.resize((size_t)desc->num_triangles);
  for (int64_t i = 0; i < desc->num_triangles; ++i) {
    const float* v = desc->vertices + 9 * i;
    OTri& t = sc.tris[(size_t)i];
    t.v0 = load3(v);
    t.e1 = sub(load3(v + 3), t.v0);
    t.e2 = sub(load3(v + 6), t.v0);
  }
  for (int64_t r = 0; r < num_rays; ++r)
    blocked[r] = segment_blocked(sc, load3(origins + 3 * r), load3(dirs + 3 * r)) ? 1 : 0;
  return 0;
}

// ------------------------------------------------ FloatBuffer post-process
// Restated from src/Recorder.cpp; the track holds `capacity` samples and
// [first, last) is the FloatBuffer range (first_sample, real_length).

// FloatBuffer::Power (src/Recorder.cpp:103-108)
void oracle_track_power(float* data, int32_t first, int32_t last, float a) {
  for (int32_t i = first; i < last; ++i) {
    const float f = std::pow(std::fabs(data[i]), a);
    data[i] = data[i] < 0 ? (f * -1.0f) : f;
  }
}
// FloatBuffer::Maximum (src/Recorder.cpp:76-83)
float oracle_track_maximum(const float* data, int32_t first, int32_t last) {
  float x = 0.0f;
  for (int32_t i = first; i < last; ++i) {
    const float a = std::fabs(data[i]);
    if (a > x) x = a;
  }
  return x;
}
// FloatBuffer::getLength(tresh) (src/Recorder.cpp:110-118)
int32_t oracle_track_length(const float* data, int32_t capacity, int32_t first, int32_t last,
                            float tresh) {
  if (tresh < 0.0f) return last;
  int32_t mx = 0;
  for (int32_t i = first; i < capacity; ++i)
    if (std::fabs(data[i]) >= tresh) mx = i;
  return mx + 1;
}
// RecorderTrack::T60 (src/Recorder.cpp:303-340).  The reference reads two
// uninitialised ints when no decreasing sample is found; 0 is used here.
float oracle_track_t60(const float* data, int32_t first, int32_t last) {
  const float attenuation_gain = std::pow(10.0f, 60.0f / 20.0f);
  float direct_intensity = 0.0f, min_gain = 0.0f;
  int last_significant_offset = 0, direct_sound_offset = 0;
  float previous_sample = -1.0f;
  bool inside_indirect_lobe = false;
  for (int32_t j = first; j < last; ++j) {
    const float sample = data[j];
    if (inside_indirect_lobe) {
      if (sample > min_gain) last_significant_offset = j;
    } else if (sample < previous_sample) {
      inside_indirect_lobe = true;
      direct_intensity = previous_sample;
      min_gain = direct_intensity / attenuation_gain;
      direct_sound_offset = j;
    }
    previous_sample = sample;
  }
  return (float)(last_significant_offset - direct_sound_offset) / 44100.0f;
}


// ----------------------------------------------------------- auralisation
// Equalizer (lib/equalizer/Equalizer.cpp:26-96): 4th-order Linkwitz-Riley
// passes, restated with the same constants and operation order.
struct OLr {
  float b1, b2, b3, b4, a0, a1, a2, a3, a4;
  float xm1 = 0, xm2 = 0, xm3 = 0, xm4 = 0, ym1 = 0, ym2 = 0, ym3 = 0, ym4 = 0;
  OLr(float fc, bool high) {
    const float srate = 44100.0f;
    const float pi = 3.14285714285714f;
    float wc = 2.0f * pi * srate;
    float wc2 = wc * wc;
    float wc3 = wc2 * wc;
    float wc4 = wc2 * wc2;
    float k = wc / std::tan(pi * fc / srate);
    float k2 = k * k;
    float k3 = k2 * k;
    float k4 = k2 * k2;
    float sqrt2 = std::sqrt(2.0f);
    float sq_tmp1 = sqrt2 * wc3 * k;
    float sq_tmp2 = sqrt2 * wc * k3;
    float a_tmp = 4.0f * wc2 * k2 + 2.0f * sq_tmp1 + k4 + 2.0f * sq_tmp2 + wc4;
    b1 = (4.0f * (wc4 + sq_tmp1 - k4 - sq_tmp2)) / a_tmp;
    b2 = (6.0f * wc4 - 8.0f * wc2 * k2 + 6.0f * k4) / a_tmp;
    b3 = (4.0f * (wc4 - sq_tmp1 + sq_tmp2 - k4)) / a_tmp;
    b4 = (k4 - 2.0f * sq_tmp1 + wc4 - 2.0f * sq_tmp2 + 4.0f * wc2 * k2) / a_tmp;
    const float g = high ? k4 : wc4;
    a0 = g / a_tmp;
    a1 = (high ? -4.0f : 4.0f) * g / a_tmp;
    a2 = 6.0f * g / a_tmp;
    a3 = a1;
    a4 = a0;
  }
  float step(float in) {
    const float out = a0 * in + a1 * xm1 + a2 * xm2 + a3 * xm3 + a4 * xm4 - b1 * ym1 - b2 * ym2 -
                      b3 * ym3 - b4 * ym4;
    xm4 = xm3; xm3 = xm2; xm2 = xm1; xm1 = in;
    ym4 = ym3; ym3 = ym2; ym2 = ym1; ym1 = out;
    return out;
  }
};

// FloatBuffer with the reference's growth and bookkeeping
// (src/Recorder.cpp:33-66): writes through at(), reads through get().
struct OBuf {
  std::vector<float> data;
  int64_t real_length = 0, first_sample = 3 * 44100 - 1;
  OBuf() : data((size_t)(3 * 44100), 0.0f) {}
  int64_t length() const { return (int64_t)data.size(); }
  float& at(int64_t i) {
    if (i >= length()) data.resize((size_t)(i + 44100), 0.0f);
    if (i > real_length) real_length = i;
    if (i < first_sample) first_sample = i;
    return data[(size_t)i];
  }
  float get(int64_t i) const { return i < length() ? data[(size_t)i] : 0.0f; }
};

int64_t copy_out(const OBuf& b, float* out, int64_t out_cap) {
  const int64_t n = std::min(out_cap, b.length());
  std::memcpy(out, b.data.data(), sizeof(float) * (size_t)n);
  for (int64_t i = n; i < out_cap; ++i) out[i] = 0.0f;
  return b.length();
}

// A response track as the caller passes it: `cap` samples at p, zero
// beyond (the const FloatBuffer::operator[]).
struct OResp {
  const float* p;
  int64_t cap;
  float get(int64_t j) const { return j < cap ? p[j] : 0.0f; }
};

// Equalizer::Split (lib/equalizer/Equalizer.cpp:81-96) as SoundFile::Band
// calls it (frequencies in kHz times 1000, src/SoundFile.cpp:153).
void oracle_band_split(const float* data, int64_t n, float f1k, float f2k, float f3k, float* low,
                       float* mid, float* high) {
  const float f1 = f1k * 1000.0f, f2 = f2k * 1000.0f, f3 = f3k * 1000.0f;
  const float fc1 = (f1 + f2) / 2.0f;
  const float fc2 = (f2 + f3) / 2.0f;
  OLr hi_pass1(fc1, true), hi_pass2(fc2, true), lo_pass1(fc1, false), lo_pass2(fc2, false);
  for (int64_t i = 0; i < n; ++i) {
    high[i] = hi_pass2.step(data[i]);
    low[i] = lo_pass1.step(data[i]);
    mid[i] = lo_pass2.step(data[i]);
    mid[i] = hi_pass1.step(mid[i]);
  }
}

// RecorderTrack::Process of builds without FFTW (src/Recorder.cpp:247-292),
// loop for loop: the plain variant over [first, len) of the track, the
// keyframe variant (ir2 != NULL) over [min first, max len) of both with the
// linear interpolation.  Writes the processed track (zero-padded to
// out_cap) and returns its FloatBuffer capacity.
int64_t oracle_process_direct(const float* ir, int64_t cap, int64_t first, int64_t len,
                              const float* ir2, int64_t cap2, int64_t first2, int64_t len2,
                              const float* dry, int64_t n, int64_t offset, float* out,
                              int64_t out_cap) {
  OBuf result;
  const OResp a{ir, cap}, b{ir2, cap2};
  if (!ir2) {
    for (int64_t i = 0; i < n; ++i) {
      const float sfs = dry[i];
      int64_t index = i + offset + first;
      for (int64_t j = first; j < len; ++j) result.at(index++) += sfs * a.get(j);
    }
  } else {
    const float flt_samples = 1.0f / (float)(uint32_t)n;
    const int64_t l = std::max(len, len2);
    const int64_t f = std::min(first, first2);
    for (int64_t i = 0; i < n; ++i) {
      const float i1 = (float)(uint32_t)i * flt_samples;
      const float i2 = 1.0f - i1;
      const float sfs = dry[i];
      int64_t index = i + offset + f;
      for (int64_t j = f; j < l; ++j) {
        const float p = i2 * a.get(j) + i1 * b.get(j);
        result.at(index++) += sfs * p;
      }
    }
  }
  return copy_out(result, out, out_cap);
}

// The FFT variant (src/Recorder.cpp:145-243) in double precision: the
// response [0, len) convolved with the dry section, faded as the reference
// fades it (FP32 ramp stepped in sequence, FP32 products), written to
// offset + [0, len + n + 1).  For a keyframe pair the faded-out and faded-in
// results are summed (RecorderTrack::Add).  out64 receives the values,
// zero-padded to out_cap; the return value is the capacity of the processed
// track.
int64_t oracle_process_fft64(const float* ir, int64_t cap, int64_t len, const float* ir2,
                             int64_t cap2, int64_t len2, const float* dry, int64_t n,
                             int64_t offset, double* out64, int64_t out_cap) {
  for (int64_t i = 0; i < out_cap; ++i) out64[i] = 0.0;
  auto one = [&](const OResp& t, int64_t m, int fade, OBuf* shape) {
    std::vector<float> b((size_t)n);
    for (int64_t i = 0; i < n; ++i) b[(size_t)i] = dry[i];
    if (fade != 0) {
      float factor = fade < 0 ? 1.0f : 0.0f;
      const float df = (fade < 0 ? -1.0f : 1.0f) / (float)(uint32_t)n;
      for (int64_t i = 0; i < n; ++i) {
        b[(size_t)i] *= factor;
        factor += df;
      }
    }
    const int64_t mn = m + n + 1;
    for (int64_t x = 0; x < mn; ++x) {
      double acc = 0.0;
      const int64_t lo = std::max<int64_t>(0, x - (m - 1)), hi = std::min<int64_t>(n - 1, x);
      for (int64_t i = lo; i <= hi; ++i) acc += (double)b[(size_t)i] * (double)t.get(x - i);
      if (offset + x < out_cap) out64[offset + x] += acc;
      shape->at(offset + x) += 0.0f;  // the reference writes every index
    }
  };
  OBuf ra;
  one(OResp{ir, cap}, len, ir2 ? -1 : 0, &ra);
  if (!ir2) return ra.length();
  OBuf rb;
  one(OResp{ir2, cap2}, len2, 1, &rb);
  const int64_t lb = rb.length();  // RecorderTrack::Add reads getLength(0.0f)
  for (int64_t i = 0; i < lb; ++i) ra.at(i) += rb.get(i);
  return ra.length();
}

}  // extern "C"
