// ear_record.cuh -- the recorder splat arithmetic shared by the trace
// kernels (path contributions) and the finalize kernel (direct sound).
#pragma once

#include "ear_internal.h"

namespace ear {

constexpr int kInitialFirstSample = 3 * 44100 - 1;  // src/Recorder.cpp:46

// (int)(t * 44100.0) evaluated in double as the reference does
// (src/MonoRecorder.cpp:84); values outside the int range (undefined
// behaviour in the reference) are mapped beyond any window.
//
// On the device the same value comes from single precision (the GB300's
// double-precision rate is a small fraction of its single-precision rate):
// the double product of a float and 44100 (14 significant bits) is exact
// and equals p + e, p = fl(t * 44100), e = fma(t, 44100, -p) exactly
// (Dekker's two-product).  Below 2^24 the floats are dense enough that
// trunc(p + e) differs from trunc(p) only when p is integral, and then by
// one step towards zero as e pushes it under (or, for negative p, over)
// that integer.  Larger products take the double path.
EAR_HD long long sample_index(float t) {
#ifdef __CUDA_ARCH__
  const float p = __fmul_rn(t, 44100.0f);
  if (fabsf(p) < 16777216.0f) {
    const float e = __fmaf_rn(t, 44100.0f, -p);
    float q = truncf(p);
    if (q == p) {
      if (p > 0.0f && e < 0.0f) q -= 1.0f;
      if (p < 0.0f && e > 0.0f) q += 1.0f;
    }
    return (long long)(int)q;
  }
#endif
  const double ts = (double)t * 44100.0;
  if (!(ts < 2147483647.0) || !(ts > -2147483648.0)) return (long long)1 << 40;
  return (long long)(int)ts;
}

// One Record() call: per track, the first sample s, the first amplitude
// and the per-sample decrement of the triangular splat of width w.
struct SplatPlan {
  long long s[2];
  float ampl[2];
  float step[2];
  int w;
  int tracks;
};

// MonoRecorder::Record (src/MonoRecorder.cpp:83-97) and
// StereoRecorder::Record (src/StereoRecorder.cpp:97-130): interaural time
// shift +-dot(dir, ear) * head / 343 s, intensity factor
// head_absorption[band]^(|dot| head) squared on the far ear.  FAST: the
// power of the fast kernels (pow_sel).
template <bool FAST>
EAR_HD SplatPlan record_plan(const DevRecorder& R, int band, V3 dir, float amp, float t,
                             float dist) {
  SplatPlan p;
  const float width = f_sqrt(dist);
  p.w = (int)f_ceil(width);
  const float ampl = 2.0f * amp / width;
  if (R.channels == 2) {
    const float dt = dot(dir, mk(R.right[0], R.right[1], R.right[2]));
    const float time_difference = R.head_size / 343.0f;
    p.s[1] = sample_index(t - (dt * time_difference));  // right
    p.s[0] = sample_index(t + (dt * time_difference));  // left
    float al = ampl, ar = ampl;
    const float factor = pow_sel<FAST>(R.habs[band], f_abs(dt) * R.head_size);
    if (dt < 0) {
      ar *= factor * factor;
    } else {
      al *= factor * factor;
    }
    p.ampl[0] = al;
    p.ampl[1] = ar;
    p.step[0] = al / (float)p.w;
    p.step[1] = ar / (float)p.w;
    p.tracks = 2;
  } else {
    p.s[0] = sample_index(t);
    p.ampl[0] = ampl;
    p.step[0] = ampl / (float)p.w;
    p.s[1] = 0;
    p.ampl[1] = 0.0f;
    p.step[1] = 0.0f;
    p.tracks = 1;
  }
  return p;
}

}  // namespace ear
