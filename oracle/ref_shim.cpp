// ref_shim.cpp -- C entry points into the two reference libraries that
// compile on their own: lib/equalizer/Equalizer.cpp (the band split) and
// lib/wave/WaveFile.cpp (WAV input and output).
//
// TEST INFRASTRUCTURE ONLY.  oracle/build_ref.py compiles this file with
// those two reference sources, where they lie in the reference tree, into
// oracle/_ref/ (never committed).  The tests use it to pin the oracle's
// band split and the CLI's WAV reader and writer to the reference itself;
// nothing in the product loads it.
#include <cstdlib>
#include <cstring>

#include "Equalizer.h"
#include "WaveFile.h"

extern "C" {

// Equalizer::Split (lib/equalizer/Equalizer.cpp:81-96); f1..f3 in Hz.
void ref_equalizer_split(float* data, float* low, float* mid, float* high, unsigned length,
                         float f1, float f2, float f3) {
  Equalizer::Split(data, low, mid, high, length, f1, f2, f3);
}

// WaveFile(fn).ToFloat() as SoundFile::SoundFile uses it
// (src/SoundFile.cpp:33-42): copies up to cap samples, returns the sample
// count (GetSampleSize), or -1 when ToFloat returns no data.
long ref_wave_to_float(const char* fn, float* out, unsigned cap) {
  WaveFile w(fn);
  float* f = w.ToFloat();
  if (!f) return -1;
  const unsigned n = w.GetSampleSize();
  std::memcpy(out, f, sizeof(float) * (n < cap ? n : cap));
  delete[] f;
  return (long)n;
}

// WaveFile::FromFloat + Save, mono (lib/wave/WaveFile.cpp:190-222).
void ref_wave_save_mono(const char* fn, const float* f, int length, int norm, float max) {
  WaveFile w;
  w.FromFloat(f, length, norm != 0, max);
  w.Save(fn);
}

// WaveFile::FromFloat + Save, stereo (lib/wave/WaveFile.cpp:224-255).
void ref_wave_save_stereo(const char* fn, const float* left, const float* right, int length1,
                          int length2, int norm) {
  WaveFile w;
  w.FromFloat(left, right, length1, length2, norm != 0);
  w.Save(fn);
}

}  // extern "C"
