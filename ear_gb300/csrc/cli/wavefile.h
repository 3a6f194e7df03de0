// wavefile.h -- WAV input and output of the EAR command line, with the
// conventions of the reference's WaveFile (lib/wave/WaveFile.cpp).
#pragma once

#include <string>
#include <vector>

namespace wav {

// WaveFile(fn).ToFloat() (lib/wave/WaveFile.cpp:36-110,157-188): PCM
// (format 1) with 8, 16 or 24 bits; every sample frame becomes the mean of
// its channels, each divided by 2^(bits-1).  Returns false when the file
// cannot be opened or holds no such data (the reference then reports
// "Failed to open sound file").  Unlike the reference, chunks before or
// after "data" and a longer "fmt " chunk are skipped properly.
bool read_float(const std::string& fn, std::vector<float>* out);

// WaveFile::FromFloat + Save: 16-bit PCM at 44.1 kHz.  One channel
// (lib/wave/WaveFile.cpp:190-222): with norm, divide by max|x|/0.8 when
// norm_max < 0, else by norm_max/0.95.  Two channels (:224-255): with norm,
// divide by (the largest signed sample of both)/0.8; the shorter channel is
// zero-padded.  Samples are converted with (short)(x / max * 32768.0f).
bool write(const std::string& fn, const std::vector<const float*>& ch,
           const std::vector<int>& len, bool norm, float norm_max);

}  // namespace wav
