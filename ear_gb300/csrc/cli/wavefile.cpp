// wavefile.cpp -- see wavefile.h.
#include "wavefile.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>

namespace wav {
namespace {

uint32_t u32(const uint8_t* p) { return p[0] | (p[1] << 8) | (p[2] << 16) | ((uint32_t)p[3] << 24); }
uint16_t u16(const uint8_t* p) { return (uint16_t)(p[0] | (p[1] << 8)); }

void put32(std::FILE* f, uint32_t v) {
  const uint8_t b[4] = {(uint8_t)v, (uint8_t)(v >> 8), (uint8_t)(v >> 16), (uint8_t)(v >> 24)};
  std::fwrite(b, 1, 4, f);
}
void put16(std::FILE* f, uint16_t v) {
  const uint8_t b[2] = {(uint8_t)v, (uint8_t)(v >> 8)};
  std::fwrite(b, 1, 2, f);
}

}  // namespace

bool read_float(const std::string& fn, std::vector<float>* out) {
  out->clear();
  std::FILE* f = std::fopen(fn.c_str(), "rb");
  if (!f) return false;
  std::vector<uint8_t> bytes;
  uint8_t buf[65536];
  size_t got;
  while ((got = std::fread(buf, 1, sizeof buf, f)) > 0) bytes.insert(bytes.end(), buf, buf + got);
  std::fclose(f);
  if (bytes.size() < 12 || std::memcmp(bytes.data() + 8, "WAVE", 4) != 0) return false;
  int channels = 0, bits = 0;
  bool have_fmt = false;
  std::vector<uint8_t> data;
  size_t at = 12;
  while (at + 8 <= bytes.size()) {
    const uint8_t* h = bytes.data() + at;
    const size_t size = u32(h + 4);
    const size_t body = at + 8;
    const size_t avail = std::min(size, bytes.size() - body);
    if (std::memcmp(h, "fmt", 3) == 0 && avail >= 16) {
      if (u16(h + 8) != 1) return false;  // PCM only (WaveFile::Load)
      channels = (int16_t)u16(h + 10);
      bits = (int16_t)u16(h + 22);
      have_fmt = true;
    } else if (std::memcmp(h, "data", 4) == 0 && have_fmt) {
      data.insert(data.end(), bytes.begin() + body, bytes.begin() + body + avail);
    }
    at = body + size + (size & 1);
  }
  if (!have_fmt || (bits != 8 && bits != 16 && bits != 24) || channels <= 0 || data.empty())
    return false;
  const int bps = bits >> 3;
  const size_t frames = data.size() / (size_t)bps / (size_t)channels;
  const float max_sample = (float)(2 << (bits - 2));
  out->resize(frames);
  const uint8_t* p = data.data();
  for (size_t i = 0; i < frames; ++i) {
    float v = 0.0f;
    for (int c = 0; c < channels; ++c) {
      float s = 0.0f;
      if (bps == 1) {
        s = (float)p[0] - 128.0f;
      } else if (bps == 2) {
        s = (float)(int16_t)u16(p);
      } else {
        const int32_t x = p[0] | (p[1] << 8) | (p[2] << 16) | ((p[2] & 0x80) ? (int32_t)0xff000000 : 0);
        s = (float)x;
      }
      p += bps;
      v += s / max_sample;
    }
    (*out)[i] = v / (float)channels;
  }
  return !out->empty();
}

bool write(const std::string& fn, const std::vector<const float*>& ch, const std::vector<int>& len,
           bool norm, float norm_max) {
  const int channels = (int)ch.size();
  int length = 0;
  for (int l : len) length = std::max(length, l);
  float max = 1.0f;
  if (norm) {
    if (channels == 1) {
      if (norm_max < 0) {
        max = -1e9f;
        for (int i = 0; i < len[0]; ++i) max = std::max(max, std::fabs(ch[0][i]));
        max /= 0.8f;
      } else {
        max = norm_max / 0.95f;
      }
    } else {
      max = -1e9f;
      for (int c = 0; c < channels; ++c)
        for (int i = 0; i < len[(size_t)c]; ++i) max = std::max(max, ch[(size_t)c][i]);
      max /= 0.8f;
    }
  }
  std::vector<int16_t> pcm((size_t)length * channels, 0);
  for (int i = 0; i < length; ++i)
    for (int c = 0; c < channels; ++c)
      if (i < len[(size_t)c]) pcm[(size_t)i * channels + c] = (int16_t)(ch[(size_t)c][i] / max * 32768.0f);
  std::FILE* f = std::fopen(fn.c_str(), "wb");
  if (!f) return false;
  const uint32_t data_bytes = (uint32_t)(pcm.size() * 2);
  std::fwrite("RIFF", 1, 4, f);
  put32(f, data_bytes + 36);
  std::fwrite("WAVEfmt ", 1, 8, f);
  put32(f, 16);
  put16(f, 1);
  put16(f, (uint16_t)channels);
  put32(f, 44100);
  put32(f, 44100u * 2u * (uint32_t)channels);
  put16(f, (uint16_t)(2 * channels));
  put16(f, 16);
  std::fwrite("data", 1, 4, f);
  put32(f, data_bytes);
  for (int16_t v : pcm) put16(f, (uint16_t)v);
  const bool ok = std::ferror(f) == 0;
  std::fclose(f);
  return ok;
}

}  // namespace wav
