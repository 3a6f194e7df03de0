// ear_cli.cpp -- the `EAR` command line on the GB300 core.
//
//   EAR render <file.EAR> [options]     src/EAR.cpp:402-411
//   EAR calc T60 <file.EAR> [options]   src/EAR.cpp:412-423
//   EAR test                            src/EAR.cpp:424-426 (returns 0)
//   EAR info <file.EAR> [--resave OUT]  parse only: print a summary (no GPU)
//
//   EAR wav2raw <in.wav> <out.f32>       WAV -> float samples, as the sources are read
//   EAR raw2wav <out.wav> <norm> <max> <ch0.f32> [<ch1.f32>]   float -> WAV
//
// options: --seed N (default: time(0), as src/EAR.cpp:58), --exact
// (kernels bit-identical to the CPU restatement), --seconds S (impulse
// response window, default 8), --device N, --out DIR (where `render` also
// writes the impulse responses when the file sets no debugdir), --conv
// fft|direct (the convolution of the reference built with or without
// FFTW; default fft), --split exact|chunked (the band split bit-identical
// to the reference's sequential filters, the default, or parallel over
// chunks), --dump-tracks DIR (also write the post-processed tracks the
// convolution reads, with their bookkeeping).
//
// Render() of the reference (src/EAR.cpp:55-393) is followed step by step:
// settings, the parse loop (the sources' WAVs are read and band-split
// before rendering), one context per (source x keyframe x band) -- here one
// ear_render call renders all bands of a (source, keyframe) -- then
// Power(0.335), the global maximum, truncation at max/256, and either
// `calc T60` (RecorderTrack::T60 with the Sabine and Norris-Eyring
// predictions) or the auralisation: every context's section of the dry
// sound convolved with every recorder track, summed per recorder,
// normalised and written to the recorder's OUT file.
#include <sys/stat.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <ctime>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "ear_gb300.h"
#include "earfile.h"
#include "wavefile.h"

namespace {

struct Options {
  unsigned long long seed = (unsigned long long)time(nullptr);
  bool exact = false;
  bool conv_direct = false;  // --conv direct: the reference built without FFTW
  bool split_chunked = false;  // --split chunked: parallel band split
  std::string dump;          // --dump-tracks DIR
  double seconds = 8.0;
  int device = 0;
  std::string out;
};

struct CliError {
  std::string msg;
};

const earfile::Value& setting(const earfile::Scene& sc, const std::string& key) {
  auto it = sc.settings.find(key);
  if (it == sc.settings.end()) throw CliError{"Setting '" + key + "' not found"};
  return it->second;
}

earfile::Vec3 at(const std::vector<earfile::Vec3>& v, int kf) {
  if (v.empty()) return earfile::Vec3();
  return (kf >= 0 && v.size() > 1) ? v[(size_t)kf] : v[0];
}

// The three band signals of one source: SoundFile::Band (the equalizer
// split of one WAV) or TripleBandSoundFile::Band (three WAVs), both with
// offset 0 (src/SoundFile.cpp:149-163).
struct DryBands {
  std::vector<float> band[3];
};

// A sound file name as the reference opens it (relative to the working
// directory), else relative to the folder of the .EAR file.
std::string resolve(const std::string& fn, const std::string& ear_path) {
  if (FILE* f = std::fopen(fn.c_str(), "rb")) {
    std::fclose(f);
    return fn;
  }
  const size_t slash = ear_path.find_last_of('/');
  if (slash != std::string::npos && !fn.empty() && fn[0] != '/') {
    const std::string alt = ear_path.substr(0, slash + 1) + fn;
    if (FILE* f = std::fopen(alt.c_str(), "rb")) {
      std::fclose(f);
      return alt;
    }
  }
  return fn;
}

// WAV data of every source, split on the GPU (SoundFile::SoundFile and
// TripleBandSoundFile::TripleBandSoundFile read the WAVs while parsing,
// src/SoundFile.cpp:33-42, 84-92; a missing file is an error).
std::vector<DryBands> load_sources(const earfile::Scene& sc, const std::string& ear_path,
                                   const Options& opt) {
  const float* fr = sc.freq;  // FREQ block or SoundFile::f1..f3 defaults
  std::vector<DryBands> out(sc.sources.size());
  for (size_t s = 0; s < sc.sources.size(); ++s) {
    const earfile::Source& src = sc.sources[s];
    if (src.triple) {
      for (int b = 0; b < 3; ++b) {
        const std::string fn = b < (int)src.files.size() ? src.files[(size_t)b] : std::string();
        if (!wav::read_float(resolve(fn, ear_path), &out[s].band[b]))
          throw CliError{"Failed to open sound file " + fn};
      }
    } else {
      const std::string fn = src.files.empty() ? std::string() : src.files[0];
      std::vector<float> x;
      if (!wav::read_float(resolve(fn, ear_path), &x)) throw CliError{"Failed to open sound file " + fn};
      for (int b = 0; b < 3; ++b) out[s].band[b].resize(x.size());
      if (ear_band_split(x.data(), (int64_t)x.size(), fr, out[s].band[0].data(),
                         out[s].band[1].data(), out[s].band[2].data(),
                         opt.split_chunked ? EAR_SPLIT_CHUNKED : 0u, nullptr, opt.device) != EAR_OK)
        throw CliError{ear_last_error()};
    }
  }
  return out;
}

// SoundFile::Section(float start, float length) of a band with offset 0
// (src/SoundFile.cpp:164-173): first sample, sample count, offset.
void section(size_t sample_length, float start, float length, int64_t* s0, int64_t* n,
             int64_t* off) {
  const unsigned int_start = (unsigned)(int)(start * 44100.0f);
  const unsigned int_length = length < 0 ? (unsigned)sample_length - int_start
                                          : (unsigned)(int)(length * 44100.0f);
  if (int_start >= sample_length) {
    *s0 = *n = *off = 0;
    return;
  }
  *s0 = int_start;
  *n = std::min<int64_t>(int_length, (int64_t)sample_length - int_start);
  *off = int_start;
}

// One rendered (source, keyframe) context: [track][band][bins] + bookkeeping.
struct Context {
  int source = 0, keyframe = -1;
  uint32_t bands = 0;
  std::vector<float> hist;
  std::vector<int32_t> first, last;
};

std::string outdir_debug(const earfile::Scene& sc) {
  const auto dd = sc.settings.find("debugdir");
  return dd != sc.settings.end() ? dd->second.s : std::string();
}

// src/EAR.cpp:292-386: every (source x keyframe x band) context convolves
// its band section with each recorder's tracks (RecorderContext ->
// Recorder::Process), keyframe pairs with the next keyframe's response;
// each recorder then sums its contexts (Recorder::Add), normalises to 0.8
// (Recorder::Normalize) and saves to its OUT file without further
// normalisation (Recorder::Save()).  Convolutions run on the GPU.
void auralise(const earfile::Scene& sc, const std::vector<Context>& contexts, int num_bins, const std::vector<DryBands>& dry, const std::string& debugdir,
              const Options& opt) {
  std::cout << std::endl << "Processing data..." << std::endl;
  const int mode = opt.conv_direct ? EAR_CONV_DIRECT : EAR_CONV_FFT;
  const int nkeys = (int)sc.keys.size();
  // the RecorderContext list in its order: (context, band) with the section
  struct Item {
    int ctx, band, next;  // next: context of the next keyframe, or -1
    int64_t s0, n, off;
  };
  std::vector<Item> items;
  for (size_t c = 0; c < contexts.size(); ++c) {
    const Context& cx = contexts[c];
    for (int b = 0; b < 3; ++b) {
      Item it;
      it.ctx = (int)c;
      it.band = b;
      it.next = -1;
      const size_t len = dry[(size_t)cx.source].band[b].size();
      if (nkeys) {
        const float offset = sc.keys[(size_t)cx.keyframe];
        if (cx.keyframe == nkeys - 1) {
          section(len, offset, -1.0f, &it.s0, &it.n, &it.off);
        } else {
          const float length = sc.keys[(size_t)cx.keyframe + 1] - offset;
          section(len, offset, length, &it.s0, &it.n, &it.off);
          it.next = (int)c + 1;  // src/EAR.cpp:311 (*(it+3): the same band one keyframe on)
        }
      } else {
        section(len, 0.0f, -1.0f, &it.s0, &it.n, &it.off);
      }
      items.push_back(it);
    }
  }
  auto ctx_of = [&](const Item& it, int t) {
    const Context& cx = contexts[(size_t)it.ctx];
    const int i = t * 3 + it.band;
    ear_conv_context e = {};
    e.ir = cx.hist.data() + (size_t)i * num_bins;
    e.ir_capacity = num_bins;
    e.ir_first = cx.first[(size_t)i];
    e.ir_length = cx.last[(size_t)i];
    if (it.next >= 0) {
      const Context& nx = contexts[(size_t)it.next];
      e.ir_next = nx.hist.data() + (size_t)i * num_bins;
      e.ir_next_capacity = num_bins;
      e.ir_next_first = nx.first[(size_t)i];
      e.ir_next_length = nx.last[(size_t)i];
    }
    const std::vector<float>& band = dry[(size_t)cx.source].band[it.band];
    e.dry = it.n > 0 ? band.data() + it.s0 : nullptr;
    e.dry_length = it.n;
    e.offset = it.off;
    return e;
  };
  double gpu_ms = 0;
  int64_t conv_calls = 0;
  // per-context processed recorders (debugdir, src/EAR.cpp:362-372):
  // Recorder::Save(fn) with the base class defaults, i.e. normalised
  if (!debugdir.empty()) {
    int t0 = 0;
    for (size_t ri = 0; ri < sc.recorders.size(); ++ri) {
      const int ch = sc.recorders[ri].channels;
      for (const Item& it : items) {
        std::vector<std::vector<float>> out((size_t)ch);
        std::vector<const float*> ptr;
        std::vector<int> len;
        for (int k = 0; k < ch; ++k) {
          ear_conv_context e = ctx_of(it, t0 + k);
          const int64_t cap = ear_conv_processed_capacity(&e, mode);
          out[(size_t)k].assign((size_t)cap, 0.0f);
          ear_conv_stats st = {};
          if (ear_convolve(&e, 1, mode, out[(size_t)k].data(), cap, 0, nullptr, opt.device, &st) != EAR_OK)
            throw CliError{ear_last_error()};
          gpu_ms += st.kernel_ms;
          ++conv_calls;
          ptr.push_back(out[(size_t)k].data());
          len.push_back((int)ear_conv_processed_length(&e, mode));
        }
        const Context& cx = contexts[(size_t)it.ctx];
        std::ostringstream ss;
        ss << debugdir << "/rec-" << ri << ".sound-" << cx.source;
        if (cx.keyframe != -1) ss << ".frame-" << std::setw(2) << std::setfill('0') << cx.keyframe;
        ss << ".band-" << it.band << ".wav";
        if (!wav::write(ss.str(), ptr, len, true, -1.0f)) throw CliError{"cannot write " + ss.str()};
      }
      t0 += ch;
    }
  }
  std::cout << "Merging result..." << std::endl;
  // every track of every recorder in one call: context lists per track
  int num_tracks = 0;
  for (const auto& r : sc.recorders) num_tracks += r.channels;
  std::vector<ear_conv_context> cs;
  std::vector<int32_t> track_of;
  std::vector<int64_t> cap((size_t)num_tracks, 0);
  for (int t = 0; t < num_tracks; ++t)
    for (const Item& it : items) {
      cs.push_back(ctx_of(it, t));
      track_of.push_back(t);
      cap[(size_t)t] = std::max(cap[(size_t)t], ear_conv_processed_capacity(&cs.back(), mode));
    }
  std::vector<std::vector<float>> out((size_t)num_tracks);
  std::vector<float*> ptr((size_t)num_tracks);
  for (int t = 0; t < num_tracks; ++t) {
    out[(size_t)t].assign((size_t)cap[(size_t)t], 0.0f);
    ptr[(size_t)t] = out[(size_t)t].data();
  }
  ear_conv_stats st = {};
  if (ear_convolve_tracks(cs.data(), track_of.data(), (int32_t)cs.size(), mode, ptr.data(),
                          cap.data(), num_tracks, 0, nullptr, opt.device, &st) != EAR_OK)
    throw CliError{ear_last_error()};
  gpu_ms += st.kernel_ms;
  ++conv_calls;
  int t0 = 0;
  for (size_t ri = 0; ri < sc.recorders.size(); ++ri) {
    const earfile::Recorder& rec = sc.recorders[ri];
    const int ch = rec.channels;
    // Recorder::Add reads each processed track over its capacity: the sum
    // ends at index cap - 1 (its real_length)
    std::vector<int> real((size_t)ch);
    for (int k = 0; k < ch; ++k) real[(size_t)k] = (int)(cap[(size_t)(t0 + k)] - 1);
    // Recorder::Normalize(0.8) over the processed tracks
    // (src/Recorder.cpp:443-460, FloatBuffer::Maximum / Multiply)
    float max = -1e9f;
    for (int k = 0; k < ch; ++k) {
      const std::vector<float>& o = out[(size_t)(t0 + k)];
      float x = 0.0f;
      for (int i = 0; i < real[(size_t)k]; ++i) x = std::max(x, std::fabs(o[(size_t)i]));
      max = std::max(max, x);
    }
    if (max > 0.0f) {
      const float f = 0.8f / max;
      for (int k = 0; k < ch; ++k)
        for (int i = 0; i < real[(size_t)k]; ++i) out[(size_t)(t0 + k)][(size_t)i] *= f;
    }
    std::vector<const float*> chans;
    for (int k = 0; k < ch; ++k) chans.push_back(out[(size_t)(t0 + k)].data());
    if (!wav::write(rec.filename, chans, real, false, 1.0f)) throw CliError{"cannot write " + rec.filename};
    std::cout << " " << rec.filename << ": " << ch << " channel(s), "
              << *std::max_element(real.begin(), real.end()) << " samples" << std::endl;
    t0 += ch;
  }
  std::cout << " convolution (" << (opt.conv_direct ? "direct" : "fft") << "): " << items.size()
            << " contexts, " << conv_calls << " calls, " << std::setprecision(1) << gpu_ms
            << " ms on the GPU" << std::setprecision(3) << std::endl;
}

int render_file(const std::string& path, const Options& opt, bool calc_t60, float* t60) {
  earfile::Scene sc;
  std::string err;
  if (!earfile::load(path, &sc, &err)) {
    std::cout << err << std::endl;
    return 1;
  }
  if (!sc.has_settings) {
    std::cout << "No settings block found in file" << std::endl;  // src/EAR.cpp:72
    return 1;
  }
  const earfile::Value& ab = setting(sc, "absorption");
  const float absorption[3] = {ab.v.x, ab.v.y, ab.v.z};
  const float dry_level = setting(sc, "drylevel").f;
  const int samples = setting(sc, "samples").i;
  // release builds trace samples / 10 rays (src/EAR.cpp:78-82); the
  // 'raysexact' setting (ignored by the reference) traces all of them
  const auto rx = sc.settings.find("raysexact");
  const bool exact_rays = rx != sc.settings.end() && rx->second.i > 0;
  const long long num_samples = exact_rays ? samples : samples / 10;
  std::cout << "Settings" << std::endl;
  for (const auto& kv : sc.settings) {
    std::cout << " +- " << kv.first << ": ";
    const earfile::Value& v = kv.second;
    if (v.tag == "int4") std::cout << v.i;
    else if (v.tag == "flt4") std::cout << v.f;
    else if (v.tag == "vec3") std::cout << "[" << v.v.x << ", " << v.v.y << ", " << v.v.z << "]";
    else std::cout << v.s;
    std::cout << std::endl;
  }
  for (const std::string& b : sc.unknown_blocks) std::cout << "Unknown block '" << b << "'" << std::endl;
  if (sc.sources.empty()) {
    std::cout << std::endl << "No sound sources defined" << std::endl << std::endl;
    return 1;
  }
  if (sc.recorders.empty()) {
    std::cout << std::endl << "No listeners defined" << std::endl << std::endl;
    return 1;
  }
  if (sc.meshes.empty())
    std::cout << std::endl << "Warning: no reflective geometry" << std::endl << std::endl;
  const int nkeys = (int)sc.keys.size();
  auto check_anim = [&](const std::vector<earfile::Vec3>& v) {
    if (v.size() > 1 && nkeys == 0) throw CliError{"Keyframe data not read"};
    if (v.size() > 1 && (int)v.size() != nkeys) throw CliError{"Keyframe count does not match"};
  };
  for (const auto& r : sc.recorders) {
    check_anim(r.location);
    check_anim(r.right_ear);
  }
  for (const auto& s : sc.sources) check_anim(s.location);

  // materials by name, meshes merged in file order (src/Scene.cpp:103-109)
  std::map<std::string, int> mat_index;
  std::vector<ear_material> mats;
  for (const auto& m : sc.materials) {
    ear_material e = {};
    for (int i = 0; i < 3; ++i) {
      e.reflection[i] = m.refl[i];
      e.refraction[i] = m.refr[i];
      e.specularity[i] = m.spec[i];
    }
    e.has_refraction = m.has_refr;
    e.has_specularity = m.has_spec;
    auto it = mat_index.find(m.name);
    if (it == mat_index.end()) {
      mat_index[m.name] = (int)mats.size();
      mats.push_back(e);
    } else {
      mats[(size_t)it->second] = e;  // a later MAT with the same name replaces it
    }
  }
  std::vector<float> verts;
  std::vector<int32_t> ids;
  std::vector<int64_t> blocks;
  for (const auto& m : sc.meshes) {
    auto it = mat_index.find(m.material);
    if (it == mat_index.end()) throw CliError{"Unknown material '" + m.material + "'"};
    verts.insert(verts.end(), m.tris.begin(), m.tris.end());
    ids.insert(ids.end(), m.tris.size() / 9, it->second);
    blocks.push_back((int64_t)(m.tris.size() / 9));
  }
  const auto dd0 = sc.settings.find("debugdir");
  const bool has_debugdir = dd0 != sc.settings.end();
  const bool noprocess0 = sc.settings.count("noprocessing") && sc.settings.at("noprocessing").i > 0;
  const bool process = !noprocess0 && !calc_t60;
  std::vector<DryBands> dry;
  if (process || has_debugdir) dry = load_sources(sc, path, opt);
  if (has_debugdir && !dry.empty()) {
    // equalizer output (src/EAR.cpp:122-146): WaveFile::FromFloat without
    // normalisation; calc T60 keeps the mid band of the first source
    const std::string dir = dd0->second.s;
    ::mkdir(dir.c_str(), 0755);
    const char* lomihi[] = {"low", "mid", "high"};
    for (size_t s = 0; s < dry.size(); ++s) {
      for (int b = 0; b < 3; ++b) {
        if (calc_t60 && b != 1) continue;
        const std::vector<float>& x = dry[s].band[b];
        std::ostringstream ss;
        ss << dir << "/sound-" << s << ".band-" << b << lomihi[b] << ".wav";
        if (!wav::write(ss.str(), {x.data()}, {(int)x.size()}, false, 1.0f))
          throw CliError{"cannot write " + ss.str()};
      }
      if (calc_t60) break;
    }
  }
  ear_scene_desc desc = {(int64_t)ids.size(), verts.data(), ids.data(), (int32_t)mats.size(),
                         mats.data(), opt.device};
  ear_scene* scene = nullptr;
  if (ear_scene_create(&desc, &scene) != EAR_OK || ear_scene_build_bvh(scene, nullptr) != EAR_OK)
    throw CliError{ear_last_error()};
  std::cout << "Rendering..." << std::endl;

  const int num_bins = (int)std::lround(opt.seconds * EAR_SAMPLE_RATE);
  std::vector<Context> contexts;
  std::vector<ear_recorder> recs(sc.recorders.size());
  int tracks = 0;
  for (const auto& r : sc.recorders) tracks += r.channels;
  for (int s = 0; s < (int)sc.sources.size(); ++s) {
    for (int kf = nkeys ? 0 : -1; kf < nkeys; ++kf) {
      const earfile::Source& src = sc.sources[(size_t)s];
      ear_source es = {};
      const earfile::Vec3 loc = at(src.location, kf);
      es.location[0] = loc.x;
      es.location[1] = loc.y;
      es.location[2] = loc.z;
      es.gain = src.gain;
      es.num_emitter_triangles = (int64_t)(src.emitter.size() / 9);
      es.emitter_vertices = src.emitter.empty() ? nullptr : src.emitter.data();
      for (size_t i = 0; i < sc.recorders.size(); ++i) {
        const earfile::Recorder& r = sc.recorders[i];
        ear_recorder& e = recs[i];
        e = {};
        e.channels = r.channels;
        const earfile::Vec3 p = at(r.location, kf), q = at(r.right_ear, kf);
        e.location[0] = p.x;
        e.location[1] = p.y;
        e.location[2] = p.z;
        e.right_ear[0] = q.x;
        e.right_ear[1] = q.y;
        e.right_ear[2] = q.z;
        e.head_size = r.head_size;
        e.head_absorption[0] = r.head_absorption.x;
        e.head_absorption[1] = r.head_absorption.y;
        e.head_absorption[2] = r.head_absorption.z;
      }
      Context c;
      c.source = s;
      c.keyframe = kf;
      c.bands = calc_t60 ? 2u : 7u;  // calc T60 renders the mid band only
      ear_render_params p = {};
      p.seed = opt.seed;
      p.context = ((uint32_t)s << 16) | (uint32_t)(kf + 1);
      p.bands_mask = c.bands;
      p.num_rays = (uint64_t)std::max<long long>(num_samples, 0);
      p.max_bounces = EAR_REFERENCE_MAX_BOUNCES;
      p.num_bins = num_bins;
      p.cutoff = EAR_REFERENCE_CUTOFF;
      for (int b = 0; b < 3; ++b) p.air_absorption[b] = absorption[b];
      p.dry_level = dry_level;
      p.flags = opt.exact ? EAR_FLAG_EXACT : 0u;
      c.hist.assign((size_t)tracks * 3 * (size_t)num_bins, 0.0f);
      c.first.assign((size_t)tracks * 3, 0);
      c.last.assign((size_t)tracks * 3, 0);
      ear_histograms out = {c.hist.data(), c.first.data(), c.last.data(), 0, 0};
      ear_render_stats st = {};
      if (ear_render(scene, &es, recs.data(), (int32_t)recs.size(), &p, &out, &st) != EAR_OK)
        throw CliError{ear_last_error()};
      std::cout << " source " << s << " keyframe " << kf << ": " << st.rays << " rays, "
                << st.segments << " segments, " << std::setprecision(1) << st.kernel_ms << " ms"
                << std::setprecision(3) << std::endl;
      contexts.push_back(std::move(c));
      if (calc_t60) break;  // first keyframe only (src/EAR.cpp:186)
    }
    if (calc_t60) break;  // first source only (src/EAR.cpp:190)
  }

  // src/EAR.cpp:209-228: Power(0.335), global maximum, truncate at max/256
  float max = 0.0f;
  for (Context& c : contexts)
    for (int b = 0; b < 3; ++b) {
      if (!((c.bands >> b) & 1u)) continue;
      for (int t = 0; t < tracks; ++t) {
        float* h = c.hist.data() + ((size_t)t * 3 + b) * num_bins;
        const int i = t * 3 + b;
        ear_track_power(h, c.first[(size_t)i], c.last[(size_t)i], 0.335f);
        max = std::max(max, ear_track_maximum(h, c.first[(size_t)i], c.last[(size_t)i]));
      }
    }
  const float treshold = max / 256.0f;
  for (Context& c : contexts)
    for (int b = 0; b < 3; ++b) {
      if (!((c.bands >> b) & 1u)) continue;
      int t0 = 0;
      for (const auto& r : sc.recorders) {
        // Recorder::getLength(tresh): 0 without samples, else the longest track
        int len = 0;
        bool has_samples = false;
        for (int k = 0; k < r.channels; ++k) {
          const int i = (t0 + k) * 3 + b;
          const float* h = c.hist.data() + (size_t)i * num_bins;
          has_samples |= c.last[(size_t)i] > 0 || c.first[(size_t)i] < 3 * 44100 - 1;
          len = std::max(len, ear_track_length(h, num_bins, c.first[(size_t)i], c.last[(size_t)i], treshold));
        }
        if (!has_samples) len = 0;
        for (int k = 0; k < r.channels; ++k) c.last[(size_t)((t0 + k) * 3 + b)] = std::max(len, 1);
        t0 += r.channels;
      }
    }

  if (!opt.dump.empty()) {
    // every post-processed track with its bookkeeping, as the convolution
    // reads them: context-<source>-<keyframe>.f32 = float[tracks][3][bins],
    // .txt = "tracks bins" then first and last per (track, band)
    ::mkdir(opt.dump.c_str(), 0755);
    for (const Context& c : contexts) {
      std::ostringstream ss;
      ss << opt.dump << "/context-" << c.source << "-" << c.keyframe;
      FILE* f = std::fopen((ss.str() + ".f32").c_str(), "wb");
      if (!f) throw CliError{"cannot write " + ss.str() + ".f32"};
      std::fwrite(c.hist.data(), sizeof(float), c.hist.size(), f);
      std::fclose(f);
      std::ofstream t(ss.str() + ".txt");
      t << tracks << " " << num_bins << "\n";
      for (size_t i = 0; i < c.first.size(); ++i) t << c.first[i] << " " << c.last[i] << "\n";
    }
  }
  const auto dd = sc.settings.find("debugdir");
  std::string outdir = dd != sc.settings.end() ? dd->second.s : opt.out;
  const bool noprocess = sc.settings.count("noprocessing") && sc.settings.at("noprocessing").i > 0;
  if (!outdir.empty()) {
    ::mkdir(outdir.c_str(), 0755);
    const char* lomihi[] = {"low", "mid", "high"};
    for (const Context& c : contexts)
      for (int b = 0; b < 3; ++b) {
        if (!((c.bands >> b) & 1u)) continue;
        int t0 = 0;
        for (size_t ri = 0; ri < sc.recorders.size(); ++ri) {
          const auto& r = sc.recorders[ri];
          std::ostringstream ss;
          ss << outdir << "/response-" << ri << ".sound-" << c.source;
          if (c.keyframe != -1) ss << ".frame-" << std::setw(2) << std::setfill('0') << c.keyframe;
          ss << ".band-" << b << lomihi[b];
          std::vector<const float*> ch;
          std::vector<int> len;
          for (int k = 0; k < r.channels; ++k) {
            const int i = (t0 + k) * 3 + b;
            ch.push_back(c.hist.data() + (size_t)i * num_bins);
            len.push_back(std::min(c.last[(size_t)i], num_bins));
          }
          if (!wav::write(ss.str() + ".wav", ch, len, true, max)) throw CliError{"cannot write " + ss.str() + ".wav"};
          // FloatBuffer::Write: real_length + 1 floats of track 0 (src/Recorder.cpp:120-123)
          FILE* f = std::fopen((ss.str() + ".bin").c_str(), "wb");
          if (f) {
            std::fwrite(ch[0], sizeof(float), (size_t)std::min(len[0] + 1, num_bins), f);
            std::fclose(f);
          }
          t0 += r.channels;
        }
      }
  }
  if (noprocess || calc_t60) {
    std::cout << std::endl << "Not processing data" << std::endl;
  } else {
    auralise(sc, contexts, num_bins, dry, outdir_debug(sc), opt);
  }
  int rc = 0;
  if (calc_t60) {
    const Context& c = contexts.front();
    const int i = 0 * 3 + 1;  // recorder 0, track 0, mid band
    t60[0] = ear_track_t60(c.hist.data() + (size_t)i * num_bins, c.first[(size_t)i], c.last[(size_t)i]);
    float stats[5] = {0, 0, 0, 0, 0};
    if (!blocks.empty()) {
      const auto it = mat_index.find(sc.meshes[0].material);
      if (ear_statistical_t60(verts.data(), blocks.data(), (int32_t)blocks.size(),
                              &mats[(size_t)it->second], absorption[1], stats) != EAR_OK)
        throw CliError{ear_last_error()};
    }
    t60[1] = stats[3];
    t60[2] = stats[4];
  }
  ear_scene_destroy(scene);
  return rc;
}

int info_file(const std::string& path, const std::string& resave) {
  earfile::Scene sc;
  std::string err;
  if (!earfile::load(path, &sc, &err)) {
    std::cout << "Error: " << err << std::endl;
    return 1;
  }
  size_t tris = 0;
  for (const auto& m : sc.meshes) tris += m.tris.size() / 9;
  std::cout << "{\"materials\": " << sc.materials.size() << ", \"meshes\": " << sc.meshes.size()
            << ", \"triangles\": " << tris << ", \"recorders\": " << sc.recorders.size()
            << ", \"stereo\": "
            << std::count_if(sc.recorders.begin(), sc.recorders.end(),
                             [](const earfile::Recorder& r) { return r.channels == 2; })
            << ", \"sources\": " << sc.sources.size() << ", \"keys\": " << sc.keys.size()
            << ", \"settings\": " << sc.settings.size() << ", \"unknown\": " << sc.unknown_blocks.size()
            << "}" << std::endl;
  if (!resave.empty() && !earfile::save(resave, sc, &err)) {
    std::cout << "Error: " << err << std::endl;
    return 1;
  }
  return 0;
}

}  // namespace

int main(int argc, char** argv) {
  const bool quiet = argc > 1 && std::string(argv[1]) == "info";
  if (!quiet)
    std::cout << "E.A.R ray-tracing core on GB300 (" << ear_version() << ")" << std::endl << std::endl;
  std::cout << std::setprecision(3) << std::fixed;
  Options opt;
  std::string resave;
  std::vector<std::string> pos;
  for (int i = 1; i < argc; ++i) {
    const std::string a(argv[i]);
    auto value = [&](const char* name) -> std::string {
      if (i + 1 >= argc) throw CliError{std::string("missing value for ") + name};
      return std::string(argv[++i]);
    };
    try {
      if (a == "--seed") opt.seed = std::stoull(value("--seed"));
      else if (a == "--exact") opt.exact = true;
      else if (a == "--dump-tracks") opt.dump = value("--dump-tracks");
      else if (a == "--split") {
        const std::string m = value("--split");
        if (m != "exact" && m != "chunked") throw CliError{"--split takes exact or chunked"};
        opt.split_chunked = m == "chunked";
      }
      else if (a == "--conv") {
        const std::string m = value("--conv");
        if (m != "fft" && m != "direct") throw CliError{"--conv takes fft or direct"};
        opt.conv_direct = m == "direct";
      }
      else if (a == "--seconds") opt.seconds = std::stod(value("--seconds"));
      else if (a == "--device") opt.device = std::stoi(value("--device"));
      else if (a == "--out") opt.out = value("--out");
      else if (a == "--resave") resave = value("--resave");
      else pos.push_back(a);
    } catch (const std::exception&) {
      std::cout << "Error: bad value for " << a << std::endl;
      return 1;
    } catch (const CliError& e) {
      std::cout << "Error: " << e.msg << std::endl;
      return 1;
    }
  }
  for (size_t i = 0; i < pos.size(); ++i) {
    const std::string& cmd = pos[i];
    const std::string arg1 = i + 1 < pos.size() ? pos[i + 1] : "";
    const std::string arg2 = i + 2 < pos.size() ? pos[i + 2] : "";
    if (cmd == "render" && !arg1.empty()) {
      int rc = 1;
      try {
        float t[3];
        rc = render_file(arg1, opt, false, t);
      } catch (const CliError& e) {
        std::cout << std::endl << "Error: " << e.msg << std::endl << std::endl;
      }
      return rc;
    } else if (cmd == "calc" && arg1 == "T60" && !arg2.empty()) {
      int rc = 1;
      try {
        float t[3] = {0, 0, 0};
        rc = render_file(arg2, opt, true, t);
        if (rc == 0) {
          std::cout << "T60_ear   : " << std::setprecision(9) << std::fixed << t[0] << "s" << std::endl;
          std::cout << "T60_sabine: " << std::setprecision(9) << std::fixed << t[1] << "s" << std::endl;
          std::cout << "T60_eyring: " << std::setprecision(9) << std::fixed << t[2] << "s" << std::endl;
        }
      } catch (const CliError& e) {
        std::cout << std::endl << "Error: " << e.msg << std::endl << std::endl;
      }
      return rc;
    } else if (cmd == "test") {
      return 0;
    } else if (cmd == "info" && !arg1.empty()) {
      return info_file(arg1, resave);
    } else if (cmd == "wav2raw" && !arg2.empty()) {
      std::vector<float> x;
      if (!wav::read_float(arg1, &x)) {
        std::cout << "Failed to open sound file " << arg1 << std::endl;
        return 1;
      }
      FILE* f = std::fopen(arg2.c_str(), "wb");
      if (!f) return 1;
      std::fwrite(x.data(), sizeof(float), x.size(), f);
      std::fclose(f);
      std::cout << x.size() << " samples" << std::endl;
      return 0;
    } else if (cmd == "raw2wav" && i + 4 < pos.size()) {
      std::vector<std::vector<float>> chans;
      for (size_t k = i + 4; k < pos.size() && k < i + 6; ++k) {
        std::vector<float> x;
        FILE* f = std::fopen(pos[k].c_str(), "rb");
        if (!f) return 1;
        float v;
        while (std::fread(&v, sizeof v, 1, f) == 1) x.push_back(v);
        std::fclose(f);
        chans.push_back(std::move(x));
      }
      std::vector<const float*> ptr;
      std::vector<int> len;
      for (const auto& c : chans) {
        ptr.push_back(c.data());
        len.push_back((int)c.size());
      }
      return wav::write(arg1, ptr, len, std::stoi(arg2) != 0, std::stof(pos[i + 3])) ? 0 : 1;
    }
  }
  std::cout << "Usage:" << std::endl
            << " EAR render <filename> [--seed N] [--exact] [--seconds S] [--out DIR]"
               " [--conv fft|direct] [--split exact|chunked]" << std::endl
            << " EAR calc T60 <filename> [--seed N] [--exact] [--seconds S]" << std::endl;
  return 1;
}
