// ear_cli.cpp -- the `EAR` command line on the GB300 core.
//
//   EAR render <file.EAR> [options]     src/EAR.cpp:402-411
//   EAR calc T60 <file.EAR> [options]   src/EAR.cpp:412-423
//   EAR test                            src/EAR.cpp:424-426 (returns 0)
//   EAR info <file.EAR> [--resave OUT]  parse only: print a summary (no GPU)
//
// options: --seed N (default: time(0), as src/EAR.cpp:58), --exact
// (kernels bit-identical to the CPU restatement), --seconds S (impulse
// response window, default 8), --device N, --out DIR (where `render` writes
// the impulse responses when the file sets no debugdir).
//
// Render() of the reference (src/EAR.cpp:55-393) is followed step by step:
// settings, the parse loop, one context per (source x keyframe x band) --
// here one ear_render call renders all bands of a (source, keyframe) --
// then Power(0.335), the global maximum, truncation at max/256 and, for
// `calc T60`, RecorderTrack::T60 with the Sabine and Norris-Eyring
// predictions.  The convolution with the dry sound (auralisation) is not
// part of this build: `render` writes the impulse responses instead.
#include <sys/stat.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <ctime>
#include <iomanip>
#include <iostream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "ear_gb300.h"
#include "earfile.h"

namespace {

struct Options {
  unsigned long long seed = (unsigned long long)time(nullptr);
  bool exact = false;
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

// 16-bit PCM WAV, as WaveFile::FromFloat + WaveFile::Save
// (lib/wave/WaveFile.cpp:124-154, 190-255).
void write_wav(const std::string& fn, const std::vector<const float*>& ch,
               const std::vector<int>& len, bool norm, float norm_max) {
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
        for (int i = 0; i < len[c]; ++i) max = std::max(max, ch[c][i]);
      max /= 0.8f;
    }
  }
  std::vector<int16_t> pcm((size_t)length * channels, 0);
  for (int i = 0; i < length; ++i)
    for (int c = 0; c < channels; ++c)
      if (i < len[c]) pcm[(size_t)i * channels + c] = (int16_t)(ch[c][i] / max * 32768.0f);
  FILE* f = std::fopen(fn.c_str(), "wb");
  if (!f) throw CliError{"cannot write " + fn};
  const uint32_t data_bytes = (uint32_t)(pcm.size() * 2);
  const uint32_t riff = data_bytes + 36, fmt_size = 16, rate = 44100;
  const uint32_t byte_rate = rate * 2 * (uint32_t)channels;
  const uint16_t format = 1, nch = (uint16_t)channels, align = (uint16_t)(2 * channels), bits = 16;
  std::fwrite("RIFF", 1, 4, f);
  std::fwrite(&riff, 4, 1, f);
  std::fwrite("WAVEfmt ", 1, 8, f);
  std::fwrite(&fmt_size, 4, 1, f);
  std::fwrite(&format, 2, 1, f);
  std::fwrite(&nch, 2, 1, f);
  std::fwrite(&rate, 4, 1, f);
  std::fwrite(&byte_rate, 4, 1, f);
  std::fwrite(&align, 2, 1, f);
  std::fwrite(&bits, 2, 1, f);
  std::fwrite("data", 1, 4, f);
  std::fwrite(&data_bytes, 4, 1, f);
  std::fwrite(pcm.data(), 2, pcm.size(), f);
  std::fclose(f);
}

// One rendered (source, keyframe) context: [track][band][bins] + bookkeeping.
struct Context {
  int source = 0, keyframe = -1;
  uint32_t bands = 0;
  std::vector<float> hist;
  std::vector<int32_t> first, last;
};

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

  const auto dd = sc.settings.find("debugdir");
  std::string outdir = dd != sc.settings.end() ? dd->second.s : opt.out;
  const bool noprocess = sc.settings.count("noprocessing") && sc.settings.at("noprocessing").i > 0;
  if (!calc_t60 && outdir.empty()) outdir = path + ".responses";
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
          write_wav(ss.str() + ".wav", ch, len, true, max);
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
    std::cout << std::endl
              << "Auralisation (convolution with the dry sound) is not part of this build; "
                 "impulse responses written to "
              << outdir << std::endl;
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
    }
  }
  std::cout << "Usage:" << std::endl
            << " EAR render <filename> [--seed N] [--exact] [--seconds S] [--out DIR]" << std::endl
            << " EAR calc T60 <filename> [--seed N] [--exact] [--seconds S]" << std::endl;
  return 1;
}
