// ref_render.cpp -- C entry points that run the reference's own
// Scene::Render (src/Scene.cpp:111-318) on a .EAR scene, for the tests that
// pin the oracle to the reference.
//
// TEST INFRASTRUCTURE ONLY.  oracle/build_ref.py compiles this file with
// the reference's src/ files where they lie, against the GMTL / Boost
// interface shim in oracle/refshim/, into oracle/_ref/ (never committed).
// Nothing in the product loads it.
//
// The scene is read by the reference's own parsers (Datatype, Settings,
// Material, Mesh, Triangle, MonoRecorder, StereoRecorder, SoundFile), in
// the block loop of src/EAR.cpp:92-119, and one band of one context is
// rendered as SceneContext does it (src/SceneContext.h:36-48: blank
// recorder copies, Scene::Render on them).  gmtl::Math::unitRandom
// replays a tape of uniforms that the oracle recorded for the same rays
// (oracle_random_tape), so the reference consumes the counter-based draws
// in its own call order; pow / powf go to the portable power function
// (oracle/refshim/prelude.h).
//
// ref_calc_t60 runs the `EAR calc T60` branch of src/EAR.cpp's Render
// (lines 55-284) on the same parsed scene: the mid band of the first source
// at samples / 10 rays, Recorder::Power(0.335), the global track maximum,
// Recorder::Truncate(getLength(max / 256)), RecorderTrack::T60 of recorder
// 0 track 0, and the Sabine / Norris-Eyring formulas on meshes[0].  That
// branch lives inside EAR.cpp's main program (Boost threads, FFTW, the
// command line), so its few statements are restated here in order, calling
// the reference's own Recorder / RecorderTrack / Mesh member functions for
// everything they compute.
#include <stdint.h>
#include <cmath>
#include <cstring>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

#include "Datatype.h"
#include "Material.h"
#include "Mesh.h"
#include "MonoRecorder.h"
#include "Recorder.h"
#include "Scene.h"
#include "Settings.h"
#include "SoundFile.h"
#include "StereoRecorder.h"

extern "C" float oracle_powf(float x, float y);
extern "C" float ear_ref_powf(float x, float y) { return oracle_powf(x, y); }

namespace {
const float* g_tape = 0;
int64_t g_tape_len = 0;
int64_t g_tape_pos = 0;
bool g_tape_overrun = false;
std::string g_error;
}  // namespace

namespace gmtl {
namespace Math {
float unitRandom() {
  if (g_tape_pos >= g_tape_len) {
    g_tape_overrun = true;
    ++g_tape_pos;
    return 0.5f;
  }
  return g_tape[g_tape_pos++];
}
}  // namespace Math
}  // namespace gmtl

extern "C" {

const char* ref_last_error(void) { return g_error.c_str(); }

// Renders band `band` (0..2) of source 0, static configuration, with
// `num_samples` rays, on the .EAR file at `path`.  The recorders' tracks
// (in file order; a stereo recorder gives left then right) are copied into
// tracks[track][0 .. window-1], with each track's first_sample and
// real_length.  *tape_used receives the number of uniforms consumed (more
// than tape_len when the tape ran out).  Returns the number of tracks, or
// -1 with ref_last_error() set.
int ref_render_band(const char* path, int band, int num_samples, const float* tape,
                    int64_t tape_len, int64_t* tape_used, int window, int max_tracks,
                    float* tracks, int32_t* first_sample, int32_t* real_length) {
  g_error.clear();
  std::streambuf* saved = std::cout.rdbuf();
  std::ostringstream sink;
  std::cout.rdbuf(sink.rdbuf());  // the parsers and the progress bar print
  int ntracks = -1;
  try {
    if (!Datatype::SetInput(path)) throw DatatypeException("cannot read the scene file");
    Datatype* settings = Datatype::Scan("SET ");
    if (!settings) throw DatatypeException("no settings block");
    Settings::init(settings);
    delete settings;
    const gmtl::Vec3f absorption = Settings::GetVec("absorption");
    const float dry = Settings::GetFloat("drylevel");
    Scene* scene = new Scene();
    while (Datatype::input_length) {
      const std::string peak = Datatype::PeakId();
      if (peak == "OUT1")
        scene->addListener(new MonoRecorder());
      else if (peak == "OUT2")
        scene->addListener(new StereoRecorder());
      else if (peak == "SSRC")
        scene->addSoundSource(new SoundFile());
      else if (peak == "MESH")
        scene->addMesh(new Mesh());
      else if (peak == "MAT ")
        scene->addMaterial(new Material());
      else
        delete Datatype::Read();  // SET, VRSN, FREQ: not needed to render
    }
    if (scene->sources.empty() || scene->listeners.empty() || scene->meshes.empty())
      throw DatatypeException("the scene needs a source, a recorder and a mesh");
    std::vector<Recorder*> recs;
    for (size_t i = 0; i < scene->listeners.size(); ++i)
      recs.push_back(scene->listeners[i]->getBlankCopy(4));
    g_tape = tape;
    g_tape_len = tape_len;
    g_tape_pos = 0;
    g_tape_overrun = false;
    scene->Render(band, 0, 1.0f - absorption[band], num_samples, dry, recs, -1);
    *tape_used = g_tape_pos;
    ntracks = 0;
    for (size_t ri = 0; ri < recs.size(); ++ri)
      for (size_t ti = 0; ti < recs[ri]->tracks.size(); ++ti) {
        const RecorderTrack* t = recs[ri]->tracks[ti];
        if (ntracks < max_tracks) {
          const RecorderTrack& ct = *t;
          for (int i = 0; i < window; ++i) tracks[(size_t)ntracks * window + i] = ct[(unsigned)i];
          first_sample[ntracks] = (int32_t)t->first_sample;
          real_length[ntracks] = (int32_t)t->real_length;
        }
        ++ntracks;
      }
  } catch (const std::exception& e) {
    g_error = e.what();
    ntracks = -1;
  }
  Datatype::Dispose();
  std::cout.rdbuf(saved);
  return ntracks;
}

// The `EAR calc T60` branch of src/EAR.cpp (see the file comment).
// out[0..2] = T60_ear, T60_sabine, T60_eyring; *num_rays receives the ray
// count the branch used (Settings "samples" / 10, src/EAR.cpp:80-84).
// Returns 0, or -1 with ref_last_error() set.
int ref_calc_t60(const char* path, const float* tape, int64_t tape_len, int64_t* tape_used,
                 int32_t* num_rays, float* out) {
  g_error.clear();
  std::streambuf* saved = std::cout.rdbuf();
  std::ostringstream sink;
  std::cout.rdbuf(sink.rdbuf());
  int rc = -1;
  try {
    if (!Datatype::SetInput(path)) throw DatatypeException("cannot read the scene file");
    Datatype* settings = Datatype::Scan("SET ");
    if (!settings) throw DatatypeException("no settings block");
    Settings::init(settings);
    delete settings;
    const gmtl::Vec3f absorption = Settings::GetVec("absorption");
    const float dry_level = Settings::GetFloat("drylevel");
    const int num_samples = Settings::GetInt("samples") / 10;  // src/EAR.cpp:83
    Scene* scene = new Scene();
    while (Datatype::input_length) {
      const std::string peak = Datatype::PeakId();
      if (peak == "OUT1")
        scene->addListener(new MonoRecorder());
      else if (peak == "OUT2")
        scene->addListener(new StereoRecorder());
      else if (peak == "SSRC")
        scene->addSoundSource(new SoundFile());
      else if (peak == "MESH")
        scene->addMesh(new Mesh());
      else if (peak == "MAT ")
        scene->addMaterial(new Material());
      else
        delete Datatype::Read();
    }
    if (scene->sources.empty() || scene->listeners.empty() || scene->meshes.empty())
      throw DatatypeException("the scene needs a source, a recorder and a mesh");
    // src/EAR.cpp:171-190: one context, band 1, sound 0, static
    const int band_id = 1;
    const float absorption_factor = 1.0f - absorption[band_id];
    std::vector<Recorder*> recs;
    for (size_t i = 0; i < scene->listeners.size(); ++i)
      recs.push_back(scene->listeners[i]->getBlankCopy(4));
    g_tape = tape;
    g_tape_len = tape_len;
    g_tape_pos = 0;
    g_tape_overrun = false;
    scene->Render(band_id, 0, absorption_factor, num_samples, dry_level, recs, -1);
    *tape_used = g_tape_pos;
    *num_rays = num_samples;
    // src/EAR.cpp:209-228
    float max = 0.0f;
    for (size_t ri = 0; ri < recs.size(); ++ri) {
      Recorder* r1 = recs[ri];
      r1->Power(0.335f);
      for (int i = 0; i < r1->trackCount(); ++i) {
        const float m = r1->tracks[i]->Maximum();
        if (m > max) max = m;
      }
    }
    const float treshold = max / 256.0f;
    for (size_t ri = 0; ri < recs.size(); ++ri) recs[ri]->Truncate(recs[ri]->getLength(treshold));
    // src/EAR.cpp:259-284
    out[0] = recs[0]->tracks[0]->T60();
    const Mesh* mesh = scene->meshes[0];
    const float V = mesh->Volume();
    const float A = mesh->TotalAbsorption();
    const float S = mesh->Area();
    const float a = mesh->AverageAbsorption();
    const float m = absorption[1];
    out[1] = 0.1611f * V / (A + 4.0f * m * V);
    out[2] = 0.1611f * V / (-S * log(1.0f - a) + 4.0f * m * V);
    rc = 0;
  } catch (const std::exception& e) {
    g_error = e.what();
    rc = -1;
  }
  Datatype::Dispose();
  std::cout.rdbuf(saved);
  return rc;
}

}  // extern "C"
