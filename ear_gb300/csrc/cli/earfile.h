// earfile.h -- reader and writer of the tagged binary .EAR scene format.
//
// Format (as written by the Blender exporter,
// blender/render_EAR/__init__.py:154-196, and read by src/Datatype.cpp):
// the magic ".EAR", then items.  An item is a 4-byte tag; the scalar tags
// carry no length ("int4" + int32, "flt4" + float32, "str " + NUL-padded
// bytes to a multiple of 4 with at least one NUL, "vec3" + 3 "flt4" items,
// "tri " + 3 "vec3" items); every other tag is a block: tag, int32 byte
// length, payload items.  Top-level blocks: VRSN, MAT, SET, KEYS, FREQ,
// MESH, OUT1, OUT2, SSRC, 3SRC; nested blocks: "anim" (per-keyframe
// triplets) and "mesh" (emitter triangles).
#pragma once

#include <cstdint>
#include <map>
#include <string>
#include <vector>

namespace earfile {

struct Vec3 {
  float x = 0, y = 0, z = 0;
};

struct Material {  // MAT (src/Material.cpp:26-72)
  std::string name;
  float refl[3] = {0, 0, 0};
  bool has_refr = false;
  float refr[3] = {0, 0, 0};
  bool has_spec = false;
  float spec[3] = {0, 0, 0};
};

struct Mesh {  // MESH (src/Mesh.cpp:77-108)
  std::string material;
  std::vector<float> tris;  // 9 floats per triangle
};

struct Recorder {  // OUT1 / OUT2 (src/MonoRecorder.cpp:38-59, src/StereoRecorder.cpp:33-67)
  int channels = 1;
  std::string filename;
  float unused = 0;            // the float after the filename (35.0 from the exporter)
  std::vector<Vec3> location;  // 1 entry, or one per keyframe (anim)
  std::vector<Vec3> right_ear; // stereo
  float head_size = 0;
  Vec3 head_absorption;        // as written in the file
};

struct Source {  // SSRC / 3SRC (src/SoundFile.cpp:33-117)
  bool triple = false;
  std::vector<std::string> files;
  std::vector<Vec3> location;  // 1 entry, or one per keyframe (anim)
  std::vector<float> emitter;  // "mesh" emitter triangles, 9 floats each
  bool has_gain = false;
  float gain = 1.0f;
  bool has_offset = false;
  float offset = 0.0f;
};

struct Value {  // one SET entry (src/Settings.cpp:23-52)
  std::string tag;  // "int4", "flt4", "vec3", "str "
  int32_t i = 0;
  float f = 0;
  Vec3 v;
  std::string s;
};

struct Scene {
  std::map<std::string, Value> settings;
  std::vector<std::string> settings_order;  // keys in file order
  bool has_settings = false;
  std::vector<float> keys;  // KEYS
  bool has_freq = false;
  float freq[3] = {0.2f, 1.0f, 2.0f};  // SoundFile::f1..f3 defaults (src/SoundFile.cpp:238-240)
  std::vector<Material> materials;
  std::vector<Mesh> meshes;
  std::vector<Recorder> recorders;
  std::vector<Source> sources;
  std::vector<std::string> unknown_blocks;
};

// Returns false and sets *err on a malformed or truncated file.
bool load(const std::string& path, Scene* out, std::string* err);
bool parse(const std::vector<uint8_t>& bytes, Scene* out, std::string* err);
// Writes the exporter's encoding of `s` (used to make test scenes).
bool save(const std::string& path, const Scene& s, std::string* err);
std::vector<uint8_t> serialize(const Scene& s);

}  // namespace earfile
