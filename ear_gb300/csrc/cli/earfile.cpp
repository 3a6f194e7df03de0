// earfile.cpp -- .EAR reader and writer (format described in earfile.h).
// Reading follows src/Datatype.cpp and the block constructors it drives
// (src/EAR.cpp:92-119), with bounds checks: a truncated or malformed file
// is an error here, where the reference reads past its buffer.
#include "earfile.h"

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>

namespace earfile {
namespace {

bool is_scalar(const std::string& t) {
  return t == "int4" || t == "flt4" || t == "str " || t == "vec3" || t == "vecf" || t == "tri ";
}

class Reader {
 public:
  Reader(const uint8_t* p, size_t n) : p_(p), end_(p + n), pos_(p) {}
  const uint8_t* pos() const { return pos_; }
  void seek(const uint8_t* q) { pos_ = q; }
  bool at_end(const uint8_t* limit) const { return pos_ >= limit; }
  std::string err;

  bool peek(std::string* tag, const uint8_t* limit) const {
    if (pos_ + 4 > limit) return false;
    tag->assign(reinterpret_cast<const char*>(pos_), 4);
    return true;
  }
  bool tag(const char* want) {
    if (pos_ + 4 > end_) return fail("truncated file");
    if (std::memcmp(pos_, want, 4) != 0)
      return fail("Found '" + std::string(reinterpret_cast<const char*>(pos_), 4) + "' while expecting '" +
                  want + "'");
    pos_ += 4;
    return true;
  }
  bool i32(int32_t* v) {
    if (pos_ + 4 > end_) return fail("truncated file");
    std::memcpy(v, pos_, 4);
    pos_ += 4;
    return true;
  }
  bool f32(float* v) {
    if (pos_ + 4 > end_) return fail("truncated file");
    std::memcpy(v, pos_, 4);
    pos_ += 4;
    return true;
  }
  // ReadFloat (src/Datatype.cpp:114-120)
  bool read_float(float* v) { return tag("flt4") && f32(v); }
  bool read_int(int32_t* v) { return tag("int4") && i32(v); }
  // ReadString: NUL-terminated, padded to a multiple of 4 with >= 1 NUL
  // (src/Datatype.cpp:104-109, 137-147)
  bool read_string(std::string* s) {
    if (!tag("str ")) return false;
    const uint8_t* q = pos_;
    while (q < end_ && *q) ++q;
    if (q >= end_) return fail("unterminated string");
    const size_t n = (size_t)(q - pos_);
    s->assign(reinterpret_cast<const char*>(pos_), n);
    const size_t padded = n + 4 - (n % 4);
    if (pos_ + padded > end_) return fail("truncated string");
    pos_ += padded;
    return true;
  }
  // ReadVec / ReadTriplet: "vec3" (the exporter; ReadTriplet expects "vecf"
  // but does not enforce it, src/Datatype.h:83-90) + 3 flt4
  bool read_vec(Vec3* v) {
    if (pos_ + 4 > end_) return fail("truncated file");
    if (std::memcmp(pos_, "vec3", 4) != 0 && std::memcmp(pos_, "vecf", 4) != 0)
      return fail("Found '" + std::string(reinterpret_cast<const char*>(pos_), 4) +
                  "' while expecting 'vec3'");
    pos_ += 4;
    return read_float(&v->x) && read_float(&v->y) && read_float(&v->z);
  }
  // block header: tag + int32 length; returns the payload end
  bool block(const char* want, const uint8_t** block_end) {
    int32_t len = 0;
    if (!tag(want) || !i32(&len)) return false;
    if (len < 0 || pos_ + len > end_) return fail(std::string("block '") + want + "' overruns the file");
    *block_end = pos_ + len;
    return true;
  }
  // skips one item of any kind
  bool skip_item() {
    std::string t;
    if (!peek(&t, end_)) return fail("truncated file");
    if (t == "int4" || t == "flt4") {
      pos_ += 8;
    } else if (t == "str ") {
      std::string s;
      return read_string(&s);
    } else if (t == "vec3" || t == "vecf") {
      Vec3 v;
      return read_vec(&v);
    } else if (t == "tri ") {
      pos_ += 4;
      Vec3 v;
      return read_vec(&v) && read_vec(&v) && read_vec(&v);
    } else {
      const uint8_t* e = nullptr;
      if (!block(t.c_str(), &e)) return false;
      pos_ = e;
    }
    if (pos_ > end_) return fail("truncated file");
    return true;
  }
  bool fail(const std::string& m) {
    if (err.empty()) err = m;
    return false;
  }

 private:
  const uint8_t* p_;
  const uint8_t* end_;
  const uint8_t* pos_;
};

// Animated<T> (src/Animated.h:71-88) or a single vec3
bool read_location(Reader& r, const uint8_t* limit, std::vector<Vec3>* out) {
  std::string t;
  if (!r.peek(&t, limit)) return r.fail("truncated block");
  out->clear();
  if (t == "anim") {
    const uint8_t* e = nullptr;
    if (!r.block("anim", &e)) return false;
    while (!r.at_end(e)) {
      Vec3 v;
      if (!r.read_vec(&v)) return false;
      out->push_back(v);
    }
    return true;
  }
  Vec3 v;
  if (!r.read_vec(&v)) return false;
  out->push_back(v);
  return true;
}

bool read_triangles(Reader& r, const uint8_t* limit, std::vector<float>* tris) {
  std::string t;
  while (r.peek(&t, limit) && t == "tri ") {
    if (!r.tag("tri ")) return false;
    for (int k = 0; k < 3; ++k) {
      Vec3 v;
      if (!r.read_vec(&v)) return false;
      tris->push_back(v.x);
      tris->push_back(v.y);
      tris->push_back(v.z);
    }
  }
  return true;
}

bool read_source(Reader& r, bool triple, Source* s) {
  const uint8_t* e = nullptr;
  if (!r.block(triple ? "3SRC" : "SSRC", &e)) return false;
  s->triple = triple;
  for (int k = 0; k < (triple ? 3 : 1); ++k) {
    std::string f;
    if (!r.read_string(&f)) return false;
    s->files.push_back(f);
  }
  std::string t;
  if (!r.peek(&t, e)) return r.fail("truncated source block");
  if (t == "mesh") {
    const uint8_t* me = nullptr;
    if (!r.block("mesh", &me)) return false;
    std::string mt;
    if (r.peek(&mt, me) && mt == "str ") {
      std::string name;
      if (!r.read_string(&name)) return false;
    }
    if (!read_triangles(r, me, &s->emitter)) return false;
    r.seek(me);
  } else if (!read_location(r, e, &s->location)) {
    return false;
  }
  if (r.peek(&t, e) && t == "flt4") {
    s->has_gain = true;
    if (!r.read_float(&s->gain)) return false;
  }
  if (r.peek(&t, e) && t == "flt4") {
    s->has_offset = true;
    if (!r.read_float(&s->offset)) return false;
  }
  r.seek(e);
  return true;
}

}  // namespace

bool parse(const std::vector<uint8_t>& bytes, Scene* sc, std::string* err) {
  *sc = Scene();
  if (bytes.size() < 4 || std::memcmp(bytes.data(), ".EAR", 4) != 0) {
    *err = "Failed to read file";  // src/EAR.cpp:61-63
    return false;
  }
  Reader r(bytes.data() + 4, bytes.size() - 4);
  const uint8_t* end = bytes.data() + bytes.size();
  std::string t;
  while (r.peek(&t, end)) {
    const uint8_t* e = nullptr;
    if (t == "MAT ") {
      Material m;
      if (!r.block("MAT ", &e) || !r.read_string(&m.name)) break;
      bool ok = true;
      for (int i = 0; i < 3 && ok; ++i) ok = r.read_float(&m.refl[i]);
      if (!ok) break;
      std::string n;
      if (r.peek(&n, e) && n == "flt4") {
        m.has_refr = true;
        for (int i = 0; i < 3 && ok; ++i) ok = r.read_float(&m.refr[i]);
      }
      if (ok && r.peek(&n, e) && n == "flt4") {
        m.has_spec = true;
        for (int i = 0; i < 3 && ok; ++i) ok = r.read_float(&m.spec[i]);
      }
      if (!ok) break;
      sc->materials.push_back(m);
      r.seek(e);
    } else if (t == "SET ") {
      if (!r.block("SET ", &e)) break;
      sc->has_settings = true;
      bool ok = true;
      std::string k;
      while (ok && r.peek(&k, e) && k == "str ") {
        std::string key;
        Value v;
        ok = r.read_string(&key) && r.peek(&v.tag, e);
        if (!ok) break;
        if (v.tag == "int4") ok = r.read_int(&v.i);
        else if (v.tag == "flt4") ok = r.read_float(&v.f);
        else if (v.tag == "vec3") ok = r.read_vec(&v.v);
        else if (v.tag == "str ") ok = r.read_string(&v.s);
        else ok = r.skip_item();
        if (!sc->settings.count(key)) sc->settings_order.push_back(key);
        sc->settings[key] = v;
      }
      if (!ok) break;
      r.seek(e);
    } else if (t == "KEYS") {
      if (!r.block("KEYS", &e)) break;
      bool ok = true;
      while (ok && !r.at_end(e)) {
        float f;
        ok = r.read_float(&f);
        if (ok) sc->keys.push_back(f);
      }
      if (!ok) break;
    } else if (t == "FREQ") {
      if (!r.block("FREQ", &e)) break;
      if (!r.read_float(&sc->freq[0]) || !r.read_float(&sc->freq[1]) || !r.read_float(&sc->freq[2]))
        break;
      sc->has_freq = true;
      r.seek(e);
    } else if (t == "MESH") {
      Mesh m;
      if (!r.block("MESH", &e) || !r.read_string(&m.material) || !read_triangles(r, e, &m.tris)) break;
      sc->meshes.push_back(std::move(m));
      r.seek(e);
    } else if (t == "OUT1" || t == "OUT2") {
      Recorder rec;
      rec.channels = t == "OUT2" ? 2 : 1;
      if (!r.block(t.c_str(), &e) || !r.read_string(&rec.filename) || !r.read_float(&rec.unused) ||
          !read_location(r, e, &rec.location))
        break;
      if (rec.channels == 2) {
        if (!read_location(r, e, &rec.right_ear) || !r.read_float(&rec.head_size) ||
            !r.read_vec(&rec.head_absorption))
          break;
      }
      sc->recorders.push_back(rec);
      r.seek(e);
    } else if (t == "SSRC" || t == "3SRC") {
      Source s;
      if (!read_source(r, t == "3SRC", &s)) break;
      sc->sources.push_back(std::move(s));
    } else {
      // VRSN and unknown blocks are skipped (src/EAR.cpp:106-118); the
      // exporter's lowercase "ssrc"/"3src" mesh emitters land here too.
      if (t != "VRSN") sc->unknown_blocks.push_back(t);
      if (!r.skip_item()) break;
    }
  }
  if (!r.err.empty()) {
    *err = r.err;
    return false;
  }
  return true;
}

bool load(const std::string& path, Scene* out, std::string* err) {
  std::ifstream f(path.c_str(), std::ios::binary);
  if (!f.good()) {
    *err = "Failed to read file";
    return false;
  }
  std::vector<uint8_t> bytes((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
  return parse(bytes, out, err);
}

// ------------------------------------------------------------------ writer
namespace {

struct Writer {
  std::vector<uint8_t> b;
  void raw(const void* p, size_t n) {
    const uint8_t* c = static_cast<const uint8_t*>(p);
    b.insert(b.end(), c, c + n);
  }
  void tag(const char* t) { raw(t, 4); }
  void i32(int32_t v) { raw(&v, 4); }
  void flt(float v) {
    tag("flt4");
    raw(&v, 4);
  }
  void integer(int32_t v) {
    tag("int4");
    i32(v);
  }
  void str(const std::string& s) {  // pack(): '\0' * (4 - len % 4)
    tag("str ");
    raw(s.data(), s.size());
    const size_t pad = 4 - s.size() % 4;
    for (size_t i = 0; i < pad; ++i) b.push_back(0);
  }
  void vec(const Vec3& v) {
    tag("vec3");
    flt(v.x);
    flt(v.y);
    flt(v.z);
  }
  size_t open(const char* t) {
    tag(t);
    i32(0);
    return b.size();
  }
  void close(size_t start) {
    const int32_t len = (int32_t)(b.size() - start);
    std::memcpy(b.data() + start - 4, &len, 4);
  }
  void location(const std::vector<Vec3>& v) {
    if (v.size() == 1) {
      vec(v[0]);
      return;
    }
    const size_t s = open("anim");
    for (const Vec3& x : v) vec(x);
    close(s);
  }
};

}  // namespace

std::vector<uint8_t> serialize(const Scene& sc) {
  Writer w;
  w.tag(".EAR");
  {
    const size_t s = w.open("VRSN");
    w.integer(0);
    w.close(s);
  }
  for (const Material& m : sc.materials) {
    const size_t s = w.open("MAT ");
    w.str(m.name);
    for (float f : m.refl) w.flt(f);
    if (m.has_refr)
      for (float f : m.refr) w.flt(f);
    if (m.has_spec)
      for (float f : m.spec) w.flt(f);
    w.close(s);
  }
  if (sc.has_settings) {
    const size_t s = w.open("SET ");
    std::vector<std::string> order = sc.settings_order;
    for (const auto& kv : sc.settings)
      if (std::find(order.begin(), order.end(), kv.first) == order.end()) order.push_back(kv.first);
    for (const std::string& key : order) {
      w.str(key);
      const Value& v = sc.settings.at(key);
      if (v.tag == "int4") w.integer(v.i);
      else if (v.tag == "flt4") w.flt(v.f);
      else if (v.tag == "vec3") w.vec(v.v);
      else w.str(v.s);
    }
    w.close(s);
  }
  if (!sc.keys.empty()) {
    const size_t s = w.open("KEYS");
    for (float k : sc.keys) w.flt(k);
    w.close(s);
  }
  if (sc.has_freq) {
    const size_t s = w.open("FREQ");
    for (float f : sc.freq) w.flt(f);
    w.close(s);
  }
  for (const Mesh& m : sc.meshes) {
    const size_t s = w.open("MESH");
    w.str(m.material);
    for (size_t i = 0; i + 9 <= m.tris.size(); i += 9) {
      w.tag("tri ");
      for (int k = 0; k < 3; ++k) w.vec(Vec3{m.tris[i + 3 * k], m.tris[i + 3 * k + 1], m.tris[i + 3 * k + 2]});
    }
    w.close(s);
  }
  for (const Source& src : sc.sources) {
    const size_t s = w.open(src.triple ? "3SRC" : "SSRC");
    for (const std::string& f : src.files) w.str(f);
    if (!src.emitter.empty()) {
      const size_t ms = w.open("mesh");
      for (size_t i = 0; i + 9 <= src.emitter.size(); i += 9) {
        w.tag("tri ");
        for (int k = 0; k < 3; ++k)
          w.vec(Vec3{src.emitter[i + 3 * k], src.emitter[i + 3 * k + 1], src.emitter[i + 3 * k + 2]});
      }
      w.close(ms);
    } else {
      w.location(src.location);
    }
    if (src.has_gain) w.flt(src.gain);
    if (src.has_offset) w.flt(src.offset);
    w.close(s);
  }
  for (const Recorder& r : sc.recorders) {
    const size_t s = w.open(r.channels == 2 ? "OUT2" : "OUT1");
    w.str(r.filename);
    w.flt(r.unused);
    w.location(r.location);
    if (r.channels == 2) {
      w.location(r.right_ear);
      w.flt(r.head_size);
      w.vec(r.head_absorption);
    }
    w.close(s);
  }
  return w.b;
}

bool save(const std::string& path, const Scene& s, std::string* err) {
  const std::vector<uint8_t> b = serialize(s);
  std::ofstream f(path.c_str(), std::ios::binary);
  if (!f.good()) {
    *err = "cannot write " + path;
    return false;
  }
  f.write(reinterpret_cast<const char*>(b.data()), (std::streamsize)b.size());
  return f.good();
}

}  // namespace earfile
