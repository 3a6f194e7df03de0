// Runs the CPU restatement under AddressSanitizer and UndefinedBehavior-
// Sanitizer (tests/test_oracle_sanitized.py compiles this file, which
// includes the oracle's single source, with -fsanitize=address,undefined).
// The reference has real data races and no sanitizer runs; the checker
// every GPU result is compared with gets one here.
//
// Cases: a 12-triangle shoebox with a refracting and a specular material,
// a mono and a stereo recorder, two threads, a window shorter than the
// responses (contributions past it are dropped); the per-bounce debug
// record; the adjoint; an area emitter; empty and single-triangle scenes;
// the random tape of the reference pin.  Exit status 0 when every call
// succeeded and produced energy.
#include "../oracle/ear_oracle.cpp"

#include <cstdlib>

namespace {

void quad(std::vector<float>& v, const float* a, const float* b, const float* c, const float* d) {
  const float* t[6] = {a, b, c, a, c, d};
  for (const float* p : t) v.insert(v.end(), p, p + 3);
}

int fail(const char* what) {
  std::fprintf(stderr, "FAILED: %s\n", what);
  return 1;
}

}  // namespace

int main() {
  // 10 x 7 x 4 m box, two triangles per wall
  const float L = 10.f, W = 7.f, H = 4.f;
  const float p[8][3] = {{0, 0, 0}, {L, 0, 0}, {L, W, 0}, {0, W, 0},
                         {0, 0, H}, {L, 0, H}, {L, W, H}, {0, W, H}};
  std::vector<float> v;
  quad(v, p[0], p[1], p[2], p[3]);
  quad(v, p[4], p[7], p[6], p[5]);
  quad(v, p[0], p[4], p[5], p[1]);
  quad(v, p[3], p[2], p[6], p[7]);
  quad(v, p[0], p[3], p[7], p[4]);
  quad(v, p[1], p[5], p[6], p[2]);
  const int64_t nt = (int64_t)v.size() / 9;
  std::vector<int32_t> mids((size_t)nt);
  for (int64_t i = 0; i < nt; ++i) mids[(size_t)i] = (int32_t)(i % 2);
  ear_material mats[2] = {};
  for (int b = 0; b < 3; ++b) {
    mats[0].reflection[b] = 0.8f - 0.1f * (float)b;
    mats[0].refraction[b] = 0.05f;
    mats[1].reflection[b] = 0.9f;
    mats[1].specularity[b] = 0.7f;
  }
  mats[0].has_refraction = 1;
  mats[1].has_specularity = 1;
  ear_scene_desc desc = {};
  desc.num_triangles = nt;
  desc.vertices = v.data();
  desc.material_ids = mids.data();
  desc.num_materials = 2;
  desc.materials = mats;

  ear_source src = {};
  src.location[0] = 2.f;
  src.location[1] = 3.5f;
  src.location[2] = 1.5f;
  src.gain = 0.8f;
  ear_recorder recs[2] = {};
  recs[0].channels = 1;
  recs[0].location[0] = 7.f;
  recs[0].location[1] = 3.5f;
  recs[0].location[2] = 1.5f;
  recs[1].channels = 2;
  recs[1].location[0] = 5.f;
  recs[1].location[1] = 2.f;
  recs[1].location[2] = 1.2f;
  recs[1].right_ear[0] = 5.f;
  recs[1].right_ear[1] = 1.f;
  recs[1].right_ear[2] = 1.2f;
  recs[1].head_size = 0.18f;
  recs[1].head_absorption[0] = 0.1f;
  recs[1].head_absorption[1] = 0.3f;
  recs[1].head_absorption[2] = 0.9f;

  ear_render_params prm = {};
  prm.seed = 7;
  prm.context = 3;
  prm.bands_mask = 7;
  prm.num_rays = 300;
  prm.max_bounces = 60;
  prm.num_bins = 8820;  // 0.2 s: later contributions fall past the window
  prm.cutoff = 1e-6;
  prm.air_absorption[0] = 0.01f;
  prm.air_absorption[1] = 0.02f;
  prm.air_absorption[2] = 0.05f;
  prm.dry_level = 1.f;
  const int tracks = 3;
  const size_t n = (size_t)tracks * 3 * (size_t)prm.num_bins;
  std::vector<double> h64(n);
  std::vector<float> h32(n);
  std::vector<int32_t> first((size_t)tracks * 3), last((size_t)tracks * 3);
  uint64_t cnt[5] = {};
  oracle_output out = {};
  out.hist64 = h64.data();
  out.hist32 = h32.data();
  out.first_sample = first.data();
  out.last_sample = last.data();
  out.counters = cnt;
  if (oracle_render(&desc, &src, recs, 2, &prm, 2, 0, &out) != 0) return fail("render");
  double e = 0.0;
  for (double x : h64) e += x * x;
  if (!(e > 0.0) || cnt[1] == 0 || cnt[3] == 0) return fail("render produced no energy");

  // per-bounce debug record of band 1
  const int dr = 40, dm = 20;
  std::vector<int32_t> hit((size_t)dr * dm);
  std::vector<uint8_t> bt((size_t)dr * dm);
  std::vector<uint32_t> vis((size_t)dr * dm);
  oracle_output dbg = out;
  dbg.debug_band = 1;
  dbg.debug_max_record = dm;
  dbg.debug_rays = dr;
  dbg.hit_tri = hit.data();
  dbg.bounce_type = bt.data();
  dbg.visible = vis.data();
  ear_render_params p1 = prm;
  p1.bands_mask = 2;
  p1.num_rays = dr;
  if (oracle_render(&desc, &src, recs, 2, &p1, 1, 0, &dbg) != 0) return fail("debug render");

  // adjoint of sum(g * h) with a seeded upstream gradient
  std::vector<double> g(n), grad(2 * 3 * 2);
  uint64_t s = 12345;
  for (double& x : g) {
    s = s * 6364136223846793005ull + 1442695040888963407ull;
    x = (double)(s >> 11) * (1.0 / 9007199254740992.0) - 0.5;
  }
  if (oracle_render_adjoint(&desc, &src, recs, 2, &prm, 2, 0, g.data(), grad.data()) != 0)
    return fail("adjoint");

  // area emitter: the floor's two triangles
  ear_source area = src;
  area.num_emitter_triangles = 2;
  area.emitter_vertices = v.data();
  if (oracle_render(&desc, &area, recs, 2, &prm, 2, 0, &out) != 0) return fail("area emitter");

  // empty and single-triangle scenes (the direct sound only, or one wall)
  for (int64_t k : {(int64_t)0, (int64_t)1}) {
    ear_scene_desc d2 = desc;
    d2.num_triangles = k;
    if (oracle_render(&d2, &src, recs, 2, &prm, 1, 0, &out) != 0) return fail("small scene");
  }

  // the random tape the reference pin replays
  std::vector<float> tape(1 << 16);
  int64_t used = 0;
  ear_render_params p0 = prm;
  p0.bands_mask = 1;
  p0.num_rays = 60;
  if (oracle_random_tape(&desc, &src, recs, 2, &p0, tape.data(), (int64_t)tape.size(), &used) != 0 ||
      used <= 0)
    return fail("random tape");
  std::printf("ok energy %.6g segments %llu tape %lld\n", e, (unsigned long long)cnt[1],
              (long long)used);
  return 0;
}
