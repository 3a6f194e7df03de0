// Host-side check of the listener visibility maps' conservativeness: the
// map build's and the visibility test's own geometry (vismap_geom.h),
// compiled for the host, on seeded random cases.  For each case -- a
// recorder, a triangle (sizes from 1 mm to 3 m, 1 cm to 40 m away, some
// slivers, some straddling the recorder's planes), a resolution -- it
// samples points where the triangle test could report a hit (on the
// triangle, moved by up to the tree's box padding), places a path vertex
// beyond each on the line from the recorder, and checks that the cell the
// visibility test computes from the vertex is one the build lists the
// triangle in, and that the walk's distance cut does not stop before the
// triangle's entry.  Prints the counts; exit status 1 on any miss.
//
// Built by tests/test_vismap_geom.py with nvcc, host code only, no
// contraction (-ffp-contract=off), like the device build of the maps.

#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>

#include "../ear_gb300/csrc/vismap_geom.h"

using namespace ear;

namespace {

uint64_t g_state = 0x9E3779B97F4A7C15ull;

uint64_t next_u64() {  // xorshift64*
  g_state ^= g_state >> 12;
  g_state ^= g_state << 25;
  g_state ^= g_state >> 27;
  return g_state * 0x2545F4914F6CDD1Dull;
}
double uni() { return (double)(next_u64() >> 11) * (1.0 / 9007199254740992.0); }
double uni(double a, double b) { return a + (b - a) * uni(); }
double gauss() {
  double s = 0.0;
  for (int i = 0; i < 12; ++i) s += uni();
  return s - 6.0;
}

}  // namespace

int main(int argc, char** argv) {
  const int cases = argc > 1 ? atoi(argv[1]) : 20000;
  g_state ^= argc > 2 ? (uint64_t)atoll(argv[2]) : 0ull;
  const int resolutions[6] = {8, 64, 512, 2048, 2560, 4096};
  const double sizes[5] = {0.001, 0.02, 0.05, 0.3, 3.0};
  long queries = 0, misses = 0, cut_misses = 0, with_tri = 0;
  for (int c = 0; c < cases; ++c) {
    const int res = resolutions[(c + c / 5) % 6];
    float loc[3];
    for (int k = 0; k < 3; ++k) loc[k] = (float)uni(-30.0, 30.0);
    // triangle centre: a random direction and distance from the recorder,
    // or (every fifth case) straddling the recorder's coordinate planes
    double dir[3], n2 = 0.0;
    for (int k = 0; k < 3; ++k) {
      dir[k] = gauss();
      n2 += dir[k] * dir[k];
    }
    const double dist = (c % 5 == 0) ? uni(0.0, 0.05) : uni(0.01, 40.0);
    const double size = sizes[c % 5 == 0 ? 4 : (c / 5) % 5];
    double cen[3];
    for (int k = 0; k < 3; ++k) cen[k] = loc[k] + dir[k] / sqrt(n2) * dist;
    float v[9];
    for (int i = 0; i < 3; ++i)
      for (int k = 0; k < 3; ++k) v[3 * i + k] = (float)(cen[k] + gauss() * size);
    if (c % 7 == 3)  // a sliver: the third vertex nearly on the first edge
      for (int k = 0; k < 3; ++k)
        v[6 + k] = (float)(v[k] + (v[3 + k] - v[k]) * uni() + gauss() * 1e-5);
    // the tree's padding for coordinates up to 60 (2^-18 of the largest
    // plus 1e-5) and the maps' (twice that)
    const float box_pad = 60.0f * 3.814697265625e-6f + 1e-5f;
    const float pad = 2.0f * box_pad;
    float lo[3], hi[3], t[3][3];
    const float entry_dist = vis_rel_box(v, loc, pad, lo, hi, t);
    VisFaceRect rect[6];
    VisTriProj proj[6];
    bool has_rect[6], has_proj[6];
    for (int f = 0; f < 6; ++f) {
      has_rect[f] = vis_face_rect(lo, hi, f, res, rect[f]);
      has_proj[f] = has_rect[f] && vis_tri_proj(t, f, pad, proj[f]);
    }
    for (int j = 0; j < 8; ++j) {
      // a point of the triangle, moved by up to box_pad on each axis
      double b0 = uni(), b1 = uni();
      if (b0 + b1 > 1.0) {
        b0 = 1.0 - b0;
        b1 = 1.0 - b1;
      }
      float q[3], p[3], sdir[3];
      for (int k = 0; k < 3; ++k) {
        const double x = v[k] + b0 * ((double)v[3 + k] - v[k]) + b1 * ((double)v[6 + k] - v[k]);
        q[k] = (float)(x + uni(-1.0, 1.0) * box_pad);
      }
      // the path vertex: beyond q on the line from the recorder
      const double s = uni(0.02, 1.0);
      for (int k = 0; k < 3; ++k) p[k] = (float)(loc[k] + ((double)q[k] - loc[k]) / s);
      for (int k = 0; k < 3; ++k) sdir[k] = loc[k] - p[k];
      int f, iu, iv;
      if (!vis_query_cell(sdir[0], sdir[1], sdir[2], res, f, iu, iv)) continue;
      ++queries;
      bool listed = has_rect[f] && rect[f].u0 <= iu && iu <= rect[f].u1 && rect[f].v0 <= iv &&
                    iv <= rect[f].v1;
      if (listed && has_proj[f]) {
        ++with_tri;
        listed = vis_cell_meets(proj[f], iu, iv, res);
      }
      if (!listed) {
        if (misses < 5)
          printf("miss: case %d point %d res %d face %d cell (%d, %d)\n", c, j, res, f, iu, iv);
        ++misses;
      }
      // the walk stops at the first entry farther than the cut; q lies on
      // the segment, so the triangle's entry must come before it
      const float len = sqrtf(sdir[0] * sdir[0] + sdir[1] * sdir[1] + sdir[2] * sdir[2]);
      if (entry_dist > vis_cut(len)) ++cut_misses;
    }
  }
  printf("cases %d queries %ld projected %ld misses %ld cut_misses %ld\n", cases, queries, with_tri,
         misses, cut_misses);
  return (misses || cut_misses) ? 1 : 0;
}
