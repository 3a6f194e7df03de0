// Host-side check that a visibility test answered from the listener
// visibility maps equals the brute-force any-hit test, on seeded random
// scenes.  Each case places a recorder among ~150 random triangles (1 cm to
// 3 m, some large ones close to the recorder), builds the cell lists the
// map build would (vismap_geom.h: box cells, projected-triangle cells,
// entry distances), and for path vertices on the triangles (and in free
// space, and beyond the edges and corners of triangles) compares
//   brute force: any triangle with 1e-5 < t < 1 (Mesh::LineIntersection,
//                src/Mesh.cpp:58-71), and
//   map walk:    the triangles listed in the query's cell whose entry
//                distance is within the walk's cut,
// with the Moller-Trumbore test in both evaluation orders the trace kernels
// use (exact kernels divide first; fast kernels compare unscaled).  The map
// may only test fewer triangles, never decide differently.  It also
// reports, over every reported hit, how far outside the triangle's
// unpadded box (in units of the tree's padding box_pad) lie the point at
// the reported t and the exact crossing of the segment's line with the
// triangle's plane (both in double), and how far that crossing's parameter
// lies outside [0, 1]: the quantities the padding argument bounds.  For
// segments grazing a triangle's plane the float test's rounding exceeds
// them.  Prints the counts; exit status 1 on any mismatch.
//
// Built by tests/test_vismap_geom.py with nvcc, host code only, no
// contraction (-ffp-contract=off).

#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>

#include <vector>

#include "../ear_gb300/csrc/vismap_geom.h"

using namespace ear;

namespace {

uint64_t g_state = 0x2545F4914F6CDD1Dull;

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

// Moller & Trumbore (1997), non-culling, in the trace kernels' two orders.
bool mt(V3 v0, V3 e1, V3 e2, V3 o, V3 d, bool fast, float& t) {
  const V3 pvec = cross(d, e2);
  const float det = dot(e1, pvec);
  if (det > -1e-6f && det < 1e-6f) return false;
  const V3 tvec = sub(o, v0);
  if (fast) {
    const float un = dot(tvec, pvec);
    const V3 qvec = cross(tvec, e1);
    const float vn = dot(d, qvec);
    if (det > 0.0f) {
      if (un < 0.0f || un > det || vn < 0.0f || un + vn > det) return false;
    } else {
      if (un > 0.0f || un < det || vn > 0.0f || un + vn < det) return false;
    }
    t = dot(e2, qvec) / det;
    return true;
  }
  const float inv_det = 1.0f / det;
  const float u = dot(tvec, pvec) * inv_det;
  if (u < 0.0f || u > 1.0f) return false;
  const V3 qvec = cross(tvec, e1);
  const float v = dot(d, qvec) * inv_det;
  if (v < 0.0f || u + v > 1.0f) return false;
  t = dot(e2, qvec) * inv_det;
  return true;
}

struct Tri {
  float v[9];
  V3 v0, e1, e2;
  float dist;
  bool has_rect[6], has_proj[6];
  VisFaceRect rect[6];
  VisTriProj proj[6];
};

bool listed(const Tri& T, int f, int iu, int iv, int res) {
  if (!T.has_rect[f]) return false;
  const VisFaceRect& r = T.rect[f];
  if (iu < r.u0 || iu > r.u1 || iv < r.v0 || iv > r.v1) return false;
  return !T.has_proj[f] || vis_cell_meets(T.proj[f], iu, iv, res);
}

}  // namespace

int main(int argc, char** argv) {
  const int cases = argc > 1 ? atoi(argv[1]) : 2000;
  g_state ^= argc > 2 ? (uint64_t)atoll(argv[2]) * 0x9E3779B97F4A7C15ull : 0ull;
  const int resolutions[3] = {16, 128, 1024};
  long queries = 0, blocked = 0, mismatches = 0, tested_brute = 0, tested_map = 0;
  double worst_outside = 0.0;  // largest (distance outside the box) / box_pad
  double worst_crossing = 0.0;  // the same for the exact crossing point
  double worst_t = -1.0;        // largest distance of its parameter outside [0, 1]
  std::vector<Tri> tris;
  for (int c = 0; c < cases; ++c) {
    const int res = resolutions[c % 3];
    const bool fast = (c / 3) % 2 == 1;
    float loc[3];
    for (int k = 0; k < 3; ++k) loc[k] = (float)uni(-10.0, 10.0);
    const int n = 150;
    tris.assign(n, Tri{});
    float maxc = 0.0f;
    for (int k = 0; k < 3; ++k) maxc = fmaxf(maxc, fabsf(loc[k]));
    for (int i = 0; i < n; ++i) {
      Tri& T = tris[i];
      const bool big = i < 6;  // large triangles close to the recorder
      const double spread = big ? 1.5 : 8.0, size = big ? 3.0 : uni(0.01, 1.0);
      double cen[3];
      for (int k = 0; k < 3; ++k) cen[k] = loc[k] + gauss() * spread;
      for (int j = 0; j < 3; ++j)
        for (int k = 0; k < 3; ++k) T.v[3 * j + k] = (float)(cen[k] + gauss() * size);
      for (int k = 0; k < 9; ++k) maxc = fmaxf(maxc, fabsf(T.v[k]));
    }
    // the tree's padding (2^-18 of the largest coordinate plus 1e-5) and
    // the maps' (twice that)
    const float box_pad = maxc * 3.814697265625e-6f + 1e-5f;
    const float pad = 2.0f * box_pad;
    for (Tri& T : tris) {
      T.v0 = mk(T.v[0], T.v[1], T.v[2]);
      T.e1 = sub(mk(T.v[3], T.v[4], T.v[5]), T.v0);
      T.e2 = sub(mk(T.v[6], T.v[7], T.v[8]), T.v0);
      float lo[3], hi[3], t[3][3];
      T.dist = vis_rel_box(T.v, loc, pad, lo, hi, t);
      for (int f = 0; f < 6; ++f) {
        T.has_rect[f] = vis_face_rect(lo, hi, f, res, T.rect[f]);
        T.has_proj[f] = T.has_rect[f] && vis_tri_proj(t, f, pad, T.proj[f]);
      }
    }
    for (int qi = 0; qi < 40; ++qi) {
      V3 p;
      if (qi % 4 == 3) {
        p = mk((float)(loc[0] + gauss() * 6.0), (float)(loc[1] + gauss() * 6.0),
               (float)(loc[2] + gauss() * 6.0));
      } else if (qi % 4 == 2) {
        // a vertex whose segment to the recorder crosses a triangle's edge
        // or corner: where rounding decides the triangle test
        const Tri& T = tris[next_u64() % n];
        const int a = (int)(next_u64() % 3), b = (a + 1) % 3;
        const double s = (next_u64() % 4 == 0) ? 0.0 : uni();
        double e[3];
        for (int k = 0; k < 3; ++k) e[k] = T.v[3 * a + k] + s * ((double)T.v[3 * b + k] - T.v[3 * a + k]);
        const double kk = uni(1.02, 3.0);
        p = mk((float)(loc[0] + (e[0] - loc[0]) * kk), (float)(loc[1] + (e[1] - loc[1]) * kk),
               (float)(loc[2] + (e[2] - loc[2]) * kk));
      } else {  // a path vertex on a triangle, as a hit point is
        const Tri& T = tris[next_u64() % n];
        double b0 = uni(), b1 = uni();
        if (b0 + b1 > 1.0) {
          b0 = 1.0 - b0;
          b1 = 1.0 - b1;
        }
        const float f0 = (float)b0, f1 = (float)b1;
        p = mk((T.v0.x + f0 * T.e1.x) + f1 * T.e2.x, (T.v0.y + f0 * T.e1.y) + f1 * T.e2.y,
               (T.v0.z + f0 * T.e1.z) + f1 * T.e2.z);
      }
      const V3 sdir = sub(mk(loc[0], loc[1], loc[2]), p);
      int f, iu, iv;
      if (!vis_query_cell(sdir.x, sdir.y, sdir.z, res, f, iu, iv)) continue;
      ++queries;
      const float cut = vis_cut(length(sdir));
      bool hit_brute = false, hit_map = false;
      for (const Tri& T : tris) {
        float t;
        ++tested_brute;
        if (mt(T.v0, T.e1, T.e2, p, sdir, fast, t) && t > 1e-5f && t < 1.0f) {
          hit_brute = true;
          const double q[3] = {p.x + (double)t * sdir.x, p.y + (double)t * sdir.y,
                               p.z + (double)t * sdir.z};
          for (int k = 0; k < 3; ++k) {
            const double lo = fmin(fmin(T.v[k], T.v[3 + k]), T.v[6 + k]);
            const double hi = fmax(fmax(T.v[k], T.v[3 + k]), T.v[6 + k]);
            const double out = fmax(fmax(lo - q[k], q[k] - hi), 0.0);
            worst_outside = fmax(worst_outside, out / box_pad);
          }
          // exact crossing of the segment's line with the triangle's plane
          const double e1[3] = {T.e1.x, T.e1.y, T.e1.z}, e2[3] = {T.e2.x, T.e2.y, T.e2.z};
          const double nrm[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2],
                                 e1[0] * e2[1] - e1[1] * e2[0]};
          const double d[3] = {sdir.x, sdir.y, sdir.z};
          const double w[3] = {(double)T.v0.x - p.x, (double)T.v0.y - p.y, (double)T.v0.z - p.z};
          const double nd = nrm[0] * d[0] + nrm[1] * d[1] + nrm[2] * d[2];
          const double te = (nrm[0] * w[0] + nrm[1] * w[1] + nrm[2] * w[2]) / nd;
          worst_t = fmax(worst_t, fmax(-te, te - 1.0));
          for (int k = 0; k < 3; ++k) {
            const double x = p.x * (k == 0) + p.y * (k == 1) + p.z * (k == 2) + te * d[k];
            const double lo = fmin(fmin(T.v[k], T.v[3 + k]), T.v[6 + k]);
            const double hi = fmax(fmax(T.v[k], T.v[3 + k]), T.v[6 + k]);
            worst_crossing = fmax(worst_crossing, fmax(fmax(lo - x, x - hi), 0.0) / box_pad);
          }
        }
        if (listed(T, f, iu, iv, res) && T.dist <= cut) {
          ++tested_map;
          if (mt(T.v0, T.e1, T.e2, p, sdir, fast, t) && t > 1e-5f && t < 1.0f) hit_map = true;
        }
      }
      blocked += hit_brute;
      if (hit_brute != hit_map) {
        if (mismatches < 5)
          printf("mismatch: case %d query %d res %d fast %d brute %d map %d\n", c, qi, res,
                 (int)fast, (int)hit_brute, (int)hit_map);
        ++mismatches;
      }
    }
  }
  printf("cases %d queries %ld blocked %ld mismatches %ld brute_tests %ld map_tests %ld "
         "worst_outside_over_pad %.6f worst_crossing_over_pad %.6f worst_t_beyond %.3g\n",
         cases, queries, blocked, mismatches, tested_brute, tested_map, worst_outside,
         worst_crossing, worst_t);
  return mismatches ? 1 : 0;
}
