// vismap_geom.h -- the geometry of the listener visibility maps, shared by
// the map build (vismap.cu), the visibility test of the trace kernels
// (trace_impl.cuh) and a host-side check of the lists' conservativeness
// (tests/vismap_geom_check.cu).  Host and device evaluate the same IEEE
// operations (no contraction in the build, correctly rounded division and
// square root on both), so a cell the host finds is the cell the device
// finds.
//
// A recorder's map is a cube map around its location: face f = 2 * major
// axis + (major component < 0) of a direction d, cell (iu, iv) =
// vis_cell(minor / |major|) of its two minor components (x before y before
// z).  The lists are conservative: the tree traversal already relies on
// every point where the triangle test can report a hit lying inside the
// triangle's box padded by box_pad, and the maps pad by P = 2 box_pad,
// which also covers the rounding of the segment's direction.  (For a
// segment grazing a triangle's plane the test's rounding can report a
// crossing farther out; neither the tree nor the maps are sure to
// reproduce such an artefact.)
#pragma once

#include <math.h>

#include "ear_internal.h"

#if defined(__CUDACC__)
#define EAR_VIS_HD __host__ __device__ __forceinline__
#else
#define EAR_VIS_HD inline
#endif

namespace ear {

struct VisFaceRect {
  int u0, u1, v0, v1;
};

// Range of the ratio y / a over a box's points with major coordinate a in
// (xa, a1] (xa = max(a0, 0)) and minor coordinate y in [y0, y1]: from
// y0 / a1 (y0 >= 0) or y0 / xa (y0 < 0) to y1 / a1 (y1 <= 0) or y1 / xa
// (y1 > 0), unbounded where xa = 0; widened by a relative 2e-6 against
// the rounding of the divisions and clipped to the face, [-1, 1].
EAR_VIS_HD void vis_ratio_range(float y0, float y1, float xa, float a1, float& lo, float& hi) {
  lo = y0 >= 0.0f ? y0 / a1 : (xa > 0.0f ? y0 / xa : -INFINITY);
  hi = y1 <= 0.0f ? y1 / a1 : (xa > 0.0f ? y1 / xa : INFINITY);
  lo -= 2e-6f + 2e-6f * fabsf(lo);
  hi += 2e-6f + 2e-6f * fabsf(hi);
  lo = fmaxf(lo, -1.0f);
  hi = fminf(hi, 1.0f);
}

// Cells of face f met by the box [lo, hi] (coordinates relative to the
// recorder); false when it meets none.
EAR_VIS_HD bool vis_face_rect(const float* lo, const float* hi, int f, int res, VisFaceRect& r) {
  const int m = f >> 1;
  const bool neg = f & 1;
  const float a0 = neg ? -hi[m] : lo[m];
  const float a1 = neg ? -lo[m] : hi[m];
  if (!(a1 > 0.0f)) return false;
  const float xa = fmaxf(a0, 0.0f);
  const int p = m == 0 ? 1 : 0;
  const int q = m == 2 ? 1 : 2;
  float ulo, uhi, vlo, vhi;
  vis_ratio_range(lo[p], hi[p], xa, a1, ulo, uhi);
  vis_ratio_range(lo[q], hi[q], xa, a1, vlo, vhi);
  if (!(ulo <= uhi) || !(vlo <= vhi)) return false;
  r.u0 = vis_cell(ulo, res);
  r.u1 = vis_cell(uhi, res);
  r.v0 = vis_cell(vlo, res);
  r.v1 = vis_cell(vhi, res);
  return true;
}

// Box of the triangle v[9] padded by `pad`, relative to the recorder at
// `loc`, its distance from the recorder (rounded down) and the relative
// vertices t[3][3].
EAR_VIS_HD float vis_rel_box(const float* v, const float* loc, float pad, float* lo, float* hi,
                             float (*t)[3]) {
  float d2 = 0.0f;
  for (int k = 0; k < 3; ++k) {
    const float x0 = v[k], x1 = v[3 + k], x2 = v[6 + k];
    lo[k] = (fminf(fminf(x0, x1), x2) - pad) - loc[k];
    hi[k] = (fmaxf(fmaxf(x0, x1), x2) + pad) - loc[k];
    t[0][k] = x0 - loc[k];
    t[1][k] = x1 - loc[k];
    t[2][k] = x2 - loc[k];
    const float g = fmaxf(fmaxf(lo[k], -hi[k]), 0.0f);
    d2 += g * g;
  }
  return sqrtf(d2) * 0.99999f;
}

// The triangle seen from the recorder on face f: where all three vertices
// lie beyond the padding in front of the face, the directions of the
// padded triangle T + [-P, P]^3 fall inside the projected triangle
// (u_i, v_i) = (y_i, z_i) / a_i widened by du = P (1 + max |u_i|) /
// (min a_i - P) (and dv alike): u(t + d) - u(t) = (d_y - u(t) d_a) /
// (t_a + d_a).  P carries a tenth more for the rounding of the relative
// vertices, the widths 1e-5 more for the divisions.
struct VisTriProj {
  float u[3], v[3];
  float du, dv;
  float umin, umax, vmin, vmax;
  float eps;  // bound on the rounding of u_i, v_i (relative 1e-6 of the largest)
};

EAR_VIS_HD bool vis_tri_proj(const float (*t)[3], int f, float pad, VisTriProj& tp) {
  const int m = f >> 1;
  const bool neg = f & 1;
  const int p = m == 0 ? 1 : 0;
  const int q = m == 2 ? 1 : 2;
  const float P = pad * 1.1f;
  float amin = INFINITY, mu = 0.0f, mv = 0.0f;
  float ai[3];
  for (int i = 0; i < 3; ++i) {
    ai[i] = neg ? -t[i][m] : t[i][m];
    amin = fminf(amin, ai[i]);
  }
  if (!(amin > 2.0f * P)) return false;
  tp.umin = tp.vmin = INFINITY;
  tp.umax = tp.vmax = -INFINITY;
  for (int i = 0; i < 3; ++i) {
    tp.u[i] = t[i][p] / ai[i];
    tp.v[i] = t[i][q] / ai[i];
    mu = fmaxf(mu, fabsf(tp.u[i]));
    mv = fmaxf(mv, fabsf(tp.v[i]));
    tp.umin = fminf(tp.umin, tp.u[i]);
    tp.umax = fmaxf(tp.umax, tp.u[i]);
    tp.vmin = fminf(tp.vmin, tp.v[i]);
    tp.vmax = fmaxf(tp.vmax, tp.v[i]);
  }
  const float den = amin - P;
  tp.du = P * (1.0f + mu) / den * 1.0001f + 1e-5f;
  tp.dv = P * (1.0f + mv) / den * 1.0001f + 1e-5f;
  tp.eps = 1e-6f * (1.0f + fmaxf(mu, mv));
  return true;
}

// Does cell (iu, iv) meet the widened projected triangle?  Separating axes:
// the cell's own (the triangle's bounding box) and the three edge normals.
// An edge function n . (c - P_i) moves by at most 2 eps (|c - P_i| + |P_j -
// P_i|) when the vertices move by eps, so a corner separates only beyond
// that (plus the products' rounding); an edge whose orientation the same
// bound leaves open (a sliver seen edge-on) never separates.
EAR_VIS_HD bool vis_cell_meets(const VisTriProj& tp, int iu, int iv, int res) {
  const float w = 2.0f / (float)res;
  const float x0 = (-1.0f + (float)iu * w) - tp.du, x1 = (-1.0f + (float)(iu + 1) * w) + tp.du;
  const float y0 = (-1.0f + (float)iv * w) - tp.dv, y1 = (-1.0f + (float)(iv + 1) * w) + tp.dv;
  if (x1 < tp.umin || x0 > tp.umax || y1 < tp.vmin || y0 > tp.vmax) return false;
  for (int e = 0; e < 3; ++e) {
    const int i = e, j = e == 2 ? 0 : e + 1, k = e == 0 ? 2 : e - 1;
    float nx = -(tp.v[j] - tp.v[i]), ny = tp.u[j] - tp.u[i];
    const float len = fabsf(nx) + fabsf(ny);
    const float dk = fabsf(tp.u[k] - tp.u[i]) + fabsf(tp.v[k] - tp.v[i]);
    const float side = nx * (tp.u[k] - tp.u[i]) + ny * (tp.v[k] - tp.v[i]);
    if (!(fabsf(side) > 2.0f * tp.eps * (dk + len) + 1e-6f * len * dk)) continue;
    if (side < 0.0f) {
      nx = -nx;
      ny = -ny;
    }
    const float cu = nx > 0.0f ? x1 : x0, cv = ny > 0.0f ? y1 : y0;
    const float reach = nx * (cu - tp.u[i]) + ny * (cv - tp.v[i]);
    const float dc = fabsf(cu - tp.u[i]) + fabsf(cv - tp.v[i]);
    if (reach < -(2.0f * tp.eps * (dc + len) + 1e-6f * len * dc)) return false;
  }
  return true;
}

// Cell of the direction q = -sdir (from the recorder to the vertex):
// face, iu, iv.  False for a zero or non-finite direction.
EAR_VIS_HD bool vis_query_cell(float sx, float sy, float sz, int res, int& f, int& iu, int& iv) {
  const float qx = -sx, qy = -sy, qz = -sz;
  const float ax = fabsf(qx), ay = fabsf(qy), az = fabsf(qz);
  float m, u, v;
  if (ax >= ay && ax >= az) {
    f = qx > 0.0f ? 0 : 1;
    m = ax;
    u = qy;
    v = qz;
  } else if (ay >= az) {
    f = qy > 0.0f ? 2 : 3;
    m = ay;
    u = qx;
    v = qz;
  } else {
    f = qz > 0.0f ? 4 : 5;
    m = az;
    u = qx;
    v = qy;
  }
  if (!(m > 0.0f)) return false;
#ifdef __CUDA_ARCH__
  // correctly rounded even where a unit is compiled with approximate division
  iu = vis_cell(__fdiv_rn(u, m), res);
  iv = vis_cell(__fdiv_rn(v, m), res);
#else
  iu = vis_cell(u / m, res);
  iv = vis_cell(v / m, res);
#endif
  return true;
}

// A visibility test stops at the first entry farther than this: a hit
// point of the segment lies nearer than its length (t > 1e-5).
EAR_VIS_HD float vis_cut(float len) { return len * 1.000244140625f; }

}  // namespace ear
