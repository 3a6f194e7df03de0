// vismap.cu -- listener visibility maps: an exact accelerator for the
// visibility (any-hit) tests between path vertices and recorders.
//
// Every path vertex tests the segment to each recorder with
// Mesh::LineIntersection (src/Scene.cpp:188-190, src/Mesh.cpp:58-71).  All
// of a recorder's segments end at the same point, so they can be binned by
// direction around it: a cube map of res x res cells per face, and per cell
// the list of triangles whose padded bounding box meets the cell's cone of
// directions, sorted by the box's distance from the recorder.  A test then
// reads the cell of its direction and runs the ordinary triangle test on
// the entries nearer than the vertex, instead of descending the tree from
// its root.
//
// The lists are conservative, so the result is the tree traversal's bit
// for bit; the geometry that makes them so (cells of a padded box, of a
// projected triangle, of a query direction) is in vismap_geom.h.
//
// Compiled with --fmad=false: the count and fill passes must compute the
// same cells.

#include <cub/block/block_reduce.cuh>
#include <cub/block/block_scan.cuh>
#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>

#include <stdio.h>

#include <algorithm>

#include "ear_internal.h"
#include "vismap_geom.h"

namespace ear {
namespace {

struct VisBuildArgs {
  float loc[kMaxRecorders][3];
  int nrec;
  int res;
  float pad;
  const float4* tris;   // leaf order; .w of the first float4 = file-order index
  const float* verts;   // [n][9], file order
  int num_tris;
};

// Padded box of the triangle at leaf position `pos`, relative to recorder
// `ri`, its distance from the recorder (rounded down) and the relative
// vertices t[3][3].
__device__ __forceinline__ float rel_box(const VisBuildArgs& a, int ri, int pos, float* lo,
                                         float* hi, float (*t)[3]) {
  const int orig = __float_as_int(__ldg(&a.tris[4 * (size_t)pos].w));
  const float* src = a.verts + 9 * (size_t)orig;
  float v[9];
  for (int k = 0; k < 9; ++k) v[k] = __ldg(src + k);
  return vis_rel_box(v, a.loc[ri], a.pad, lo, hi, t);
}

// (recorder, triangle) items whose cell rectangles cover more than this
// many cells -- large triangles close to a recorder -- are counted and
// filled by a whole block each (k_vis_count_big, k_vis_fill_big), in the
// same cell order as one thread would.
constexpr uint64_t kVisBigItem = 1024;
constexpr int kVisBigBlock = 256;

__device__ __forceinline__ uint64_t rect_cells(const float* lo, const float* hi, int res) {
  uint64_t n = 0;
  for (int f = 0; f < 6; ++f) {
    VisFaceRect r;
    if (vis_face_rect(lo, hi, f, res, r)) n += (uint64_t)(r.u1 - r.u0 + 1) * (uint64_t)(r.v1 - r.v0 + 1);
  }
  return n;
}

__global__ void k_vis_count(const VisBuildArgs a, uint64_t* __restrict__ count,
                            int64_t* __restrict__ big, unsigned long long* __restrict__ num_big) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (int64_t)a.nrec * a.num_tris) return;
  const int ri = (int)(i / a.num_tris), pos = (int)(i % a.num_tris);
  float lo[3], hi[3], t[3][3];
  rel_box(a, ri, pos, lo, hi, t);
  if (rect_cells(lo, hi, a.res) > kVisBigItem) {
    big[atomicAdd(num_big, 1ull)] = i;
    count[i] = 0;  // k_vis_count_big
    return;
  }
  uint64_t n = 0;
  for (int f = 0; f < 6; ++f) {
    VisFaceRect r;
    if (!vis_face_rect(lo, hi, f, a.res, r)) continue;
    VisTriProj tp;
    if (!vis_tri_proj(t, f, a.pad, tp)) {
      n += (uint64_t)(r.u1 - r.u0 + 1) * (uint64_t)(r.v1 - r.v0 + 1);
      continue;
    }
    for (int v = r.v0; v <= r.v1; ++v)
      for (int u = r.u0; u <= r.u1; ++u) n += vis_cell_meets(tp, u, v, a.res) ? 1u : 0u;
  }
  count[i] = n;
}

__global__ void __launch_bounds__(kVisBigBlock) k_vis_count_big(const VisBuildArgs a,
                                                                const int64_t* __restrict__ big,
                                                                uint64_t* __restrict__ count) {
  using Reduce = cub::BlockReduce<unsigned long long, kVisBigBlock>;
  __shared__ typename Reduce::TempStorage tmp;
  const int64_t i = big[blockIdx.x];
  const int ri = (int)(i / a.num_tris), pos = (int)(i % a.num_tris);
  float lo[3], hi[3], t[3][3];
  rel_box(a, ri, pos, lo, hi, t);
  unsigned long long n = 0;
  for (int f = 0; f < 6; ++f) {
    VisFaceRect r;
    if (!vis_face_rect(lo, hi, f, a.res, r)) continue;
    VisTriProj tp;
    const bool tri = vis_tri_proj(t, f, a.pad, tp);
    const int64_t w = r.u1 - r.u0 + 1, area = w * (int64_t)(r.v1 - r.v0 + 1);
    for (int64_t k = threadIdx.x; k < area; k += kVisBigBlock) {
      const int u = r.u0 + (int)(k % w), v = r.v0 + (int)(k / w);
      n += (!tri || vis_cell_meets(tp, u, v, a.res)) ? 1u : 0u;
    }
  }
  const unsigned long long total = Reduce(tmp).Sum(n);
  if (threadIdx.x == 0) count[i] = total;
}

__global__ void __launch_bounds__(kVisBigBlock) k_vis_fill_big(const VisBuildArgs a,
                                                               const int64_t* __restrict__ big,
                                                               const uint64_t* __restrict__ count,
                                                               const uint64_t* __restrict__ offset,
                                                               uint64_t* __restrict__ keys,
                                                               int32_t* __restrict__ vals) {
  using Scan = cub::BlockScan<unsigned, kVisBigBlock>;
  __shared__ typename Scan::TempStorage tmp;
  const int64_t i = big[blockIdx.x];
  const int ri = (int)(i / a.num_tris), pos = (int)(i % a.num_tris);
  float lo[3], hi[3], t[3][3];
  const float dist = rel_box(a, ri, pos, lo, hi, t);
  const uint64_t cells_per_rec = 6ull * a.res * a.res;
  const uint64_t n = count[i], o = offset[i];
  const uint64_t dbits = __float_as_uint(dist);
  uint64_t w = 0;  // entries written so far (uniform over the block)
  for (int f = 0; f < 6; ++f) {
    VisFaceRect r;
    if (!vis_face_rect(lo, hi, f, a.res, r)) continue;
    VisTriProj tp;
    const bool tri = vis_tri_proj(t, f, a.pad, tp);
    const int64_t rw = r.u1 - r.u0 + 1, area = rw * (int64_t)(r.v1 - r.v0 + 1);
    for (int64_t base = 0; base < area; base += kVisBigBlock) {
      const int64_t k = base + threadIdx.x;
      const int u = r.u0 + (int)(k % rw), v = r.v0 + (int)(k / rw);
      const unsigned in = (k < area && (!tri || vis_cell_meets(tp, u, v, a.res))) ? 1u : 0u;
      unsigned at = 0, chunk = 0;
      Scan(tmp).ExclusiveSum(in, at, chunk);
      __syncthreads();  // tmp is reused by the next chunk
      if (in && w + at < n) {
        const uint64_t cell = ri * cells_per_rec + ((uint64_t)f * a.res + v) * a.res + u;
        keys[o + w + at] = (cell << 32) | dbits;
        vals[o + w + at] = pos;
      }
      w += chunk;
    }
  }
  // never reached with --fmad=false (both passes compute the same cells)
  for (uint64_t k = w + threadIdx.x; k < n; k += kVisBigBlock) {
    keys[o + k] = ((uint64_t)a.nrec * cells_per_rec) << 32;
    vals[o + k] = 0;
  }
}

__global__ void k_vis_fill(const VisBuildArgs a, const uint64_t* __restrict__ count,
                           const uint64_t* __restrict__ offset, uint64_t* __restrict__ keys,
                           int32_t* __restrict__ vals) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (int64_t)a.nrec * a.num_tris) return;
  const int ri = (int)(i / a.num_tris), pos = (int)(i % a.num_tris);
  float lo[3], hi[3], t[3][3];
  const float dist = rel_box(a, ri, pos, lo, hi, t);
  if (rect_cells(lo, hi, a.res) > kVisBigItem) return;  // k_vis_fill_big
  const uint64_t cells_per_rec = 6ull * a.res * a.res;
  const uint64_t n = count[i];
  uint64_t o = offset[i], w = 0;
  const uint64_t dbits = __float_as_uint(dist);
  for (int f = 0; f < 6; ++f) {
    VisFaceRect r;
    if (!vis_face_rect(lo, hi, f, a.res, r)) continue;
    VisTriProj tp;
    const bool tri = vis_tri_proj(t, f, a.pad, tp);
    for (int v = r.v0; v <= r.v1; ++v)
      for (int u = r.u0; u <= r.u1 && w < n; ++u) {
        if (tri && !vis_cell_meets(tp, u, v, a.res)) continue;
        const uint64_t cell = ri * cells_per_rec + ((uint64_t)f * a.res + v) * a.res + u;
        keys[o + w] = (cell << 32) | dbits;
        vals[o + w] = pos;
        ++w;
      }
  }
  // never reached with --fmad=false (both passes compute the same cells);
  // keeps every slot defined: past the last cell, dropped by the bounds
  for (; w < n; ++w) {
    keys[o + w] = ((uint64_t)a.nrec * cells_per_rec) << 32;
    vals[o + w] = 0;
  }
}

// start[c] = first entry of cell c (c = 0 .. cells): binary search.
__global__ void k_vis_start(const uint64_t* __restrict__ keys, int64_t n, uint64_t cells,
                            uint32_t* __restrict__ start) {
  const uint64_t c = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c > cells) return;
  int64_t lo = 0, hi = n;
  while (lo < hi) {
    const int64_t mid = (lo + hi) >> 1;
    if ((keys[mid] >> 32) < c)
      lo = mid + 1;
    else
      hi = mid;
  }
  start[c] = (uint32_t)lo;
}

// Entry i: the triangle at leaf position vals[i] with its test data inline
// (kVisEntryVecs float4, see VisMap) and the distance of keys[i].
__global__ void k_vis_pack(const uint64_t* __restrict__ keys, const int32_t* __restrict__ vals,
                           int64_t n, const float4* __restrict__ tris, int num_tris,
                           float4* __restrict__ entries) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int pos = vals[i];
  const int q = (unsigned)pos < (unsigned)num_tris ? pos : 0;
  const float4 A = __ldg(tris + 4 * (size_t)q), B = __ldg(tris + 4 * (size_t)q + 1),
               C = __ldg(tris + 4 * (size_t)q + 2);
  float4* E = entries + (size_t)kVisEntryVecs * (size_t)i;
  E[0] = make_float4(A.x, A.y, A.z, __uint_as_float((uint32_t)keys[i]));
  E[1] = make_float4(B.x, B.y, B.z, __int_as_float(pos));
  E[2] = make_float4(C.x, C.y, C.z, 0.0f);
}

// Cell c: (start, end, d1, d2) and its first entry with d0 (see VisMap);
// start = the binary-searched first entries, entries[] already packed.
__global__ void k_vis_cells(const uint32_t* __restrict__ start, const uint64_t* __restrict__ keys,
                            const float4* __restrict__ entries, uint64_t cells,
                            float4* __restrict__ out) {
  const uint64_t c = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= cells) return;
  const uint32_t b = start[c], e = start[c + 1];
  const float inf = __int_as_float(0x7f800000);
  const float d1 = b + 1 < e ? __uint_as_float((uint32_t)keys[b + 1]) : inf;
  const float d2 = b + 2 < e ? __uint_as_float((uint32_t)keys[b + 2]) : inf;
  float4* o = out + 4 * c;
  o[0] = make_float4(__uint_as_float(b), __uint_as_float(e), d1, d2);
  if (b < e) {
    const float4* E = entries + (size_t)kVisEntryVecs * b;
    o[1] = E[0];
    o[2] = E[1];
    o[3] = E[2];
  } else {
    o[1] = make_float4(0.0f, 0.0f, 0.0f, inf);
    o[2] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    o[3] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  }
}

int bits_for(uint64_t v) {
  int b = 0;
  while (b < 64 && (v >> b)) ++b;
  return b;
}

}  // namespace

void free_vis_map(VisMap* m) {
  cudaFree(m->cells);
  cudaFree(m->entries);
  *m = VisMap{};
}

#define VCK(x)                                                                    \
  do {                                                                            \
    cudaError_t e_ = (x);                                                         \
    if (e_ != cudaSuccess) {                                                      \
      snprintf(err, errlen, "%s: %s", #x, cudaGetErrorString(e_));                \
      rc = e_;                                                                    \
      goto done;                                                                  \
    }                                                                             \
  } while (0)

cudaError_t build_vis_map(const DeviceScene& s, const float (*locs)[3], int nrec, int res,
                          uint64_t max_entries, cudaStream_t st, VisMap* out, bool* too_large,
                          char* err, size_t errlen) {
  *too_large = false;
  *out = VisMap{};
  cudaError_t rc = cudaSuccess;
  VisBuildArgs a = {};
  uint64_t *count = nullptr, *offset = nullptr, *keys = nullptr, *keys2 = nullptr;
  uint32_t* start = nullptr;
  int32_t *vals = nullptr, *vals2 = nullptr;
  int64_t* big = nullptr;
  unsigned long long* d_num_big = nullptr;
  unsigned long long num_big = 0;
  void* tmp = nullptr;
  size_t tmp_bytes = 0, need = 0;
  uint64_t total = 0, last_count = 0;
  const int64_t items = (int64_t)nrec * s.num_tris;
  const uint64_t cells = 6ull * res * res * (uint64_t)nrec;
  constexpr int B = 256;
  if (nrec <= 0 || nrec > kMaxRecorders || res <= 0 || res > 4096 || s.num_tris <= 0 ||
      s.num_tris > kLeafStartMask || cells >= (1ull << 31)) {
    snprintf(err, errlen, "visibility map: bad sizes");
    return cudaErrorInvalidValue;
  }
  for (int r = 0; r < nrec; ++r)
    for (int k = 0; k < 3; ++k) a.loc[r][k] = locs[r][k];
  a.nrec = nrec;
  a.res = res;
  a.pad = 2.0f * s.box_pad;
  a.tris = s.tris;
  a.verts = s.vertices;
  a.num_tris = (int)s.num_tris;
  {
    VCK(cudaMalloc(&count, sizeof(uint64_t) * items));
    VCK(cudaMalloc(&offset, sizeof(uint64_t) * items));
    VCK(cudaMalloc(&big, sizeof(int64_t) * items));
    VCK(cudaMalloc(&d_num_big, sizeof(unsigned long long)));
    VCK(cudaMemsetAsync(d_num_big, 0, sizeof(unsigned long long), st));
    const unsigned g = (unsigned)((items + B - 1) / B);
    k_vis_count<<<g, B, 0, st>>>(a, count, big, d_num_big);
    VCK(cudaGetLastError());
    VCK(cudaMemcpyAsync(&num_big, d_num_big, sizeof num_big, cudaMemcpyDeviceToHost, st));
    VCK(cudaStreamSynchronize(st));
    if (num_big > 0) {
      k_vis_count_big<<<(unsigned)num_big, kVisBigBlock, 0, st>>>(a, big, count);
      VCK(cudaGetLastError());
    }
    VCK(cub::DeviceScan::ExclusiveSum(nullptr, need, count, offset, items, st));
    VCK(cudaMalloc(&tmp, need));
    tmp_bytes = need;
    VCK(cub::DeviceScan::ExclusiveSum(tmp, tmp_bytes, count, offset, items, st));
    VCK(cudaMemcpyAsync(&total, offset + items - 1, sizeof total, cudaMemcpyDeviceToHost, st));
    VCK(cudaMemcpyAsync(&last_count, count + items - 1, sizeof last_count, cudaMemcpyDeviceToHost, st));
    VCK(cudaStreamSynchronize(st));
    total += last_count;
    if (total > max_entries || total >= (1ull << 31)) {
      *too_large = true;
      snprintf(err, errlen, "visibility map: %llu entries above the limit of %llu",
               (unsigned long long)total, (unsigned long long)max_entries);
      goto done;
    }
    cudaFree(tmp);
    tmp = nullptr;
    const int64_t n = (int64_t)total;
    VCK(cudaMalloc(&keys, sizeof(uint64_t) * std::max<int64_t>(n, 1)));
    VCK(cudaMalloc(&keys2, sizeof(uint64_t) * std::max<int64_t>(n, 1)));
    VCK(cudaMalloc(&vals, sizeof(int32_t) * std::max<int64_t>(n, 1)));
    VCK(cudaMalloc(&vals2, sizeof(int32_t) * std::max<int64_t>(n, 1)));
    k_vis_fill<<<g, B, 0, st>>>(a, count, offset, keys, vals);
    VCK(cudaGetLastError());
    if (num_big > 0) {
      k_vis_fill_big<<<(unsigned)num_big, kVisBigBlock, 0, st>>>(a, big, count, offset, keys, vals);
      VCK(cudaGetLastError());
    }
    cub::DoubleBuffer<uint64_t> dk(keys, keys2);
    cub::DoubleBuffer<int32_t> dv(vals, vals2);
    const int end_bit = 32 + bits_for(cells);
    need = 0;
    VCK(cub::DeviceRadixSort::SortPairs(nullptr, need, dk, dv, (int)n, 0, end_bit, st));
    VCK(cudaMalloc(&tmp, std::max<size_t>(need, 1)));
    tmp_bytes = need;
    VCK(cub::DeviceRadixSort::SortPairs(tmp, tmp_bytes, dk, dv, (int)n, 0, end_bit, st));
    VCK(cudaMalloc(&start, sizeof(uint32_t) * (cells + 1)));
    VCK(cudaMalloc(&out->cells, kVisCellBytes * (size_t)cells));
    VCK(cudaMalloc(&out->entries, kVisEntryBytes * (size_t)std::max<int64_t>(n, 1)));
    k_vis_start<<<(unsigned)((cells + 1 + B - 1) / B), B, 0, st>>>(dk.Current(), n, cells, start);
    VCK(cudaGetLastError());
    if (n > 0) {
      k_vis_pack<<<(unsigned)((n + B - 1) / B), B, 0, st>>>(dk.Current(), dv.Current(), n, s.tris,
                                                             (int)s.num_tris, out->entries);
      VCK(cudaGetLastError());
    }
    k_vis_cells<<<(unsigned)((cells + B - 1) / B), B, 0, st>>>(start, dk.Current(), out->entries,
                                                               cells, out->cells);
    VCK(cudaGetLastError());
    VCK(cudaStreamSynchronize(st));
    out->res = res;
    out->num_recs = nrec;
    out->num_entries = (uint64_t)n;
    out->bytes = kVisCellBytes * (size_t)cells + kVisEntryBytes * (size_t)n;
  }
done:
  cudaFree(start);
  cudaFree(count);
  cudaFree(offset);
  cudaFree(big);
  cudaFree(d_num_big);
  cudaFree(keys);
  cudaFree(keys2);
  cudaFree(vals);
  cudaFree(vals2);
  cudaFree(tmp);
  if (rc != cudaSuccess || *too_large) free_vis_map(out);
  return rc;
}

}  // namespace ear
