// bvh_build.cu -- linear BVH built on the device.
//
// The reference has no acceleration structure (src/Scene.h:37-41): every
// query loops over all triangles (src/Mesh.cpp:33-71).  This file builds a
// binary LBVH (Karras, "Maximizing parallelism in the construction of BVHs,
// octrees, and k-d trees", HPG 2012): 30-bit Morton codes of the box
// centres, a device radix sort, one thread per internal node to find its
// range and split, and a bottom-up refit with one atomic visit counter per
// node.  Compiled with --fmad=false: the per-triangle edges and normals it
// writes must equal the CPU restatement's bit for bit.
//
// The alternative builder is PLOC (Meister and Bittner, "Parallel Locally-
// Ordered Clustering for Bounding Volume Hierarchy Construction", IEEE TVCG
// 2018): starting from the same Morton-sorted leaves, every cluster finds
// the cluster within `radius` positions whose union box has the smallest
// surface area; mutual nearest neighbours merge into a new node; the
// survivors are compacted in order and the step repeats until one cluster
// is left.  Nearest neighbours are ranked by (area, lower index, higher
// index), a strict order in which the globally closest pair is always
// mutual, so every step merges at least one pair.  Internal nodes are
// numbered backwards in creation order, so the root is node 0.

#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>

#include <stdio.h>

#include <utility>

#include "ear_internal.h"

namespace ear {
namespace {

// float <-> order-preserving uint for atomicMin/atomicMax on floats
__device__ __forceinline__ uint32_t ord(float f) {
  const uint32_t u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__host__ __device__ __forceinline__ float unord(uint32_t u) {
#ifdef __CUDA_ARCH__
  return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
#else
  return u2f((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
#endif
}

// bounds[0..2] = min centre, [3..5] = max centre, [6] = max |coordinate|
__global__ void k_tri_boxes(const float* __restrict__ v, int64_t n, float4* __restrict__ lo,
                            float4* __restrict__ hi, uint32_t* __restrict__ bounds) {
  __shared__ uint32_t sb[7];
  if (threadIdx.x < 7) sb[threadIdx.x] = (threadIdx.x < 3) ? 0xffffffffu : 0u;
  __syncthreads();
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    const float* p = v + 9 * i;
    float l[3], h[3];
    float mabs = 0.0f;
    for (int a = 0; a < 3; ++a) {
      const float x = p[a], y = p[3 + a], z = p[6 + a];
      l[a] = fminf(fminf(x, y), z);
      h[a] = fmaxf(fmaxf(x, y), z);
      mabs = fmaxf(mabs, fmaxf(fabsf(l[a]), fabsf(h[a])));
    }
    lo[i] = make_float4(l[0], l[1], l[2], 0.0f);
    hi[i] = make_float4(h[0], h[1], h[2], 0.0f);
    for (int a = 0; a < 3; ++a) {
      const float c = 0.5f * l[a] + 0.5f * h[a];
      atomicMin(&sb[a], ord(c));
      atomicMax(&sb[3 + a], ord(c));
    }
    atomicMax(&sb[6], ord(mabs));
  }
  __syncthreads();
  if (threadIdx.x < 3) atomicMin(&bounds[threadIdx.x], sb[threadIdx.x]);
  else if (threadIdx.x < 7) atomicMax(&bounds[threadIdx.x], sb[threadIdx.x]);
}

__device__ __forceinline__ uint32_t spread10(uint32_t x) {
  x &= 0x3ffu;
  x = (x | (x << 16)) & 0x030000FFu;
  x = (x | (x << 8)) & 0x0300F00Fu;
  x = (x | (x << 4)) & 0x030C30C3u;
  x = (x | (x << 2)) & 0x09249249u;
  return x;
}

__global__ void k_morton(const float4* __restrict__ lo, const float4* __restrict__ hi, int64_t n,
                         const uint32_t* __restrict__ bounds, uint32_t* __restrict__ codes,
                         int32_t* __restrict__ idx) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 l = lo[i], h = hi[i];
  const float c[3] = {0.5f * l.x + 0.5f * h.x, 0.5f * l.y + 0.5f * h.y, 0.5f * l.z + 0.5f * h.z};
  uint32_t code = 0;
  for (int a = 0; a < 3; ++a) {
    const float mn = unord(bounds[a]), mx = unord(bounds[3 + a]);
    const float ext = mx - mn;
    float f = ext > 0.0f ? (c[a] - mn) / ext : 0.5f;
    f = fminf(fmaxf(f * 1024.0f, 0.0f), 1023.0f);
    code |= spread10((uint32_t)f) << (2 - a);
  }
  codes[i] = code;
  idx[i] = (int32_t)i;
}

// Common-prefix length of the augmented keys (code, index).
__device__ __forceinline__ int delta(const uint32_t* __restrict__ codes, int n, int i, int j) {
  if (j < 0 || j >= n) return -1;
  const uint32_t a = codes[i], b = codes[j];
  if (a == b) return 32 + __clz((uint32_t)i ^ (uint32_t)j);
  return __clz(a ^ b);
}

// One thread per internal node (Karras 2012, Fig. 4).
__global__ void k_karras(const uint32_t* __restrict__ codes, int n, Node* __restrict__ nodes,
                         int32_t* __restrict__ leaf_parent, int2* __restrict__ range) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n - 1) return;
  const int d = (delta(codes, n, i, i + 1) - delta(codes, n, i, i - 1)) >= 0 ? 1 : -1;
  const int dmin = delta(codes, n, i, i - d);
  int lmax = 2;
  while (delta(codes, n, i, i + lmax * d) > dmin) lmax <<= 1;
  int l = 0;
  for (int t = lmax >> 1; t >= 1; t >>= 1)
    if (delta(codes, n, i, i + (l + t) * d) > dmin) l += t;
  const int j = i + l * d;
  const int dnode = delta(codes, n, i, j);
  int s = 0, t = l;
  do {
    t = (t + 1) >> 1;
    if (delta(codes, n, i, i + (s + t) * d) > dnode) s += t;
  } while (t > 1);
  const int gamma = i + s * d + (d < 0 ? d : 0);
  const int first = i < j ? i : j, last = i < j ? j : i;
  range[i] = make_int2(first, last);
  int c0, c1;
  if (first == gamma) {
    c0 = ~gamma;
    leaf_parent[gamma] = i;
  } else {
    c0 = gamma;
    nodes[gamma].d.z = i;
  }
  if (last == gamma + 1) {
    c1 = ~(gamma + 1);
    leaf_parent[gamma + 1] = i;
  } else {
    c1 = gamma + 1;
    nodes[gamma + 1].d.z = i;
  }
  nodes[i].d.x = c0;
  nodes[i].d.y = c1;
  if (i == 0) nodes[0].d.z = -1;
}

// Bottom-up refit: the second thread to reach a node merges its children.
__global__ void k_refit(const float4* __restrict__ lo, const float4* __restrict__ hi,
                        const int32_t* __restrict__ sorted_idx, const int32_t* __restrict__ leaf_parent,
                        int n, float pad, Node* nodes, float4* node_lo, float4* node_hi,
                        uint32_t* visits) {
  const int leaf = blockIdx.x * blockDim.x + threadIdx.x;
  if (leaf >= n) return;
  int p = leaf_parent[leaf];
  while (p >= 0) {
    __threadfence();
    if (atomicAdd(&visits[p], 1u) == 0u) return;
    __threadfence();
    const int4 ch = __ldcg(&nodes[p].d);
    float4 bl[2], bh[2];
    const int c[2] = {ch.x, ch.y};
    for (int k = 0; k < 2; ++k) {
      if (c[k] < 0) {
        const int t = sorted_idx[~c[k] & kLeafStartMask];
        const float4 l = lo[t], h = hi[t];
        bl[k] = make_float4(l.x - pad, l.y - pad, l.z - pad, 0.0f);
        bh[k] = make_float4(h.x + pad, h.y + pad, h.z + pad, 0.0f);
      } else {
        bl[k] = __ldcg(&node_lo[c[k]]);
        bh[k] = __ldcg(&node_hi[c[k]]);
      }
    }
    Node& nd = nodes[p];
    nd.a = make_float4(bl[0].x, bh[0].x, bl[0].y, bh[0].y);
    nd.b = make_float4(bl[0].z, bh[0].z, bl[1].x, bh[1].x);
    nd.c = make_float4(bl[1].y, bh[1].y, bl[1].z, bh[1].z);
    node_lo[p] = make_float4(fminf(bl[0].x, bl[1].x), fminf(bl[0].y, bl[1].y),
                             fminf(bl[0].z, bl[1].z), 0.0f);
    node_hi[p] = make_float4(fmaxf(bh[0].x, bh[1].x), fmaxf(bh[0].y, bh[1].y),
                             fmaxf(bh[0].z, bh[1].z), 0.0f);
    p = __ldcg(&nodes[p].d.z);
  }
}

// ------------------------------------------------------------------ PLOC
__device__ __forceinline__ float union_area(float4 al, float4 ah, float4 bl, float4 bh) {
  const float dx = fmaxf(ah.x, bh.x) - fminf(al.x, bl.x);
  const float dy = fmaxf(ah.y, bh.y) - fminf(al.y, bl.y);
  const float dz = fmaxf(ah.z, bh.z) - fminf(al.z, bl.z);
  return 2.0f * (dx * dy + dy * dz + dz * dx);
}

// Nearest neighbour of every cluster within +-radius positions; ties go
// to the lowest index, which is the (area, min, max) order for a fixed i.
__global__ void k_ploc_nn(const float4* __restrict__ lo, const float4* __restrict__ hi, int count,
                          int radius, int* __restrict__ nn) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  const float4 il = lo[i], ih = hi[i];
  const int j0 = i - radius < 0 ? 0 : i - radius;
  const int j1 = i + radius > count - 1 ? count - 1 : i + radius;
  float best = 0.0f;
  int bj = -1;
  for (int j = j0; j <= j1; ++j) {
    if (j == i) continue;
    const float a = union_area(il, ih, lo[j], hi[j]);
    if (bj < 0 || a < best) {
      best = a;
      bj = j;
    }
  }
  nn[i] = bj;
}

__global__ void k_ploc_flags(const int* __restrict__ nn, int count, int* __restrict__ merge,
                             int* __restrict__ keep) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  const int j = nn[i];
  const bool mutual = j >= 0 && nn[j] == i;
  merge[i] = (mutual && i < j) ? 1 : 0;
  keep[i] = (mutual && i > j) ? 0 : 1;
}

__global__ void k_ploc_totals(const int* __restrict__ merge, const int* __restrict__ mrank,
                              const int* __restrict__ keep, const int* __restrict__ kpos, int count,
                              int2* __restrict__ totals) {
  totals[0] = make_int2(mrank[count - 1] + merge[count - 1], kpos[count - 1] + keep[count - 1]);
}

// Writes the merged nodes and the compacted cluster list of one step.
__global__ void k_ploc_write(const float4* __restrict__ lo, const float4* __restrict__ hi,
                             const int* __restrict__ id, const int* __restrict__ nn,
                             const int* __restrict__ merge, const int* __restrict__ mrank,
                             const int* __restrict__ keep, const int* __restrict__ kpos, int count,
                             int node_base, float4* __restrict__ lo2, float4* __restrict__ hi2,
                             int* __restrict__ id2, Node* __restrict__ nodes,
                             int* __restrict__ leaf_parent) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count || !keep[i]) return;
  const int p = kpos[i];
  if (!merge[i]) {
    lo2[p] = lo[i];
    hi2[p] = hi[i];
    id2[p] = id[i];
    return;
  }
  const int j = nn[i];
  const int idx = node_base - mrank[i];
  const float4 l0 = lo[i], h0 = hi[i], l1 = lo[j], h1 = hi[j];
  Node nd;
  nd.a = make_float4(l0.x, h0.x, l0.y, h0.y);
  nd.b = make_float4(l0.z, h0.z, l1.x, h1.x);
  nd.c = make_float4(l1.y, h1.y, l1.z, h1.z);
  nd.d = make_int4(id[i], id[j], -1, 0);
  nodes[idx] = nd;
  const int c[2] = {id[i], id[j]};
  for (int k = 0; k < 2; ++k) {
    if (c[k] >= 0) {
      nodes[c[k]].d.z = idx;
    } else {
      leaf_parent[~c[k] & kLeafStartMask] = idx;
    }
  }
  lo2[p] = make_float4(fminf(l0.x, l1.x), fminf(l0.y, l1.y), fminf(l0.z, l1.z), 0.0f);
  hi2[p] = make_float4(fmaxf(h0.x, h1.x), fmaxf(h0.y, h1.y), fmaxf(h0.z, h1.z), 0.0f);
  id2[p] = idx;
}

// Initial clusters: the padded leaf boxes in sorted order, leaf code ~k.
__global__ void k_ploc_init(const float4* __restrict__ lo, const float4* __restrict__ hi,
                            const int32_t* __restrict__ sorted_idx, int n, float pad,
                            float4* __restrict__ clo, float4* __restrict__ chi,
                            int* __restrict__ cid) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const int t = sorted_idx[k];
  const float4 l = lo[t], h = hi[t];
  clo[k] = make_float4(l.x - pad, l.y - pad, l.z - pad, 0.0f);
  chi[k] = make_float4(h.x + pad, h.y + pad, h.z + pad, 0.0f);
  cid[k] = ~k;
}

// Leaf collapse: an internal child whose subtree spans at most max_leaf
// triangles (a contiguous range of the sorted order) becomes one leaf over
// that range.  Its box in the parent is already the union of the subtree.
// The nodes below it stay in memory but are no longer reachable.
__global__ void k_collapse(const int2* __restrict__ range, int n, int max_leaf, Node* nodes) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n - 1) return;
  int4 d = nodes[i].d;
  int c[2] = {d.x, d.y};
  for (int k = 0; k < 2; ++k) {
    if (c[k] < 0) continue;
    const int2 r = range[c[k]];
    const int cnt = r.y - r.x + 1;
    if (cnt <= max_leaf) c[k] = ~(r.x | ((cnt - 1) << kLeafCountShift));
  }
  d.x = c[0];
  d.y = c[1];
  nodes[i].d = d;
}

// ---------------------------------------------------- depth-first layout
// Internal nodes are renumbered in depth-first preorder (a node, its child
// 0 subtree, its child 1 subtree), so a node's first child is the next
// 64 bytes and every subtree is one contiguous range: traversal steps that
// descend touch neighbouring cache lines.  Subtree sizes (internal nodes)
// come bottom-up with one atomic visit counter per node, as in the refit;
// each node then finds its position by walking up to the root.
__global__ void k_subtree_size(const int32_t* __restrict__ leaf_parent, int n, const Node* nodes,
                               uint32_t* visits, int* size) {
  const int leaf = blockIdx.x * blockDim.x + threadIdx.x;
  if (leaf >= n) return;
  int p = leaf_parent[leaf];
  while (p >= 0) {
    __threadfence();
    if (atomicAdd(&visits[p], 1u) == 0u) return;
    __threadfence();
    const int4 ch = __ldcg(&nodes[p].d);
    const int s0 = ch.x >= 0 ? __ldcg(&size[ch.x]) : 0;
    const int s1 = ch.y >= 0 ? __ldcg(&size[ch.y]) : 0;
    size[p] = 1 + s0 + s1;
    p = ch.z;
  }
}

__global__ void k_preorder(const Node* __restrict__ nodes, const int* __restrict__ size, int nn,
                           int* __restrict__ pos) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= nn) return;
  int p = 0, cur = v;
  for (int guard = 0; guard < 4096; ++guard) {
    const int par = nodes[cur].d.z;
    if (par < 0) break;
    const int4 pc = nodes[par].d;
    p += (pc.x == cur) ? 1 : 1 + (pc.x >= 0 ? size[pc.x] : 0);
    cur = par;
  }
  pos[v] = p;
}

__global__ void k_permute(const Node* __restrict__ nodes, const int* __restrict__ pos, int nn,
                          Node* __restrict__ out) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= nn) return;
  const int pv = pos[v];
  if ((unsigned)pv >= (unsigned)nn) return;  // cannot happen for a valid tree
  Node nd = nodes[v];
  if (nd.d.x >= 0) nd.d.x = pos[nd.d.x];
  if (nd.d.y >= 0) nd.d.y = pos[nd.d.y];
  if (nd.d.z >= 0) nd.d.z = pos[nd.d.z];
  out[pv] = nd;
}

// ------------------------------------------------------------- 4-wide
// 4-wide nodes, built top-down from the binary tree one frontier (level) at
// a time.  A 4-wide node starts from its binary node's two children and
// repeatedly opens the internal child with the largest surface area until
// it has four children (or only leaves are left) -- the usual greedy
// collapse, which fills the slots that grouping fixed pairs of levels
// leaves empty near the leaves.  The internal children of a level's nodes
// are numbered consecutively through a prefix sum (deterministic), so a
// node's internal children are neighbours in memory; the root is node 0.
struct Slot4 {
  float lo[3], hi[3];
  int ref;  // >= 0 binary internal node, < 0 leaf code
};

__device__ __forceinline__ Slot4 slot_of(const Node& P, int c) {
  Slot4 s;
  s.lo[0] = c ? P.b.z : P.a.x;
  s.hi[0] = c ? P.b.w : P.a.y;
  s.lo[1] = c ? P.c.x : P.a.z;
  s.hi[1] = c ? P.c.y : P.a.w;
  s.lo[2] = c ? P.c.z : P.b.x;
  s.hi[2] = c ? P.c.w : P.b.y;
  s.ref = c ? P.d.y : P.d.x;
  return s;
}

__device__ __forceinline__ float slot_area(const Slot4& s) {
  const float dx = s.hi[0] - s.lo[0], dy = s.hi[1] - s.lo[1], dz = s.hi[2] - s.lo[2];
  return dx * dy + dy * dz + dz * dx;
}

// Expands the frontier's binary nodes into up to four slots each and
// counts their internal slots.
__global__ void k_expand4(const Node* __restrict__ nodes, const int* __restrict__ frontier, int nf,
                          Slot4* __restrict__ slots, int* __restrict__ nslots,
                          int* __restrict__ ninternal) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= nf) return;
  const Node P = nodes[frontier[f]];
  Slot4 s[4];
  int n = 0;
  s[n++] = slot_of(P, 0);
  if (!(P.d.y == P.d.x && P.d.x < 0)) s[n++] = slot_of(P, 1);  // the single-triangle root
  while (n < 4) {
    int best = -1;
    float area = -1.0f;
    for (int j = 0; j < n; ++j)
      if (s[j].ref >= 0 && slot_area(s[j]) > area) {
        area = slot_area(s[j]);
        best = j;
      }
    if (best < 0) break;
    const Node C = nodes[s[best].ref];
    s[n++] = slot_of(C, 1);
    s[best] = slot_of(C, 0);
  }
  int internal = 0;
  for (int j = 0; j < 4; ++j) {
    if (j < n) {
      slots[4 * f + j] = s[j];
      internal += s[j].ref >= 0 ? 1 : 0;
    }
  }
  nslots[f] = n;
  ninternal[f] = internal;
}

__global__ void k_write4(const Slot4* __restrict__ slots, const int* __restrict__ nslots,
                         const int* __restrict__ ninternal, const int* __restrict__ offset, int nf,
                         int level_base, int next_base, const int* __restrict__ parent4,
                         Node4* __restrict__ out, int* __restrict__ next_frontier,
                         int* __restrict__ next_parent4) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= nf) return;
  const int n = nslots[f];
  float v[6][4] = {{0, 0, 0, 0}, {0, 0, 0, 0}, {0, 0, 0, 0}, {0, 0, 0, 0}, {0, 0, 0, 0}, {0, 0, 0, 0}};
  int ch[4] = {0, 0, 0, 0};
  int r = 0;
  for (int j = 0; j < n; ++j) {
    const Slot4 s = slots[4 * f + j];
    for (int a = 0; a < 3; ++a) {
      v[2 * a][j] = s.lo[a];
      v[2 * a + 1][j] = s.hi[a];
    }
    if (s.ref < 0) {
      ch[j] = s.ref;
    } else {
      const int pos = offset[f] + r++;
      ch[j] = next_base + pos;
      next_frontier[pos] = s.ref;
      next_parent4[pos] = level_base + f;
    }
  }
  Node4 n4;
  n4.lox = make_float4(v[0][0], v[0][1], v[0][2], v[0][3]);
  n4.hix = make_float4(v[1][0], v[1][1], v[1][2], v[1][3]);
  n4.loy = make_float4(v[2][0], v[2][1], v[2][2], v[2][3]);
  n4.hiy = make_float4(v[3][0], v[3][1], v[3][2], v[3][3]);
  n4.loz = make_float4(v[4][0], v[4][1], v[4][2], v[4][3]);
  n4.hiz = make_float4(v[5][0], v[5][1], v[5][2], v[5][3]);
  n4.child = make_int4(ch[0], ch[1], ch[2], ch[3]);
  n4.meta = make_int4(parent4[f], (1 << n) - 1, 0, 0);
  out[level_base + f] = n4;
}

// Depth of every leaf (internal nodes on its root path + 1).
__global__ void k_depth(const int32_t* __restrict__ leaf_parent, int n, const Node* __restrict__ nodes,
                        int* max_depth) {
  const int leaf = blockIdx.x * blockDim.x + threadIdx.x;
  if (leaf >= n) return;
  int depth = 1;
  for (int p = leaf_parent[leaf]; p >= 0 && depth < 4096; p = nodes[p].d.z) ++depth;
  atomicMax(max_depth, depth);
}

// Gather triangles into leaf order with edges, normals and materials.
__global__ void k_gather(const float* __restrict__ v, const int32_t* __restrict__ mat_ids,
                         const int32_t* __restrict__ sorted_idx, int n, float4* __restrict__ tris) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  const int t = sorted_idx[j];
  const float* p = v + 9 * (int64_t)t;
  const V3 a = mk(p[0], p[1], p[2]), b = mk(p[3], p[4], p[5]), c = mk(p[6], p[7], p[8]);
  const V3 e1 = sub(b, a), e2 = sub(c, a);
  const V3 nn = normalized(cross(e1, e2));
  tris[4 * j + 0] = make_float4(a.x, a.y, a.z, __int_as_float(t));
  tris[4 * j + 1] = make_float4(e1.x, e1.y, e1.z, 0.0f);
  tris[4 * j + 2] = make_float4(e2.x, e2.y, e2.z, 0.0f);
  tris[4 * j + 3] = make_float4(nn.x, nn.y, nn.z, __int_as_float(mat_ids[t]));
}

// Single-triangle scene: a root whose two children are the same leaf.
__global__ void k_single(const float4* __restrict__ lo, const float4* __restrict__ hi, float pad,
                         Node* nodes) {
  const float4 l = lo[0], h = hi[0];
  const float lx = l.x - pad, ly = l.y - pad, lz = l.z - pad;
  const float hx = h.x + pad, hy = h.y + pad, hz = h.z + pad;
  nodes[0].a = make_float4(lx, hx, ly, hy);
  nodes[0].b = make_float4(lz, hz, lx, hx);
  nodes[0].c = make_float4(ly, hy, lz, hz);
  nodes[0].d = make_int4(~0, ~0, -1, 0);
}

#define CK(x)                                                              \
  do {                                                                     \
    cudaError_t e_ = (x);                                                  \
    if (e_ != cudaSuccess) {                                               \
      snprintf(err, errlen, "%s failed: %s", #x, cudaGetErrorString(e_));  \
      rc = e_;                                                             \
      goto done;                                                           \
    }                                                                      \
  } while (0)

}  // namespace

cudaError_t build_lbvh(DeviceScene& s, float box_pad, int max_leaf, int builder, int radius,
                       cudaStream_t stream, char* err, size_t errlen) {
  const int64_t n64 = s.num_tris;
  cudaError_t rc = cudaSuccess;
  err[0] = 0;
  if (n64 >= (int64_t)kLeafStartMask) {
    snprintf(err, errlen, "too many triangles for one scene (%lld)", (long long)n64);
    return cudaErrorInvalidValue;
  }
  const int n = (int)n64;
  float4 *lo = nullptr, *hi = nullptr, *node_lo = nullptr, *node_hi = nullptr;
  uint32_t *bounds = nullptr, *codes = nullptr, *codes2 = nullptr, *visits = nullptr;
  int32_t *idx = nullptr, *idx2 = nullptr, *leaf_parent = nullptr;
  int2* range = nullptr;
  int* dmax = nullptr;
  int *ssize = nullptr, *spos = nullptr;
  Node* reordered = nullptr;

  // PLOC
  float4 *clo = nullptr, *chi = nullptr, *clo2 = nullptr, *chi2 = nullptr;
  int *cid = nullptr, *cid2 = nullptr, *nnb = nullptr, *mflag = nullptr, *mrank = nullptr;
  int *kflag = nullptr, *kpos = nullptr;
  int2* totals = nullptr;
  void* stmp = nullptr;
  size_t stmp_bytes = 0;
  void* tmp = nullptr;
  size_t tmp_bytes = 0;
  uint32_t hb[7];
  const int nn = n > 1 ? n - 1 : 1;
  const int B = 256;
  const int G = (n + B - 1) / B;
  int depth = 1;

  if (s.nodes) cudaFree(s.nodes);
  if (s.nodes4) cudaFree(s.nodes4);
  s.nodes4 = nullptr;
  s.num_nodes4 = 0;
  s.depth4 = 0;
  if (s.tris) cudaFree(s.tris);
  s.nodes = nullptr;
  s.tris = nullptr;
  s.num_nodes = 0;
  if (n == 0) {
    s.max_depth = 0;
    s.box_pad = 0.0f;
    return cudaSuccess;
  }
  CK(cudaMalloc(&lo, sizeof(float4) * n));
  CK(cudaMalloc(&hi, sizeof(float4) * n));
  CK(cudaMalloc(&bounds, sizeof(uint32_t) * 8));
  CK(cudaMalloc(&codes, sizeof(uint32_t) * n));
  CK(cudaMalloc(&codes2, sizeof(uint32_t) * n));
  CK(cudaMalloc(&idx, sizeof(int32_t) * n));
  CK(cudaMalloc(&idx2, sizeof(int32_t) * n));
  CK(cudaMalloc(&leaf_parent, sizeof(int32_t) * n));
  CK(cudaMalloc(&node_lo, sizeof(float4) * nn));
  CK(cudaMalloc(&node_hi, sizeof(float4) * nn));
  CK(cudaMalloc(&visits, sizeof(uint32_t) * nn));
  CK(cudaMalloc(&range, sizeof(int2) * nn));
  CK(cudaMalloc(&dmax, sizeof(int)));
  CK(cudaMalloc(&s.nodes, sizeof(Node) * nn));
  CK(cudaMalloc(&s.tris, sizeof(float4) * 4 * (size_t)n));
  {
    const uint32_t init[8] = {0xffffffffu, 0xffffffffu, 0xffffffffu, 0u, 0u, 0u, 0u, 0u};
    CK(cudaMemcpyAsync(bounds, init, sizeof init, cudaMemcpyHostToDevice, stream));
  }
  CK(cudaMemsetAsync(visits, 0, sizeof(uint32_t) * nn, stream));
  CK(cudaMemsetAsync(dmax, 0, sizeof(int), stream));
  CK(cudaMemsetAsync(s.nodes, 0, sizeof(Node) * nn, stream));
  k_tri_boxes<<<G, B, 0, stream>>>(s.vertices, n, lo, hi, bounds);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(hb, bounds, sizeof(uint32_t) * 7, cudaMemcpyDeviceToHost, stream));
  CK(cudaStreamSynchronize(stream));
  {
    const float max_abs = unord(hb[6]);
    // default padding: 2^-18 of the largest coordinate (about 20 times the
    // rounding of a slab distance, a few ulp of that coordinate) plus 1e-5.
    // Padding only needs to absorb rounding; more of it makes neighbouring
    // boxes overlap (2^-12: -27% segments/s on the 2,000,000-triangle nave).
    s.box_pad = box_pad >= 0.0f ? box_pad : max_abs * (1.0f / 262144.0f) + 1e-5f;
  }
  if (n == 1) {
    k_single<<<1, 1, 0, stream>>>(lo, hi, s.box_pad, s.nodes);
    CK(cudaGetLastError());
    {
      const int32_t zero = 0;
      CK(cudaMemcpyAsync(idx2, &zero, sizeof zero, cudaMemcpyHostToDevice, stream));
    }
    depth = 1;
  } else {
    k_morton<<<G, B, 0, stream>>>(lo, hi, n, bounds, codes, idx);
    CK(cudaGetLastError());
    CK(cub::DeviceRadixSort::SortPairs(nullptr, tmp_bytes, codes, codes2, idx, idx2, n, 0, 30,
                                       stream));
    CK(cudaMalloc(&tmp, tmp_bytes));
    CK(cub::DeviceRadixSort::SortPairs(tmp, tmp_bytes, codes, codes2, idx, idx2, n, 0, 30,
                                       stream));
    if (builder == kBuilderPloc) {
      CK(cudaMalloc(&clo, sizeof(float4) * n));
      CK(cudaMalloc(&chi, sizeof(float4) * n));
      CK(cudaMalloc(&clo2, sizeof(float4) * n));
      CK(cudaMalloc(&chi2, sizeof(float4) * n));
      CK(cudaMalloc(&cid, sizeof(int) * n));
      CK(cudaMalloc(&cid2, sizeof(int) * n));
      CK(cudaMalloc(&nnb, sizeof(int) * n));
      CK(cudaMalloc(&mflag, sizeof(int) * n));
      CK(cudaMalloc(&mrank, sizeof(int) * n));
      CK(cudaMalloc(&kflag, sizeof(int) * n));
      CK(cudaMalloc(&kpos, sizeof(int) * n));
      CK(cudaMalloc(&totals, sizeof(int2)));
      CK(cub::DeviceScan::ExclusiveSum(nullptr, stmp_bytes, mflag, mrank, n, stream));
      CK(cudaMalloc(&stmp, stmp_bytes));
      k_ploc_init<<<G, B, 0, stream>>>(lo, hi, idx2, n, s.box_pad, clo, chi, cid);
      CK(cudaGetLastError());
      int count = n, created = 0;
      for (int step = 0; count > 1; ++step) {
        const int g = (count + B - 1) / B;
        k_ploc_nn<<<g, B, 0, stream>>>(clo, chi, count, radius, nnb);
        CK(cudaGetLastError());
        k_ploc_flags<<<g, B, 0, stream>>>(nnb, count, mflag, kflag);
        CK(cudaGetLastError());
        size_t tb = stmp_bytes;
        CK(cub::DeviceScan::ExclusiveSum(stmp, tb, mflag, mrank, count, stream));
        tb = stmp_bytes;
        CK(cub::DeviceScan::ExclusiveSum(stmp, tb, kflag, kpos, count, stream));
        k_ploc_totals<<<1, 1, 0, stream>>>(mflag, mrank, kflag, kpos, count, totals);
        CK(cudaGetLastError());
        k_ploc_write<<<g, B, 0, stream>>>(clo, chi, cid, nnb, mflag, mrank, kflag, kpos, count,
                                          (n - 2) - created, clo2, chi2, cid2, s.nodes, leaf_parent);
        CK(cudaGetLastError());
        int2 tot;
        CK(cudaMemcpyAsync(&tot, totals, sizeof tot, cudaMemcpyDeviceToHost, stream));
        CK(cudaStreamSynchronize(stream));
        if (tot.x <= 0 || step > 4 * n) {
          snprintf(err, errlen, "PLOC made no progress at %d clusters", count);
          rc = cudaErrorUnknown;
          goto done;
        }
        std::swap(clo, clo2);
        std::swap(chi, chi2);
        std::swap(cid, cid2);
        count = tot.y;
        created += tot.x;
      }
      k_depth<<<G, B, 0, stream>>>(leaf_parent, n, s.nodes, dmax);
      CK(cudaGetLastError());
    } else {
      k_karras<<<(nn + B - 1) / B, B, 0, stream>>>(codes2, n, s.nodes, leaf_parent, range);
      CK(cudaGetLastError());
      k_refit<<<G, B, 0, stream>>>(lo, hi, idx2, leaf_parent, n, s.box_pad, s.nodes, node_lo,
                                   node_hi, visits);
      CK(cudaGetLastError());
      k_depth<<<G, B, 0, stream>>>(leaf_parent, n, s.nodes, dmax);
      CK(cudaGetLastError());
      if (max_leaf > 1) {
        k_collapse<<<(nn + B - 1) / B, B, 0, stream>>>(range, n, max_leaf, s.nodes);
        CK(cudaGetLastError());
      }
    }
    CK(cudaMemcpyAsync(&depth, dmax, sizeof(int), cudaMemcpyDeviceToHost, stream));
    if (builder == kBuilderPloc || max_leaf <= 1) {
      // depth-first layout (not after a leaf collapse, which leaves
      // unreachable nodes behind)
      CK(cudaMalloc(&ssize, sizeof(int) * nn));
      CK(cudaMalloc(&spos, sizeof(int) * nn));
      CK(cudaMalloc(&reordered, sizeof(Node) * nn));
      CK(cudaMemsetAsync(visits, 0, sizeof(uint32_t) * nn, stream));
      k_subtree_size<<<G, B, 0, stream>>>(leaf_parent, n, s.nodes, visits, ssize);
      CK(cudaGetLastError());
      k_preorder<<<(nn + B - 1) / B, B, 0, stream>>>(s.nodes, ssize, nn, spos);
      CK(cudaGetLastError());
      k_permute<<<(nn + B - 1) / B, B, 0, stream>>>(s.nodes, spos, nn, reordered);
      CK(cudaGetLastError());
      std::swap(s.nodes, reordered);
    }
  }
  {
    // the 4-wide tree, one level per pass
    int *front = nullptr, *front2 = nullptr, *par4 = nullptr, *par4b = nullptr;
    int *nsl = nullptr, *nint = nullptr, *off = nullptr;
    Slot4* slots = nullptr;
    void* st4 = nullptr;
    size_t st4_bytes = 0;
    int levels = 0, nf = 1, base = 0, total = 0;
    bool too_deep = false;
    const int root_parent = -1, root = 0;
    const int cap = nn > 0 ? nn : 1;  // at most one 4-wide node per binary node
    CK(cudaMalloc(&s.nodes4, sizeof(Node4) * (size_t)cap));
    CK(cudaMalloc(&front, sizeof(int) * cap));
    CK(cudaMalloc(&front2, sizeof(int) * cap));
    CK(cudaMalloc(&par4, sizeof(int) * cap));
    CK(cudaMalloc(&par4b, sizeof(int) * cap));
    CK(cudaMalloc(&nsl, sizeof(int) * cap));
    CK(cudaMalloc(&nint, sizeof(int) * cap));
    CK(cudaMalloc(&off, sizeof(int) * cap));
    CK(cudaMalloc(&slots, sizeof(Slot4) * 4 * (size_t)cap));
    CK(cub::DeviceScan::ExclusiveSum(nullptr, st4_bytes, nint, off, cap, stream));
    CK(cudaMalloc(&st4, st4_bytes));
    CK(cudaMemcpyAsync(front, &root, sizeof(int), cudaMemcpyHostToDevice, stream));
    CK(cudaMemcpyAsync(par4, &root_parent, sizeof(int), cudaMemcpyHostToDevice, stream));
    while (nf > 0) {
      if (++levels > kMaxDepth4) {
        too_deep = true;  // beyond the trail: the binary tree serves the scene
        break;
      }
      if (base + nf > cap) {
        snprintf(err, errlen, "4-wide BVH larger than its binary tree");
        rc = cudaErrorInvalidValue;
        break;
      }
      const int gf = (nf + B - 1) / B;
      k_expand4<<<gf, B, 0, stream>>>(s.nodes, front, nf, slots, nsl, nint);
      CK(cudaGetLastError());
      size_t tb = st4_bytes;
      CK(cub::DeviceScan::ExclusiveSum(st4, tb, nint, off, nf, stream));
      int last_off = 0, last_int = 0;
      CK(cudaMemcpyAsync(&last_off, off + nf - 1, sizeof(int), cudaMemcpyDeviceToHost, stream));
      CK(cudaMemcpyAsync(&last_int, nint + nf - 1, sizeof(int), cudaMemcpyDeviceToHost, stream));
      k_write4<<<gf, B, 0, stream>>>(slots, nsl, nint, off, nf, base, base + nf, par4, s.nodes4,
                                     front2, par4b);
      CK(cudaGetLastError());
      CK(cudaStreamSynchronize(stream));
      base += nf;
      nf = last_off + last_int;
      std::swap(front, front2);
      std::swap(par4, par4b);
    }
    total = base;
    cudaFree(front);
    cudaFree(front2);
    cudaFree(par4);
    cudaFree(par4b);
    cudaFree(nsl);
    cudaFree(nint);
    cudaFree(off);
    cudaFree(slots);
    cudaFree(st4);
    if (rc != cudaSuccess) goto done;
    if (too_deep) {
      cudaFree(s.nodes4);
      s.nodes4 = nullptr;
      s.num_nodes4 = 0;
      s.depth4 = 0;
    } else {
      s.num_nodes4 = total;
      s.depth4 = levels;
    }
  }
  k_gather<<<G, B, 0, stream>>>(s.vertices, s.mat_ids, idx2, n, s.tris);
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(stream));
  s.num_nodes = nn;
  s.max_depth = depth;
  s.max_leaf = builder == kBuilderPloc ? 1 : max_leaf;
  s.builder = builder;
  if (depth > 62) {
    snprintf(err, errlen, "LBVH depth %d exceeds the 62 levels of the traversal trail", depth);
    rc = cudaErrorInvalidValue;
  }
done:
  cudaFree(lo);
  cudaFree(hi);
  cudaFree(bounds);
  cudaFree(codes);
  cudaFree(codes2);
  cudaFree(idx);
  cudaFree(idx2);
  cudaFree(leaf_parent);
  cudaFree(node_lo);
  cudaFree(node_hi);
  cudaFree(visits);
  cudaFree(range);
  cudaFree(dmax);
  cudaFree(ssize);
  cudaFree(spos);
  cudaFree(reordered);

  cudaFree(clo);
  cudaFree(chi);
  cudaFree(clo2);
  cudaFree(chi2);
  cudaFree(cid);
  cudaFree(cid2);
  cudaFree(nnb);
  cudaFree(mflag);
  cudaFree(mrank);
  cudaFree(kflag);
  cudaFree(kpos);
  cudaFree(totals);
  cudaFree(stmp);
  cudaFree(tmp);
  return rc;
}

}  // namespace ear
