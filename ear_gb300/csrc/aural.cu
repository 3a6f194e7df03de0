// aural.cu -- auralisation on the device: the equalizer band split of the
// dry sounds and the convolution of the recorder tracks with them, the steps
// of Render() after the impulse responses (src/EAR.cpp:295-386).
//
//  * Band split (Equalizer::Split, lib/equalizer/Equalizer.cpp:81-96): four
//    IIR recurrences per signal.  Each output sample depends on the previous
//    four, in FP32, so each filter runs sequentially -- one lane per filter
//    (low, high, and mid = HP(LP(x))) -- with the reference's operation
//    order (explicit _rn intrinsics, no contraction): bit-identical outputs.
//  * Direct convolution (RecorderTrack::Process without FFTW,
//    src/Recorder.cpp:247-292): out[x] = sum_i s_i * h(x - off - i), summed
//    for each x in ascending i as the reference's loop nest does, then added
//    to the recorder total context by context.  Register-blocked: a thread
//    owns R consecutive outputs and slides the response window through
//    registers; dry and response chunks are staged in shared memory.  The
//    sum order is the reference's, so the results are bit-identical.
//  * FFT convolution (the FFTW build, src/Recorder.cpp:145-243): a
//    hand-written radix-16 Stockham FFT (global-memory passes, L2-resident
//    for these sizes).  The response and the dry section share one complex
//    transform (response real, dry imaginary); the product of their spectra
//    is separated from it, two contexts share one inverse transform.
//    Keyframe pairs fade the section out under this keyframe's response and
//    in under the next's, with the reference's sequential FP32 fade ramp.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <vector>

#include "../../include/ear_gb300.h"
#include "host_internal.h"

namespace ear {
namespace {

// ------------------------------------------------------------- band split

struct LrFilter {
  float a0, a1, a2, a3, a4, b1, b2, b3, b4;
};

// Equalizer::Pass::Pass, LowPass::LowPass, HighPass::HighPass
// (lib/equalizer/Equalizer.cpp:33-79): the same expressions in the same
// order (host code, compiled without contraction); pi is the reference's
// 3.14285714285714f.
LrFilter lr_filter(float fc, bool high) {
  const float srate = 44100.0f;
  const float pi = 3.14285714285714f;
  const float wc = 2.0f * pi * srate;
  const float wc2 = wc * wc;
  const float wc3 = wc2 * wc;
  const float wc4 = wc2 * wc2;
  const float k = wc / std::tan(pi * fc / srate);
  const float k2 = k * k;
  const float k3 = k2 * k;
  const float k4 = k2 * k2;
  const float sqrt2 = std::sqrt(2.0f);
  const float sq_tmp1 = sqrt2 * wc3 * k;
  const float sq_tmp2 = sqrt2 * wc * k3;
  const float a_tmp = 4.0f * wc2 * k2 + 2.0f * sq_tmp1 + k4 + 2.0f * sq_tmp2 + wc4;
  LrFilter f;
  f.b1 = (4.0f * (wc4 + sq_tmp1 - k4 - sq_tmp2)) / a_tmp;
  f.b2 = (6.0f * wc4 - 8.0f * wc2 * k2 + 6.0f * k4) / a_tmp;
  f.b3 = (4.0f * (wc4 - sq_tmp1 + sq_tmp2 - k4)) / a_tmp;
  f.b4 = (k4 - 2.0f * sq_tmp1 + wc4 - 2.0f * sq_tmp2 + 4.0f * wc2 * k2) / a_tmp;
  if (high) {
    f.a0 = k4 / a_tmp;
    f.a1 = -4.0f * k4 / a_tmp;
    f.a2 = 6.0f * k4 / a_tmp;
  } else {
    f.a0 = wc4 / a_tmp;
    f.a1 = 4.0f * wc4 / a_tmp;
    f.a2 = 6.0f * wc4 / a_tmp;
  }
  f.a3 = f.a1;
  f.a4 = f.a0;
  return f;
}

struct SplitArgs {
  const float* x;
  float* out[3];  // low, mid, high
  int64_t n;
  LrFilter f[4];  // per lane: LP1, HP2, LP2, HP1 (crossovers 1 and 2)
};

constexpr int kSplitBlock = 16;

// One warp; lanes 0-3 run one filter each: lane 0 low = LP1(x), lane 1
// high = HP2(x), lane 2 LP2(x), lane 3 mid = HP1(LP2(x)).  The lanes
// advance in lock step through blocks of kSplitBlock samples; lane 3
// filters the block lane 2 finished one block earlier (handed over with
// shuffles between blocks).
//
// Equalizer::Pass::Process (lib/equalizer/Equalizer.cpp:26-31) evaluates
//   out = a0*in + a1*xm1 + a2*xm2 + a3*xm3 + a4*xm4 - b1*ym1 - b2*ym2
//         - b3*ym3 - b4*ym4
// left to right.  Its first five terms involve only inputs, so for a whole
// block they are formed first, as independent chains; the recurrence then
// only subtracts the four feedback products in the same order.  Every
// operation and its rounding are the reference's, so the outputs are the
// sequential filters' bits; the serial chain per sample shrinks to one
// multiply and four subtractions.
__global__ void __launch_bounds__(32) k_band_split(SplitArgs a) {
  constexpr int B = kSplitBlock;
  const int lane = threadIdx.x;
  const LrFilter f = a.f[lane & 3];
  float* out = lane == 0 ? a.out[0] : (lane == 1 ? a.out[2] : a.out[1]);
  const bool writer = lane == 0 || lane == 1 || lane == 3;
  const int64_t nblk = (a.n + B - 1) / B;
  float x1 = 0.0f, x2 = 0.0f, x3 = 0.0f, x4 = 0.0f;  // previous inputs
  float y1 = 0.0f, y2 = 0.0f, y3 = 0.0f, y4 = 0.0f;  // previous outputs
  float xb[B], lp2[B];
#pragma unroll
  for (int u = 0; u < B; ++u) {
    xb[u] = u < a.n ? __ldg(a.x + u) : 0.0f;
    lp2[u] = 0.0f;
  }
  for (int64_t k = 0; k <= nblk; ++k) {
    // lane 3 filters block k - 1 (from lp2); the others block k
    float in[B];
#pragma unroll
    for (int u = 0; u < B; ++u) in[u] = lane == 3 ? lp2[u] : xb[u];
    const int64_t tn = (k + 1) * B;
#pragma unroll
    for (int u = 0; u < B; ++u) xb[u] = tn + u < a.n ? __ldg(a.x + tn + u) : 0.0f;
    // the input terms, a0*in + a1*xm1 + a2*xm2 + a3*xm3 + a4*xm4
    float p[B];
#pragma unroll
    for (int u = 0; u < B; ++u) {
      const float m1 = u >= 1 ? in[u - 1] : x1;
      const float m2 = u >= 2 ? in[u - 2] : (u == 1 ? x1 : x2);
      const float m3 = u >= 3 ? in[u - 3] : (u == 2 ? x1 : (u == 1 ? x2 : x3));
      const float m4 = u >= 4 ? in[u - 4] : (u == 3 ? x1 : (u == 2 ? x2 : (u == 1 ? x3 : x4)));
      float o = __fmul_rn(f.a0, in[u]);
      o = __fadd_rn(o, __fmul_rn(f.a1, m1));
      o = __fadd_rn(o, __fmul_rn(f.a2, m2));
      o = __fadd_rn(o, __fmul_rn(f.a3, m3));
      p[u] = __fadd_rn(o, __fmul_rn(f.a4, m4));
    }
    x4 = in[B - 4];
    x3 = in[B - 3];
    x2 = in[B - 2];
    x1 = in[B - 1];
    // the feedback terms, - b1*ym1 - b2*ym2 - b3*ym3 - b4*ym4
    float ob[B];
#pragma unroll
    for (int u = 0; u < B; ++u) {
      float o = __fsub_rn(p[u], __fmul_rn(f.b1, y1));
      o = __fsub_rn(o, __fmul_rn(f.b2, y2));
      o = __fsub_rn(o, __fmul_rn(f.b3, y3));
      o = __fsub_rn(o, __fmul_rn(f.b4, y4));
      y4 = y3;
      y3 = y2;
      y2 = y1;
      y1 = o;
      ob[u] = o;
    }
#pragma unroll
    for (int u = 0; u < B; ++u) lp2[u] = __shfl_sync(0xffffffffu, ob[u], 2);
    const int64_t t0 = lane == 3 ? (k - 1) * B : k * B;
    if (writer && t0 >= 0) {
#pragma unroll
      for (int u = 0; u < B; ++u)
        if (t0 + u < a.n) out[t0 + u] = ob[u];
    }
  }
}

// ---- chunked band split (EAR_SPLIT_CHUNKED): the same filters evaluated
// in parallel over chunks of kIirChunk samples.  The recurrence is linear:
// a chunk's output is its response from a zero feedback state (inputs and
// their history known) plus the homogeneous response of the true entry
// state.  Phase 1 runs every chunk from a zero state and keeps its last four
// outputs end0(c).  The entry states follow entry(c+1) = M^K entry(c) +
// end0(c) (M: the 4x4 companion matrix of the feedback terms); the filters
// are stable and K = 512 steps shrink M^K far below rounding (|M^K| ~ 1e-6
// for a 600 Hz crossover), so phase 2 unrolls that recurrence only `depth`
// chunks back, entry(c) = sum_{i=1..depth} M^(K(i-1)) end0(c-i) in double,
// with depth chosen on the host so that |M^K|^depth < 1e-12; each chunk
// computes its own entry and re-runs from it.  Chunk 0 starts from
// the true (zero) state, so it is bit-identical to the sequential filter;
// later chunks start from entry states closer to exact arithmetic than the
// sequential FP32 run's, so they follow a different rounding path: both stay
// within the filters' FP32 accuracy (about 1e-3 of the peak in the low
// band), but not bit for bit.
constexpr int kIirChunk = 512;

struct IirJob {
  const float* x;
  float* y;
  int64_t n;
  LrFilter f;
  double mk[16];  // M^kIirChunk, row-major
  int depth;      // chunks back that reach an entry state
};

// One chunk of the filter from the given feedback state (y1..y4); input
// history read from x.  Inputs are loaded 16 at a time ahead of the
// recurrence, so the loads overlap it.
__device__ __forceinline__ void iir_chunk(const IirJob& J, int64_t t0, int64_t t1, float y1,
                                          float y2, float y3, float y4, float* y_out,
                                          float* end) {
  const LrFilter& f = J.f;
  float x1 = t0 >= 1 ? J.x[t0 - 1] : 0.0f, x2 = t0 >= 2 ? J.x[t0 - 2] : 0.0f;
  float x3 = t0 >= 3 ? J.x[t0 - 3] : 0.0f, x4 = t0 >= 4 ? J.x[t0 - 4] : 0.0f;
  for (int64_t tb = t0; tb < t1; tb += 16) {
    float xin[16];
#pragma unroll
    for (int u = 0; u < 16; ++u) xin[u] = tb + u < t1 ? __ldg(J.x + tb + u) : 0.0f;
#pragma unroll
    for (int u = 0; u < 16; ++u) {
      if (tb + u >= t1) break;
      const float in = xin[u];
      float o = __fmul_rn(f.a0, in);
      o = __fadd_rn(o, __fmul_rn(f.a1, x1));
      o = __fadd_rn(o, __fmul_rn(f.a2, x2));
      o = __fadd_rn(o, __fmul_rn(f.a3, x3));
      o = __fadd_rn(o, __fmul_rn(f.a4, x4));
      o = __fsub_rn(o, __fmul_rn(f.b1, y1));
      o = __fsub_rn(o, __fmul_rn(f.b2, y2));
      o = __fsub_rn(o, __fmul_rn(f.b3, y3));
      o = __fsub_rn(o, __fmul_rn(f.b4, y4));
      x4 = x3;
      x3 = x2;
      x2 = x1;
      x1 = in;
      y4 = y3;
      y3 = y2;
      y2 = y1;
      y1 = o;
      if (y_out) y_out[tb + u] = o;
    }
  }
  if (end) {
    end[0] = y1;
    end[1] = y2;
    end[2] = y3;
    end[3] = y4;
  }
}

// Phase 1: blockIdx.y = job, one thread per chunk; end0[job][chunk][4].
__global__ void k_iir_zero(const IirJob* __restrict__ jobs, float* __restrict__ end0, int chunks) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= chunks) return;
  const IirJob& J = jobs[blockIdx.y];
  const int64_t t0 = (int64_t)c * kIirChunk;
  if (t0 >= J.n) return;
  const int64_t t1 = min(J.n, t0 + kIirChunk);
  iir_chunk(J, t0, t1, 0.0f, 0.0f, 0.0f, 0.0f, nullptr,
            end0 + ((int64_t)blockIdx.y * chunks + c) * 4);
}

// Phase 2 and 3: each chunk forms its entry state from the zero-state ends
// of the `depth` chunks before it (Horner in double) and re-runs from it.
__global__ void k_iir_apply(const IirJob* __restrict__ jobs, const float* __restrict__ end0,
                            int chunks) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= chunks) return;
  const IirJob& J = jobs[blockIdx.y];
  const int64_t t0 = (int64_t)c * kIirChunk;
  if (t0 >= J.n) return;
  const int64_t t1 = min(J.n, t0 + kIirChunk);
  double st[4] = {0.0, 0.0, 0.0, 0.0};
  for (int i = min(J.depth, c); i >= 1; --i) {
    const float* z = end0 + ((int64_t)blockIdx.y * chunks + (c - i)) * 4;
    double nx[4];
    for (int r = 0; r < 4; ++r)
      nx[r] = J.mk[4 * r] * st[0] + J.mk[4 * r + 1] * st[1] + J.mk[4 * r + 2] * st[2] +
              J.mk[4 * r + 3] * st[3] + (double)z[r];
    for (int r = 0; r < 4; ++r) st[r] = nx[r];
  }
  iir_chunk(J, t0, t1, (float)st[0], (float)st[1], (float)st[2], (float)st[3], J.y, nullptr);
}

// M^kIirChunk for the feedback recurrence y_t = -b1 y1 - b2 y2 - b3 y3 -
// b4 y4 acting on (y1, y2, y3, y4), by repeated squaring in double.
void companion_power(const LrFilter& f, double* out) {
  double m[16] = {-(double)f.b1, -(double)f.b2, -(double)f.b3, -(double)f.b4, 1, 0, 0, 0,
                  0, 1, 0, 0, 0, 0, 1, 0};
  double r[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
  auto mul = [](const double* a, const double* b, double* c) {
    double t[16];
    for (int i = 0; i < 4; ++i)
      for (int j = 0; j < 4; ++j) {
        double v = 0;
        for (int k = 0; k < 4; ++k) v += a[4 * i + k] * b[4 * k + j];
        t[4 * i + j] = v;
      }
    std::memcpy(c, t, sizeof t);
  };
  for (int e = kIirChunk; e > 0; e >>= 1) {
    if (e & 1) mul(r, m, r);
    mul(m, m, m);
  }
  std::memcpy(out, r, sizeof r);
}

// Chunks back that an entry state needs: the smallest d with
// |M^K|^d < 1e-12 (infinity norm), or -1 when more than 256 would be.  The
// reference's FP32 coefficients (pi = 22/7, products near 1e30) put poles
// outside the unit circle for crossovers below about 110 Hz: its filters
// diverge there, and only the sequential evaluation reproduces them.
int entry_depth(const double* mk) {
  double nrm = 0;
  for (int i = 0; i < 4; ++i)
    nrm = std::max(nrm, std::fabs(mk[4 * i]) + std::fabs(mk[4 * i + 1]) + std::fabs(mk[4 * i + 2]) +
                            std::fabs(mk[4 * i + 3]));
  double p = 1.0;
  for (int d = 1; d <= 256; ++d) {
    p *= nrm;
    if (p < 1e-12) return d;
  }
  return -1;
}

// ------------------------------------------------------ direct convolution

// One context as the direct kernel reads it.  h(j) is the response at j for
// j in [first, len): ir[j] below cap, else 0; with a keyframe partner the
// two responses are read raw over the joint [first, len) (as the reference
// does, src/Recorder.cpp:276-289) and interpolated with i1 = i * inv_n.
struct DirectCtx {
  const float* ir;
  const float* ir2;
  const float* dry;
  int64_t cap, cap2;
  int64_t first, len;
  int64_t n, off;
  float inv_n;
  int interp;
};

constexpr int kDirThreads = 128;
// Outputs per thread: odd, so the window loads are bank-conflict free (9
// measured fastest: 13 cost a third more time through fewer resident
// blocks and spills).
template <bool ANY_INTERP>
struct DirShape {
  static constexpr int R = 9;
  static constexpr int Tile = kDirThreads * R;
  static constexpr int Chunk = 28 * R;  // dry samples staged per step
  static constexpr int Win = Tile + Chunk - 1;
};

__device__ __forceinline__ float dir_h(const float* p, int64_t cap, int64_t j, int64_t lo,
                                       int64_t hi) {
  return (j >= lo && j < hi && j < cap) ? p[j] : 0.0f;
}

// Sum of one context over the block's tile into acc (from +0, ascending i).
template <bool INTERP, typename SH>
__device__ __forceinline__ void direct_context(const DirectCtx& C, int64_t x0, int t, float* s_dry,
                                               float* s_h, float* s_h2, float (&acc)[SH::R]) {
  constexpr int kDirR = SH::R, kDirTile = SH::Tile, kDirChunk = SH::Chunk, kDirWin = SH::Win;
  // dry indices that reach this tile
  const int64_t ilo = max((int64_t)0, x0 - C.off - C.len + 1);
  const int64_t ihi = min(C.n - 1, x0 + kDirTile - 1 - C.off - C.first);
  for (int64_t i0 = ilo; i0 <= ihi; i0 += kDirChunk) {
    __syncthreads();
    for (int k = t; k < kDirChunk; k += kDirThreads) {
      const int64_t i = i0 + k;
      s_dry[k] = i < C.n ? C.dry[i] : 0.0f;
    }
    // response window: s_h[w] = h(jb + w)
    const int64_t jb = x0 - C.off - i0 - (kDirChunk - 1);
    for (int w = t; w < kDirWin; w += kDirThreads) {
      const int64_t j = jb + w;
      s_h[w] = dir_h(C.ir, C.cap, j, C.first, C.len);
      if (INTERP) s_h2[w] = dir_h(C.ir2, C.cap2, j, C.first, C.len);
    }
    __syncthreads();
    // output r of the thread at step k reads s_h[wb + r - k]; the value for
    // index v = r - k sits in register slot v mod kDirR, so one new value is
    // loaded per step and nothing moves
    const int wb = t * kDirR + kDirChunk - 1;
    float hw[kDirR], hw2[kDirR];
#pragma unroll
    for (int r = 0; r < kDirR; ++r) {
      hw[r] = s_h[wb + r];
      hw2[r] = INTERP ? s_h2[wb + r] : 0.0f;
    }
    for (int k0 = 0; k0 < kDirChunk; k0 += kDirR) {
#pragma unroll
      for (int u = 0; u < kDirR; ++u) {
        const int k = k0 + u;
        const float s = s_dry[k];
        if (INTERP) {
          // i1 = i * flt_samples, i2 = 1 - i1 (src/Recorder.cpp:277-278)
          const float i1 = __fmul_rn(__uint2float_rn((unsigned)(i0 + k)), C.inv_n);
          const float i2 = __fsub_rn(1.0f, i1);
#pragma unroll
          for (int r = 0; r < kDirR; ++r) {
            const int q = (r - u + kDirR) % kDirR;
            const float p = __fadd_rn(__fmul_rn(i2, hw[q]), __fmul_rn(i1, hw2[q]));
            acc[r] = __fadd_rn(acc[r], __fmul_rn(s, p));
          }
        } else {
#pragma unroll
          for (int r = 0; r < kDirR; ++r) {
            const int q = (r - u + kDirR) % kDirR;
            acc[r] = __fadd_rn(acc[r], __fmul_rn(s, hw[q]));
          }
        }
        // the slot of index kDirR-1-k leaves; index -k-1 enters
        const int qn = (kDirR - 1 - u) % kDirR;
        const int wn = wb - k - 1;
        if (wn >= 0) {
          hw[qn] = s_h[wn];
          if (INTERP) hw2[qn] = s_h2[wn];
        }
      }
    }
  }
}

// One output track and its contexts [begin, end) of the context table.
struct OutTrack {
  float* out;
  int64_t len;
  int begin, end;
};

// One block: kDirTile consecutive samples of output track blockIdx.y.  For
// each of the track's contexts in order its
// own sum t[x] is accumulated from +0 in ascending i and then added to the
// total, as RecorderTrack::Process and Recorder::Add do.  Terms outside a
// context's range read zero-padded dry or response samples and add +-0,
// which leaves every partial sum unchanged.  ANY_INTERP compiles the
// keyframe-interpolation path in as well.
template <bool ANY_INTERP>
__global__ void __launch_bounds__(kDirThreads) k_conv_direct(const DirectCtx* __restrict__ ctxs,
                                                             const OutTrack* __restrict__ tracks) {
  using SH = DirShape<ANY_INTERP>;
  constexpr int kDirR = SH::R, kDirTile = SH::Tile, kDirChunk = SH::Chunk, kDirWin = SH::Win;
  __shared__ float s_dry[kDirChunk];
  __shared__ float s_h[kDirWin];
  __shared__ float s_h2[ANY_INTERP ? kDirWin : 1];
  const OutTrack T = tracks[blockIdx.y];
  float* __restrict__ out = T.out;
  const int64_t out_len = T.len;
  const int t = threadIdx.x;
  const int64_t x0 = (int64_t)blockIdx.x * kDirTile;
  if (x0 >= out_len) return;  // block-uniform: this track is shorter
  const int64_t xt = x0 + (int64_t)t * kDirR;
  float total[kDirR];
#pragma unroll
  for (int r = 0; r < kDirR; ++r) total[r] = xt + r < out_len ? out[xt + r] : 0.0f;
  for (int c = T.begin; c < T.end; ++c) {
    const DirectCtx C = ctxs[c];
    if (C.len <= C.first || C.n <= 0) continue;
    if (x0 + kDirTile - 1 < C.off + C.first || x0 > C.off + C.n - 1 + C.len - 1) continue;
    float acc[kDirR];
#pragma unroll
    for (int r = 0; r < kDirR; ++r) acc[r] = 0.0f;
    if (ANY_INTERP && C.interp)
      direct_context<true, SH>(C, x0, t, s_dry, s_h, s_h2, acc);
    else
      direct_context<false, SH>(C, x0, t, s_dry, s_h, s_h2, acc);
#pragma unroll
    for (int r = 0; r < kDirR; ++r) total[r] = __fadd_rn(total[r], acc[r]);
  }
#pragma unroll
  for (int r = 0; r < kDirR; ++r)
    if (xt + r < out_len) out[xt + r] = total[r];
}

// --------------------------------------------------------- FFT convolution

__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// exp(-2 pi i m / 2^log2n).  The argument of sincospif is exact for
// 2^log2n <= 2^24; above that the angle is split into a coarse and a fine
// factor.
__device__ __forceinline__ float2 twiddle(uint32_t m, int log2n) {
  float s, c;
  if (log2n <= 24) {
    sincospif(ldexpf((float)m, 1 - log2n), &s, &c);
    return make_float2(c, -s);
  }
  const uint32_t hi = m >> 12, lo = m & 4095u;
  float s2, c2;
  sincospif(ldexpf((float)hi, 13 - log2n), &s, &c);
  sincospif(ldexpf((float)lo, 1 - log2n), &s2, &c2);
  return cmul(make_float2(c, -s), make_float2(c2, -s2));
}

// exp(-2 pi i q / 16), q in [0, 8)
__device__ __forceinline__ float2 w16(int q) {
  constexpr float c1 = 0.923879532511286756f, s1 = 0.382683432365089772f;
  constexpr float h = 0.707106781186547524f;
  switch (q) {
    case 0: return make_float2(1.0f, 0.0f);
    case 1: return make_float2(c1, -s1);
    case 2: return make_float2(h, -h);
    case 3: return make_float2(s1, -c1);
    case 4: return make_float2(0.0f, -1.0f);
    case 5: return make_float2(-s1, -c1);
    case 6: return make_float2(-h, -h);
    default: return make_float2(-c1, -s1);
  }
}

template <int R>
__device__ __forceinline__ int bitrev(int i) {
  int r = 0;
#pragma unroll
  for (int b = 1; b < R; b <<= 1) {
    r = (r << 1) | (i & 1);
    i >>= 1;
  }
  return r;
}

// In-register DFT of size R (2, 4, 8 or 16), natural order in and out:
// iterative radix-2 decimation in time.
template <int R>
__device__ __forceinline__ void dft(float2 (&a)[R]) {
#pragma unroll
  for (int i = 0; i < R; ++i) {
    const int j = bitrev<R>(i);
    if (j > i) {
      const float2 t = a[i];
      a[i] = a[j];
      a[j] = t;
    }
  }
#pragma unroll
  for (int m = 1; m < R; m <<= 1) {
#pragma unroll
    for (int k = 0; k < m; ++k) {
      const float2 w = w16(k * (16 / (2 * m)));
#pragma unroll
      for (int i = k; i < R; i += 2 * m) {
        const float2 u = a[i];
        const float2 v = k == 0 ? a[i + m] : cmul(a[i + m], w);
        a[i] = cadd(u, v);
        a[i + m] = csub(u, v);
      }
    }
  }
}

// One radix-R Stockham pass over every slot of a group (blockIdx.y = slot):
// combines R sub-transforms of size 2^log2ns into one of size 2^log2ns * R.
// After passes with sub-sizes 1, R1, R1*R2, ... the output is in natural
// order.
template <int R>
__global__ void __launch_bounds__(256) k_fft_pass(const float2* __restrict__ in,
                                                  float2* __restrict__ out, int log2l, int log2ns) {
  constexpr int kLogR = R == 2 ? 1 : (R == 4 ? 2 : (R == 8 ? 3 : 4));
  const int64_t l = (int64_t)1 << log2l;
  const int64_t stride = l / R;  // threads per slot
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= stride) return;
  const int64_t base = (int64_t)blockIdx.y * l;
  float2 a[R];
#pragma unroll
  for (int r = 0; r < R; ++r) a[r] = in[base + j + r * stride];
  const int64_t ns = (int64_t)1 << log2ns;
  const int64_t jm = j & (ns - 1);
  if (log2ns > 0) {
#pragma unroll
    for (int r = 1; r < R; ++r) a[r] = cmul(a[r], twiddle((uint32_t)(jm * r), log2ns + kLogR));
  }
  dft<R>(a);
  if (log2ns == 0 && (stride & 255) == 0) {
    // first pass: thread j writes outputs j*R .. j*R+R-1; staged through
    // shared memory (rows padded to R+1) so that a warp's stores are
    // contiguous instead of R-strided
    __shared__ float2 s_t[256 * (R + 1)];
    const int t = threadIdx.x;
#pragma unroll
    for (int r = 0; r < R; ++r) s_t[t * (R + 1) + r] = a[r];
    __syncthreads();
    float2* o = out + base + (int64_t)blockIdx.x * 256 * R;
#pragma unroll
    for (int q = 0; q < R; ++q) {
      const int i = t + 256 * q;
      o[i] = s_t[(i / R) * (R + 1) + (i % R)];
    }
    return;
  }
  const int64_t d = ((j >> log2ns) << (log2ns + kLogR)) + jm;
#pragma unroll
  for (int r = 0; r < R; ++r) out[base + d + r * ns] = a[r];
}

// Input slot of a group: z[t] = h(t) + i * s(t) * fade(t), h read over
// [0, m) (zero from cap on), s over [0, n).
struct FftSlot {
  const float* ir;
  const float* dry;
  const float* fade;  // null: no fade
  int64_t cap, m, n;
};

__global__ void k_fft_pack(const FftSlot* __restrict__ slots, float2* __restrict__ z, int log2l) {
  const int64_t l = (int64_t)1 << log2l;
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= l) return;
  const FftSlot S = slots[blockIdx.y];
  float re = 0.0f, im = 0.0f;
  if (t < S.m && t < S.cap) re = S.ir[t];
  if (t < S.n) im = S.fade ? __fmul_rn(S.dry[t], S.fade[t]) : S.dry[t];
  z[(int64_t)blockIdx.y * l + t] = make_float2(re, im);
}

// RecorderTrack::Process with a fade (src/Recorder.cpp:168-179): factor
// starts at 1 (fade out) or 0 (fade in) and steps by -+1/n in FP32, in
// sequence -- the ramp is the reference's rounded one, not an exact line.
// One thread per ramp.
struct FadeRamp {
  float* out;
  int64_t n;
  int fade_in;
};

__global__ void k_fade_ramp(const FadeRamp* __restrict__ ramps, int num) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= num) return;
  const FadeRamp R = ramps[r];
  float factor = R.fade_in ? 0.0f : 1.0f;
  const float df = __fdiv_rn(R.fade_in ? 1.0f : -1.0f, (float)R.n);
  for (int64_t i = 0; i < R.n; ++i) {
    R.out[i] = factor;
    factor = __fadd_rn(factor, df);
  }
}

// Spectrum product of up to two contexts sharing one inverse transform.
// Z = H + iD of a slot gives H = (Z[k] + conj Z[-k]) / 2 and
// D = (Z[k] - conj Z[-k]) / 2i; a context's spectrum is the sum over its
// one or two slots of H * D.  W = conj(Y_a + i Y_b) / l, so the forward
// transform of W is y_a - i y_b.
struct FftPair {
  int a0, a1, b0, b1;  // slots; -1 = none
};

__device__ __forceinline__ float2 slot_product(const float2* z, int64_t l, int s, int64_t k,
                                               int64_t kn) {
  const float2 zk = z[(int64_t)s * l + k];
  const float2 zn = z[(int64_t)s * l + kn];
  const float2 h = make_float2(0.5f * (zk.x + zn.x), 0.5f * (zk.y - zn.y));
  // (zk - conj zn) / 2i
  const float2 dd = make_float2(0.5f * (zk.x - zn.x), 0.5f * (zk.y + zn.y));
  const float2 d = make_float2(dd.y, -dd.x);
  return cmul(h, d);
}

__global__ void k_fft_product(const float2* __restrict__ z, const FftPair* __restrict__ pairs,
                              float2* __restrict__ w, int log2l) {
  const int64_t l = (int64_t)1 << log2l;
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= l) return;
  const FftPair P = pairs[blockIdx.y];
  const int64_t kn = (l - k) & (l - 1);
  float2 ya = slot_product(z, l, P.a0, k, kn);
  if (P.a1 >= 0) ya = cadd(ya, slot_product(z, l, P.a1, k, kn));
  float2 yb = make_float2(0.0f, 0.0f);
  if (P.b0 >= 0) {
    yb = slot_product(z, l, P.b0, k, kn);
    if (P.b1 >= 0) yb = cadd(yb, slot_product(z, l, P.b1, k, kn));
  }
  const float inv = 1.0f / (float)l;  // exact: l is a power of two
  // y = ya + i yb; w = conj(y) / l
  w[(int64_t)blockIdx.y * l + k] = make_float2((ya.x - yb.y) * inv, -(ya.y + yb.x) * inv);
}

// Processed track of one context: v[x] (real part) or -v[x] (imaginary
// part) of its pair's inverse, for x in [0, mn), landing at off + x.
struct FftOut {
  const float2* v;
  int64_t off, mn;
  int imag;
};

// Output track blockIdx.y: its contexts' processed tracks added in order.
__global__ void k_fft_accumulate(const FftOut* __restrict__ outs,
                                 const OutTrack* __restrict__ tracks) {
  const OutTrack T = tracks[blockIdx.y];
  const int64_t x = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= T.len) return;
  float* out = T.out;
  float acc = out[x];
  for (int c = T.begin; c < T.end; ++c) {
    const FftOut O = outs[c];
    const int64_t u = x - O.off;
    if (u < 0 || u >= O.mn) continue;
    const float2 v = O.v[u];
    acc += O.imag ? -v.y : v.x;
  }
  out[x] = acc;
}

// ------------------------------------------------------------ host side

constexpr int64_t kInitialCapacity = 3 * 44100;  // INITIAL_BUFFER_SIZE, src/Recorder.h:36
// Transform scratch per chunk of contexts: 4 GiB, or EAR_FFT_CHUNK_BYTES
// from the environment (tests use it to force several chunks).
size_t fft_budget() {
  const char* e = std::getenv("EAR_FFT_CHUNK_BYTES");
  if (e && *e) {
    const unsigned long long v = std::strtoull(e, nullptr, 10);
    if (v > 0) return (size_t)v;
  }
  return (size_t)4 << 30;
}
constexpr int64_t kIncrement = 44100;            // INCREMENTAL_BUFFER_SIZE, src/Recorder.h:37

// FloatBuffer capacity after writes that start at index a and then never
// jump more than one past the highest index so far, up to b
// (FloatBuffer::operator[], src/Recorder.cpp:52-59).
int64_t grown(int64_t cap, int64_t a, int64_t b) {
  if (b < a) return cap;
  if (a >= cap) cap = a + kIncrement;
  if (b >= cap) cap += kIncrement * ((b - cap) / kIncrement + 1);
  return cap;
}

// Device scratch, grown on demand and kept per device.
struct Scratch {
  std::mutex mu;
  char* buf = nullptr;
  size_t cap = 0;
  char* tab = nullptr;  // small tables
  size_t tab_cap = 0;
  cudaEvent_t ev[2] = {nullptr, nullptr};
};

Scratch& scratch(int device) {
  static Scratch s[64];
  return s[device & 63];
}

cudaError_t ensure(char** p, size_t* cap, size_t n) {
  if (*cap >= n && *p) return cudaSuccess;
  const size_t want = std::max(n, *cap + *cap / 2);
  if (*p) cudaFree(*p);
  *p = nullptr;
  *cap = 0;
  cudaError_t e = cudaMalloc((void**)p, want);
  if (e == cudaSuccess) *cap = want;
  return e;
}

int log2_ceil(int64_t v) {
  int l = 0;
  while (((int64_t)1 << l) < v) ++l;
  return l;
}

size_t align256(size_t v) { return (v + 255) & ~(size_t)255; }

bool check_context(const ear_conv_context& c, int i) {
  if (c.dry_length < 0 || c.offset < 0 || c.ir_capacity < 0 || c.ir_first < 0 || c.ir_length < 0) {
    fail(EAR_ERR_INVALID_ARG, "ear_convolve: context %d has a negative size or offset", i);
    return false;
  }
  if ((c.dry_length > 0 && !c.dry) || (c.ir_capacity > 0 && !c.ir)) {
    fail(EAR_ERR_INVALID_ARG, "ear_convolve: context %d has a null buffer", i);
    return false;
  }
  if (c.ir_next && (c.ir_next_capacity < 0 || c.ir_next_first < 0 || c.ir_next_length < 0)) {
    fail(EAR_ERR_INVALID_ARG, "ear_convolve: context %d has a negative next-keyframe size", i);
    return false;
  }
  if (c.dry_length > 0x7fffffffLL || c.ir_length > 0x7fffffffLL || c.ir_next_length > 0x7fffffffLL) {
    fail(EAR_ERR_INVALID_ARG, "ear_convolve: context %d exceeds 2^31 samples", i);
    return false;
  }
  return true;
}


// ---- ear_convolve_tracks, step by step

// One call: contexts sorted by output track (each track's in the caller's
// order), the tracks with their context ranges, statistics.
struct ConvCall {
  std::vector<ear_conv_context> ctx;
  std::vector<OutTrack> tracks;
  int64_t max_len = 0;
  cudaStream_t s = nullptr;
  Scratch* sc = nullptr;
  int launches = 0;
  double macs = 0;
  int64_t points = 0;
};

void sort_by_track(const ear_conv_context* contexts, const int32_t* context_track, int num,
                   float* const* outs, const int64_t* out_lengths, int num_tracks, ConvCall* c) {
  std::vector<int> order(num);
  for (int i = 0; i < num; ++i) order[i] = i;
  if (context_track)
    std::stable_sort(order.begin(), order.end(),
                     [&](int x, int y) { return context_track[x] < context_track[y]; });
  c->ctx.resize(num);
  c->tracks.resize(num_tracks);
  for (int o = 0; o < num_tracks; ++o) {
    c->tracks[o] = OutTrack{outs[o], out_lengths[o], 0, 0};
    c->max_len = std::max(c->max_len, out_lengths[o]);
  }
  std::vector<char> seen(num_tracks, 0);
  for (int k = 0; k < num; ++k) {
    c->ctx[k] = contexts[order[k]];
    const int o = context_track ? context_track[order[k]] : 0;
    if (!seen[o]) {
      c->tracks[o].begin = k;
      seen[o] = 1;
    }
    c->tracks[o].end = k + 1;
  }
}

// Response samples a context can read (the direct mode's joint range of a
// keyframe pair; the FFT mode's [0, length)).
int64_t ir_need(const ear_conv_context& c) {
  return std::max(c.ir_length, c.ir_next ? c.ir_next_length : (int64_t)0);
}

// Host-memory calls: every distinct host buffer copied once into the arena
// (a response serves as this keyframe's and the previous keyframe's
// partner; a band serves every recorder), then the output tracks.
struct Staging {
  std::map<const float*, int64_t> spans;  // host buffer -> samples to copy
  std::map<const float*, size_t> at;      // host buffer -> arena offset
  std::vector<size_t> at_out;
  size_t bytes = 0;
};

void plan_staging(const ConvCall& c, Staging* st) {
  auto want = [st](const float* p, int64_t n) {
    if (!p || n <= 0) return;
    int64_t& v = st->spans[p];
    v = std::max(v, n);
  };
  for (const ear_conv_context& x : c.ctx) {
    want(x.ir, std::min(x.ir_capacity, ir_need(x)));
    if (x.ir_next) want(x.ir_next, std::min(x.ir_next_capacity, ir_need(x)));
    want(x.dry, x.dry_length);
  }
  for (const auto& kv : st->spans) {
    st->at[kv.first] = st->bytes;
    st->bytes += align256(sizeof(float) * (size_t)kv.second);
  }
  for (const OutTrack& t : c.tracks) {
    st->at_out.push_back(st->bytes);
    st->bytes += align256(sizeof(float) * (size_t)t.len);
  }
}

// Copies the inputs and outputs and points the contexts and tracks at the
// device copies.
ear_status stage(ConvCall& c, const Staging& st, char* arena, float* const* outs) {
  for (const auto& kv : st.spans)
    CU(cudaMemcpyAsync(arena + st.at.at(kv.first), kv.first, sizeof(float) * kv.second,
                       cudaMemcpyHostToDevice, c.s));
  auto dev = [&](const float* p) {
    return p && st.at.count(p) ? (const float*)(arena + st.at.at(p)) : nullptr;
  };
  for (ear_conv_context& x : c.ctx) {
    const int64_t need = ir_need(x);
    x.ir_capacity = x.ir ? std::min(x.ir_capacity, need) : 0;
    x.ir = dev(x.ir);
    if (x.ir_next) {
      x.ir_next_capacity = std::min(x.ir_next_capacity, need);
      x.ir_next = dev(x.ir_next);
      if (!x.ir_next) {  // nothing to read: keep the context a keyframe pair
        x.ir_next = x.ir ? x.ir : (const float*)arena;
        x.ir_next_capacity = 0;
      }
    }
    if (!x.ir) x.ir_capacity = 0;
    x.dry = dev(x.dry);
  }
  for (size_t o = 0; o < c.tracks.size(); ++o) {
    c.tracks[o].out = (float*)(arena + st.at_out[o]);
    if (c.tracks[o].len > 0)
      CU(cudaMemcpyAsync(c.tracks[o].out, outs[o], sizeof(float) * c.tracks[o].len,
                         cudaMemcpyHostToDevice, c.s));
  }
  return EAR_OK;
}

// Appends 256-byte aligned blocks to a host table that is copied once.
size_t push_block(std::vector<char>* tab, const void* p, size_t bytes) {
  const size_t at = align256(tab->size());
  tab->resize(at + bytes);
  if (bytes) std::memcpy(tab->data() + at, p, bytes);
  return at;
}

ear_status run_direct(ConvCall& c) {
  const int num = (int)c.ctx.size();
  std::vector<DirectCtx> dc(num);
  bool any_interp = false;
  for (int i = 0; i < num; ++i) {
    const ear_conv_context& x = c.ctx[i];
    DirectCtx& d = dc[i];
    d.ir = x.ir;
    d.ir2 = x.ir_next;
    d.dry = x.dry;
    d.cap = x.ir ? x.ir_capacity : 0;
    d.cap2 = x.ir_next ? x.ir_next_capacity : 0;
    d.first = x.ir_next ? std::min(x.ir_first, x.ir_next_first) : x.ir_first;
    d.len = x.ir_next ? std::max(x.ir_length, x.ir_next_length) : x.ir_length;
    d.n = x.dry_length;
    d.off = x.offset;
    d.inv_n = x.dry_length > 0 ? 1.0f / (float)(uint32_t)x.dry_length : 0.0f;
    d.interp = x.ir_next ? 1 : 0;
    any_interp |= d.interp != 0;
    if (d.len > d.first && d.n > 0) c.macs += (double)d.n * (double)(d.len - d.first);
  }
  std::vector<char> tab;
  const size_t at = push_block(&tab, dc.data(), sizeof(DirectCtx) * num);
  const size_t at_t = push_block(&tab, c.tracks.data(), sizeof(OutTrack) * c.tracks.size());
  Scratch& sc = *c.sc;
  CU(ensure(&sc.tab, &sc.tab_cap, tab.size()));
  CU(cudaMemcpyAsync(sc.tab, tab.data(), tab.size(), cudaMemcpyHostToDevice, c.s));
  const DirectCtx* d_ctx = (const DirectCtx*)(sc.tab + at);
  const OutTrack* d_tracks = (const OutTrack*)(sc.tab + at_t);
  const int tile = any_interp ? DirShape<true>::Tile : DirShape<false>::Tile;
  const int64_t blocks = (c.max_len + tile - 1) / tile;
  if (blocks > 0x7fffffffLL) return fail(EAR_ERR_INVALID_ARG, "ear_convolve: output too long");
  const dim3 grid((unsigned)blocks, (unsigned)c.tracks.size());
  if (any_interp)
    k_conv_direct<true><<<grid, kDirThreads, 0, c.s>>>(d_ctx, d_tracks);
  else
    k_conv_direct<false><<<grid, kDirThreads, 0, c.s>>>(d_ctx, d_tracks);
  ++c.launches;
  CU(cudaGetLastError());
  return EAR_OK;
}

// FFT mode plan: groups of equal transform size inside chunks of contexts
// whose scratch fits fft_budget().  Each chunk adds its contexts to the
// outputs in order, so the sums keep the order of one pass.
struct Group {
  int log2l;
  std::vector<int> jobs;  // context indices in order
  int slots = 0, pairs = 0;
  size_t at_a = 0, at_b = 0;
};

struct Chunk {
  int begin, end;
  std::vector<Group> groups;
  size_t bytes = 0;
};

struct FftPlan {
  std::vector<Chunk> chunks;
  std::vector<int> slot0, nslot, log2l_of;
  std::vector<size_t> at_ramp;
  size_t ramp_bytes = 0, fft_bytes = 0;
};

ear_status plan_fft(const ConvCall& c, FftPlan* p) {
  const int num = (int)c.ctx.size();
  p->slot0.assign(num, -1);
  p->nslot.assign(num, 0);
  p->log2l_of.assign(num, 0);
  p->at_ramp.assign(num, 0);
  for (int i = 0; i < num; ++i) {
    const ear_conv_context& x = c.ctx[i];
    int64_t mn = x.ir_length + x.dry_length + 1;
    if (x.ir_next) mn = std::max(mn, x.ir_next_length + x.dry_length + 1);
    p->log2l_of[i] = std::max(4, log2_ceil(mn));
    if (p->log2l_of[i] > 30)
      return fail(EAR_ERR_INVALID_ARG, "ear_convolve: a context needs a 2^%d transform",
                  p->log2l_of[i]);
    p->nslot[i] = x.ir_next ? 2 : 1;
    if (x.ir_next && x.dry_length > 0) {
      p->at_ramp[i] = p->ramp_bytes;
      p->ramp_bytes += align256(sizeof(float) * 2 * (size_t)x.dry_length);
    }
  }
  size_t run = 0;
  const size_t budget = fft_budget();
  for (int i = 0; i < num; ++i) {
    // forward slots in A, pair results in B: about 2.5 transforms a slot
    const size_t est = sizeof(float2) * ((size_t)5 * p->nslot[i] / 2 + 1) << p->log2l_of[i];
    if (p->chunks.empty() || (run + est > budget && p->chunks.back().end > p->chunks.back().begin)) {
      p->chunks.push_back(Chunk{i, i, {}, 0});
      run = 0;
    }
    run += est;
    p->chunks.back().end = i + 1;
  }
  for (Chunk& ch : p->chunks) {
    for (int i = ch.begin; i < ch.end; ++i) {
      auto it = std::find_if(ch.groups.begin(), ch.groups.end(),
                             [&](const Group& g) { return g.log2l == p->log2l_of[i]; });
      if (it == ch.groups.end()) {
        ch.groups.push_back(Group{p->log2l_of[i], {}, 0, 0, 0, 0});
        it = ch.groups.end() - 1;
      }
      it->jobs.push_back(i);
    }
    for (Group& g : ch.groups) {
      for (int i : g.jobs) {
        p->slot0[i] = g.slots;
        g.slots += p->nslot[i];
      }
      g.pairs = ((int)g.jobs.size() + 1) / 2;
      const size_t l = (size_t)1 << g.log2l;
      g.at_a = ch.bytes;
      ch.bytes += align256(sizeof(float2) * l * (size_t)g.slots);
      g.at_b = ch.bytes;
      ch.bytes += align256(sizeof(float2) * l * (size_t)std::max(g.slots, g.pairs));
    }
    p->fft_bytes = std::max(p->fft_bytes, ch.bytes);
  }
  return EAR_OK;
}

// Radix-16 passes, then one of radix 2/4/8 for the remaining bits; returns
// the buffer that holds the result.
float2* fft_passes(ConvCall& c, float2* x, float2* y, int log2l, int count) {
  int ns = 0;
  float2* in = x;
  float2* o = y;
  const int64_t l = (int64_t)1 << log2l;
  while (ns < log2l) {
    const int rem = log2l - ns;
    const int lr = rem >= 4 ? 4 : rem;
    const int64_t thr = l >> lr;
    dim3 grid((unsigned)((thr + 255) / 256), (unsigned)count);
    switch (lr) {
      case 4: k_fft_pass<16><<<grid, 256, 0, c.s>>>(in, o, log2l, ns); break;
      case 3: k_fft_pass<8><<<grid, 256, 0, c.s>>>(in, o, log2l, ns); break;
      case 2: k_fft_pass<4><<<grid, 256, 0, c.s>>>(in, o, log2l, ns); break;
      default: k_fft_pass<2><<<grid, 256, 0, c.s>>>(in, o, log2l, ns); break;
    }
    ++c.launches;
    ns += lr;
    std::swap(in, o);
  }
  return in;
}

ear_status run_fft(ConvCall& c, const FftPlan& p, char* fft_arena, float* ramps) {
  const int num = (int)c.ctx.size();
  // fade ramps of keyframe pairs (every chunk's), one table at the front
  std::vector<char> tab;
  std::vector<FadeRamp> fr;
  for (int i = 0; i < num; ++i) {
    const ear_conv_context& x = c.ctx[i];
    if (!x.ir_next || x.dry_length <= 0) continue;
    float* r = (float*)((char*)ramps + p.at_ramp[i]);
    fr.push_back(FadeRamp{r, x.dry_length, 0});
    fr.push_back(FadeRamp{r + x.dry_length, x.dry_length, 1});
  }
  if (!fr.empty()) push_block(&tab, fr.data(), sizeof(FadeRamp) * fr.size());
  const size_t chunk_tab0 = align256(tab.size());
  // per chunk: slot and pair tables of its groups, its contexts' results
  // and the output tracks restricted to its contexts
  struct ChunkTabs {
    std::vector<char> tab;
    std::vector<size_t> at_slots, at_pairs;
    size_t at_outs = 0, at_tracks = 0;
  };
  std::vector<ChunkTabs> ct(p.chunks.size());
  size_t max_tab = 0;
  for (size_t ci = 0; ci < p.chunks.size(); ++ci) {
    const Chunk& ch = p.chunks[ci];
    ChunkTabs& T = ct[ci];
    std::vector<FftOut> couts((size_t)(ch.end - ch.begin));
    for (const Group& g : ch.groups) {
      std::vector<FftSlot> slots(g.slots);
      for (int i : g.jobs) {
        const ear_conv_context& x = c.ctx[i];
        const float* ra =
            x.ir_next && x.dry_length > 0 ? (float*)((char*)ramps + p.at_ramp[i]) : nullptr;
        slots[p.slot0[i]] = FftSlot{x.ir, x.dry, ra, x.ir ? x.ir_capacity : 0, x.ir_length,
                                    x.dry_length};
        if (x.ir_next)
          slots[p.slot0[i] + 1] = FftSlot{x.ir_next, x.dry, ra ? ra + x.dry_length : nullptr,
                                          x.ir_next_capacity, x.ir_next_length, x.dry_length};
      }
      std::vector<FftPair> pairs(g.pairs);
      for (int q = 0; q < g.pairs; ++q) {
        const int ia = g.jobs[2 * q];
        const int ib = 2 * q + 1 < (int)g.jobs.size() ? g.jobs[2 * q + 1] : -1;
        FftPair& P = pairs[q];
        P.a0 = p.slot0[ia];
        P.a1 = p.nslot[ia] == 2 ? p.slot0[ia] + 1 : -1;
        P.b0 = ib >= 0 ? p.slot0[ib] : -1;
        P.b1 = ib >= 0 && p.nslot[ib] == 2 ? p.slot0[ib] + 1 : -1;
      }
      T.at_slots.push_back(push_block(&T.tab, slots.data(), sizeof(FftSlot) * slots.size()));
      T.at_pairs.push_back(push_block(&T.tab, pairs.data(), sizeof(FftPair) * pairs.size()));
      // the inverse of each pair ends in A or B by the parity of the passes
      float2* A = (float2*)(fft_arena + g.at_a);
      float2* B = (float2*)(fft_arena + g.at_b);
      const int npass = (g.log2l + 3) / 4;
      float2* fwd = (npass % 2) ? B : A;
      float2* prod = fwd == A ? B : A;
      float2* inv = (npass % 2) ? (prod == A ? B : A) : prod;
      const int64_t l = (int64_t)1 << g.log2l;
      c.points += l * (int64_t)(g.slots + g.pairs);
      for (int q = 0; q < g.pairs; ++q)
        for (int h = 0; h < 2 && 2 * q + h < (int)g.jobs.size(); ++h) {
          const int i = g.jobs[2 * q + h];
          const ear_conv_context& x = c.ctx[i];
          couts[(size_t)(i - ch.begin)] = FftOut{
              inv + (int64_t)q * l, x.offset, ir_need(x) + x.dry_length + 1, h};
        }
    }
    T.at_outs = push_block(&T.tab, couts.data(), sizeof(FftOut) * couts.size());
    std::vector<OutTrack> tr(c.tracks);
    for (OutTrack& t : tr) {
      const int b = std::max(t.begin, ch.begin), e = std::min(t.end, ch.end);
      t.begin = b < e ? b - ch.begin : 0;
      t.end = b < e ? e - ch.begin : 0;
    }
    T.at_tracks = push_block(&T.tab, tr.data(), sizeof(OutTrack) * tr.size());
    max_tab = std::max(max_tab, T.tab.size());
  }
  Scratch& sc = *c.sc;
  CU(ensure(&sc.tab, &sc.tab_cap, chunk_tab0 + max_tab));
  char* dtab = sc.tab;
  if (!fr.empty()) {
    CU(cudaMemcpyAsync(dtab, tab.data(), tab.size(), cudaMemcpyHostToDevice, c.s));
    k_fade_ramp<<<((int)fr.size() + 63) / 64, 64, 0, c.s>>>((const FadeRamp*)dtab, (int)fr.size());
    ++c.launches;
  }
  for (size_t ci = 0; ci < p.chunks.size(); ++ci) {
    const Chunk& ch = p.chunks[ci];
    const ChunkTabs& T = ct[ci];
    char* ctab = dtab + chunk_tab0;
    // in stream order after the previous chunk's kernels; the pageable host
    // table is staged before cudaMemcpyAsync returns
    CU(cudaMemcpyAsync(ctab, T.tab.data(), T.tab.size(), cudaMemcpyHostToDevice, c.s));
    for (size_t gi = 0; gi < ch.groups.size(); ++gi) {
      const Group& g = ch.groups[gi];
      float2* A = (float2*)(fft_arena + g.at_a);
      float2* B = (float2*)(fft_arena + g.at_b);
      const int lg = g.log2l;
      const int64_t l = (int64_t)1 << lg;
      dim3 gp((unsigned)((l + 255) / 256), (unsigned)g.slots);
      k_fft_pack<<<gp, 256, 0, c.s>>>((const FftSlot*)(ctab + T.at_slots[gi]), A, lg);
      ++c.launches;
      float2* z = fft_passes(c, A, B, lg, g.slots);
      float2* w = z == A ? B : A;
      dim3 gq((unsigned)((l + 255) / 256), (unsigned)g.pairs);
      k_fft_product<<<gq, 256, 0, c.s>>>(z, (const FftPair*)(ctab + T.at_pairs[gi]), w, lg);
      ++c.launches;
      fft_passes(c, w, z, lg, g.pairs);
    }
    k_fft_accumulate<<<dim3((unsigned)((c.max_len + 255) / 256), (unsigned)c.tracks.size()), 256,
                       0, c.s>>>((const FftOut*)(ctab + T.at_outs),
                                 (const OutTrack*)(ctab + T.at_tracks));
    ++c.launches;
    CU(cudaGetLastError());
  }
  return EAR_OK;
}

}  // namespace
}  // namespace ear

using namespace ear;

extern "C" {

int64_t ear_conv_processed_capacity(const ear_conv_context* c, int32_t mode) {
  if (!c) return kInitialCapacity;
  const int64_t n = c->dry_length, off = c->offset;
  if (mode == EAR_CONV_DIRECT) {
    int64_t first = c->ir_first, len = c->ir_length;
    if (c->ir_next) {
      first = std::min(first, c->ir_next_first);
      len = std::max(len, c->ir_next_length);
    }
    if (n <= 0 || len <= first) return kInitialCapacity;
    return grown(kInitialCapacity, off + first, off + (n - 1) + (len - 1));
  }
  // FFT: c[i] written to off + i for i < M + N + 1
  const int64_t ca = grown(kInitialCapacity, off, off + c->ir_length + n);
  if (!c->ir_next) return ca;
  const int64_t cb = grown(kInitialCapacity, off, off + c->ir_next_length + n);
  // a->Add(b) reads b over its capacity (src/Recorder.cpp:294-299)
  return grown(ca, 0, cb - 1);
}

int64_t ear_conv_processed_length(const ear_conv_context* c, int32_t mode) {
  if (!c) return 0;
  const int64_t n = c->dry_length, off = c->offset;
  if (mode == EAR_CONV_DIRECT) {
    int64_t first = c->ir_first, len = c->ir_length;
    if (c->ir_next) {
      first = std::min(first, c->ir_next_first);
      len = std::max(len, c->ir_next_length);
    }
    if (n <= 0 || len <= first) return 0;
    return off + (n - 1) + (len - 1);
  }
  const int64_t ra = off + c->ir_length + n;  // last of off + [0, M + N + 1)
  if (!c->ir_next) return ra;
  const int64_t cb = grown(kInitialCapacity, off, off + c->ir_next_length + n);
  return std::max(ra, cb - 1);
}

ear_status ear_band_split(const float* dry, int64_t n, const float freq_khz[3], float* low,
                          float* mid, float* high, uint32_t flags, void* stream, int32_t device) {
  if (n < 0 || !freq_khz) return fail(EAR_ERR_INVALID_ARG, "ear_band_split: bad arguments");
  if (n > 0 && (!dry || !low || !mid || !high))
    return fail(EAR_ERR_INVALID_ARG, "ear_band_split: null buffer");
  for (int i = 0; i < 3; ++i)
    if (!(freq_khz[i] > 0.0f) || !(freq_khz[i] * 1000.0f < 22050.0f))
      return fail(EAR_ERR_INVALID_ARG, "ear_band_split: band frequency %d out of (0, 22.05) kHz", i);
  if (n == 0) return EAR_OK;
  CU(cudaSetDevice(device));
  // SoundFile::Band multiplies by 1000, Equalizer::Split averages
  // neighbours (src/SoundFile.cpp:153, lib/equalizer/Equalizer.cpp:84-85)
  const float f1 = freq_khz[0] * 1000.0f, f2 = freq_khz[1] * 1000.0f, f3 = freq_khz[2] * 1000.0f;
  const float fc1 = (f1 + f2) / 2.0f, fc2 = (f2 + f3) / 2.0f;
  SplitArgs a;
  a.f[0] = lr_filter(fc1, false);  // lo_pass1 -> low
  a.f[1] = lr_filter(fc2, true);   // hi_pass2 -> high
  a.f[2] = lr_filter(fc2, false);  // lo_pass2
  a.f[3] = lr_filter(fc1, true);   // hi_pass1 (of lo_pass2) -> mid
  a.n = n;
  const bool on_dev = flags & EAR_AURAL_DEVICE_MEMORY;
  cudaStream_t s = on_dev ? (cudaStream_t)stream : nullptr;
  Scratch& sc = scratch(device);
  std::lock_guard<std::mutex> lock(sc.mu);
  if (on_dev) {
    a.x = dry;
    a.out[0] = low;
    a.out[1] = mid;
    a.out[2] = high;
  } else {
    CU(ensure(&sc.buf, &sc.cap, sizeof(float) * 4 * (size_t)n));
    float* d = (float*)sc.buf;
    CU(cudaMemcpyAsync(d, dry, sizeof(float) * n, cudaMemcpyHostToDevice, s));
    a.x = d;
    a.out[0] = d + n;
    a.out[1] = d + 2 * n;
    a.out[2] = d + 3 * n;
  }
  IirJob jobs[4];
  bool chunked = (flags & EAR_SPLIT_CHUNKED) != 0;
  if (chunked) {
    // fall back to the sequential filters when a crossover is so low that
    // the entry recurrence would need more than 256 chunks
    for (int j = 0; j < 4 && chunked; ++j) {
      companion_power(a.f[j], jobs[j].mk);
      jobs[j].depth = entry_depth(jobs[j].mk);
      chunked = jobs[j].depth > 0;
    }
  }
  if (chunked) {
    // low, high and LP2 (into the mid buffer) at once, then HP1 in place of
    // it through a temporary copy of its input
    const int chunks = (int)((n + kIirChunk - 1) / kIirChunk);
    const size_t tabs = align256(sizeof(IirJob) * 4) + align256(sizeof(float) * 4 * 3 * chunks) +
                        align256(sizeof(float) * (size_t)n);
    CU(ensure(&sc.tab, &sc.tab_cap, tabs));
    const float* src[4] = {a.x, a.x, a.x, nullptr};
    float* dst[4] = {a.out[0], a.out[2], a.out[1], a.out[1]};
    char* t = sc.tab;
    IirJob* d_jobs = (IirJob*)t;
    float* end0 = (float*)(t + align256(sizeof(IirJob) * 4));
    float* tmp = (float*)((char*)end0 + align256(sizeof(float) * 4 * 3 * chunks));
    src[3] = tmp;
    for (int j = 0; j < 4; ++j) {
      jobs[j].x = src[j];
      jobs[j].y = dst[j];
      jobs[j].n = n;
      jobs[j].f = a.f[j];
    }
    CU(cudaMemcpyAsync(d_jobs, jobs, sizeof jobs, cudaMemcpyHostToDevice, s));
    const dim3 g3((unsigned)((chunks + 63) / 64), 3), g1((unsigned)((chunks + 63) / 64), 1);
    k_iir_zero<<<g3, 64, 0, s>>>(d_jobs, end0, chunks);
    k_iir_apply<<<g3, 64, 0, s>>>(d_jobs, end0, chunks);
    CU(cudaMemcpyAsync(tmp, a.out[1], sizeof(float) * n, cudaMemcpyDeviceToDevice, s));
    k_iir_zero<<<g1, 64, 0, s>>>(d_jobs + 3, end0, chunks);
    k_iir_apply<<<g1, 64, 0, s>>>(d_jobs + 3, end0, chunks);
  } else {
    k_band_split<<<1, 32, 0, s>>>(a);
  }
  CU(cudaGetLastError());
  if (!on_dev) {
    CU(cudaMemcpyAsync(low, a.out[0], sizeof(float) * n, cudaMemcpyDeviceToHost, s));
    CU(cudaMemcpyAsync(mid, a.out[1], sizeof(float) * n, cudaMemcpyDeviceToHost, s));
    CU(cudaMemcpyAsync(high, a.out[2], sizeof(float) * n, cudaMemcpyDeviceToHost, s));
  }
  CU(cudaStreamSynchronize(s));
  return EAR_OK;
}

ear_status ear_convolve(const ear_conv_context* contexts, int32_t num, int32_t mode, float* out,
                        int64_t out_length, uint32_t flags, void* stream, int32_t device,
                        ear_conv_stats* stats) {
  return ear_convolve_tracks(contexts, nullptr, num, mode, &out, &out_length, 1, flags, stream,
                             device, stats);
}

ear_status ear_convolve_tracks(const ear_conv_context* contexts, const int32_t* context_track,
                               int32_t num, int32_t mode, float* const* outs,
                               const int64_t* out_lengths, int32_t num_tracks, uint32_t flags,
                               void* stream, int32_t device, ear_conv_stats* stats) {
  if (stats) std::memset(stats, 0, sizeof *stats);
  if (num < 0 || (num > 0 && !contexts) || num_tracks < 1 || num_tracks > 65535 || !outs ||
      !out_lengths || (num_tracks > 1 && num > 0 && !context_track))
    return fail(EAR_ERR_INVALID_ARG, "ear_convolve: bad arguments");
  if (mode != EAR_CONV_FFT && mode != EAR_CONV_DIRECT)
    return fail(EAR_ERR_INVALID_ARG, "ear_convolve: unknown mode %d", mode);
  for (int o = 0; o < num_tracks; ++o)
    if (out_lengths[o] < 0 || (out_lengths[o] > 0 && !outs[o]))
      return fail(EAR_ERR_INVALID_ARG, "ear_convolve: output track %d is invalid", o);
  for (int i = 0; i < num; ++i) {
    if (!check_context(contexts[i], i)) return EAR_ERR_INVALID_ARG;
    if (context_track && (context_track[i] < 0 || context_track[i] >= num_tracks))
      return fail(EAR_ERR_INVALID_ARG, "ear_convolve: context %d names track %d of %d", i,
                  context_track[i], num_tracks);
  }
  ConvCall c;
  sort_by_track(contexts, context_track, num, outs, out_lengths, num_tracks, &c);
  if (num == 0 || c.max_len == 0) return EAR_OK;
  FftPlan plan;
  if (mode == EAR_CONV_FFT) {
    const ear_status rc = plan_fft(c, &plan);
    if (rc != EAR_OK) return rc;
  }
  CU(cudaSetDevice(device));
  const bool on_dev = flags & EAR_AURAL_DEVICE_MEMORY;
  c.s = on_dev ? (cudaStream_t)stream : nullptr;
  Scratch& sc = scratch(device);
  c.sc = &sc;
  std::lock_guard<std::mutex> lock(sc.mu);
  if (!sc.ev[0]) {
    CU(cudaEventCreate(&sc.ev[0]));
    CU(cudaEventCreate(&sc.ev[1]));
  }
  // arena: staged inputs and outputs (host calls), fade ramps, transforms
  Staging st;
  if (!on_dev) plan_staging(c, &st);
  const size_t total_bytes = st.bytes + plan.ramp_bytes + plan.fft_bytes;
  if (total_bytes > 0) CU(ensure(&sc.buf, &sc.cap, total_bytes));
  char* arena = sc.buf;
  if (!on_dev) {
    const ear_status rc = stage(c, st, arena, outs);
    if (rc != EAR_OK) return rc;
  }
  CU(cudaEventRecord(sc.ev[0], c.s));
  const ear_status rc = mode == EAR_CONV_DIRECT
                            ? run_direct(c)
                            : run_fft(c, plan, arena + st.bytes + plan.ramp_bytes,
                                      (float*)(arena + st.bytes));
  if (rc != EAR_OK) return rc;
  CU(cudaEventRecord(sc.ev[1], c.s));
  if (!on_dev)
    for (int o = 0; o < num_tracks; ++o)
      if (out_lengths[o] > 0)
        CU(cudaMemcpyAsync(outs[o], c.tracks[o].out, sizeof(float) * out_lengths[o],
                           cudaMemcpyDeviceToHost, c.s));
  CU(cudaStreamSynchronize(c.s));
  if (stats) {
    float ms = 0;
    cudaEventElapsedTime(&ms, sc.ev[0], sc.ev[1]);
    stats->kernel_ms = ms;
    stats->launches = c.launches;
    stats->fft_points = c.points;
    stats->multiply_adds = c.macs;
  }
  return EAR_OK;
}


}  // extern "C"
