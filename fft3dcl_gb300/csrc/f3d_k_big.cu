// f3d_k_big.cu -- exact-form kernels for blocks above 64 (bw or bh up to
// 512: the reference CPU backend rounds block sizes to powers of two in
// 4..512, src/params.h:62-72; its OpenCL backend stops at 64,
// src/cl/gpu.cpp:82-89).
//
// A block of up to 512 x 512 samples does not fit in registers or shared
// memory, so one CTA owns one block and keeps its half spectrum (forward) or
// its full complex spectrum (inverse, InvArgs::work) in global memory. Every
// row and column transform is the reference's radix-2 DIT
// (src/cpu/fft.cpp:28-58) run by one warp over a shared-memory buffer:
// bit-reversed load, stages len = 2..n, each butterfly (u + w*b, u - w*b)
// with the product written as in the reference, and for the inverse a final
// scale by 1/n. The butterflies of one stage are independent, so the result
// does not depend on which lane computes which; with --fmad=false the bits
// equal the reference CPU backend's.
#include "f3d_device.cuh"

namespace f3d {
namespace {

constexpr int kBigThreads = 256;
constexpr int kBigWarps = kBigThreads / 32;
constexpr int kBigMax = 512;

__device__ __forceinline__ int log2_int(int n) {
  int l = 0;
  while ((1 << l) < n) l++;
  return l;
}

__device__ __forceinline__ int bit_reverse_rt(int i, int bits) {
  return (int)(__brev((unsigned)i) >> (32 - bits));
}

// Stages len = 2..n of the radix-2 DIT on a (already in bit-reversed order),
// one warp; the j = 0 twiddle (1, -0) leaves b unchanged and is skipped as in
// fft_r2_stage (f3d_device.cuh). tw: n/2 twiddles e^(-2 pi i k/n),
// conjugated for the inverse, which then scales by 1/n.
__device__ void fft_warp(float2* a, int n, const float2* tw, bool inv, int lane) {
  for (int len = 2; len <= n; len <<= 1) {
    const int half = len >> 1, step = n / len;
    for (int k = lane; k < n / 2; k += 32) {
      const int grp = k / half, j = k - grp * half;
      const int i0 = grp * len + j, i1 = i0 + half;
      const float2 b = a[i1];
      float2 t;
      if (j == 0) {
        t = b;
      } else {
        const float2 w = tw[j * step];
        const float wy = inv ? -w.y : w.y;
        t.x = w.x * b.x - wy * b.y;
        t.y = w.x * b.y + wy * b.x;
      }
      const float2 u = a[i0];
      a[i0] = make_float2(u.x + t.x, u.y + t.y);
      a[i1] = make_float2(u.x - t.x, u.y - t.y);
    }
    __syncwarp();
  }
  if (inv) {
    const float invn = 1.0f / n;
    for (int i = lane; i < n; i += 32) a[i] = make_float2(a[i].x * invn, a[i].y * invn);
    __syncwarp();
  }
}

// Shared memory: one transform buffer per warp, then the row and column
// twiddles.
__device__ __forceinline__ void load_twiddles(const float2* twr, const float2* twc, int bw, int bh, float2* sr,
                                              float2* sc) {
  for (int i = threadIdx.x; i < bw / 2; i += kBigThreads) sr[i] = twr[i];
  for (int i = threadIdx.x; i < bh / 2; i += kBigThreads) sc[i] = twc[i];
}

// One block: gather with mirror addressing, convert, subtract the chroma
// centering, analysis window (src/cpu/reference.cpp:140-159); row transforms
// keeping fbw columns, then the fbw column transforms
// (src/cpu/fft.cpp:68-86), in place in the block's half spectrum.
__global__ void __launch_bounds__(kBigThreads) k_forward_big(const __grid_constant__ FwdArgs a) {
  extern __shared__ float2 sm_big[];
  const int bw = a.g.bw, bh = a.g.bh, fbw = bw / 2 + 1;
  const int lbw = log2_int(bw), lbh = log2_int(bh);
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  float2* buf = sm_big + w * kBigMax;
  float2* twr = sm_big + kBigWarps * kBigMax;
  float2* twc = twr + kBigMax / 2;
  load_twiddles(a.twr, a.twc, bw, bh, twr, twc);
  const int b = blockIdx.x;
  int bx, by, par;
  block_origin(a.g, b, bx, by, par);
  const bool inside = bx >= 0 && by >= 0 && bx + bw <= a.g.W && by + bh <= a.g.H;
  float2* out = a.spec + (size_t)b * bh * fbw;
  __syncthreads();
  for (int r = w; r < bh; r += kBigWarps) {
    const int y = inside ? by + r : mirror_i(by + r, a.g.H);
    const uint8_t* row = a.src + (long long)y * a.pitch;
    for (int x = lane; x < bw; x += 32) {
      const int sx = inside ? bx + x : mirror_i(bx + x, a.g.W);
      float v = load_sample(row, sx, a.fmt, a.norm);
      v -= a.chroma_norm;
      buf[bit_reverse_rt(x, lbw)] = make_float2(v * a.win[r * bw + x], 0.0f);
    }
    __syncwarp();
    fft_warp(buf, bw, twr, false, lane);
    for (int c = lane; c < fbw; c += 32) out[r * fbw + c] = buf[c];
    __syncwarp();
  }
  __syncthreads();  // the rows of every warp are in `out`
  for (int c = w; c < fbw; c += kBigWarps) {
    for (int r = lane; r < bh; r += 32) buf[bit_reverse_rt(r, lbh)] = out[r * fbw + c];
    __syncwarp();
    fft_warp(buf, bh, twc, false, lane);
    for (int r = lane; r < bh; r += 32) out[r * fbw + c] = buf[r];
    __syncwarp();
  }
}

// One block: temporal filter + sharpen per bin into the block's work area
// (bh x bw complex), Hermitian completion and column inverse transforms,
// row inverse transforms, real part times the synthesis window
// (src/cpu/reference.cpp:246-430, src/cpu/fft.cpp:88-119).
__global__ void __launch_bounds__(kBigThreads) k_inverse_big(const __grid_constant__ InvArgs a) {
  extern __shared__ float2 sm_big[];
  const int bw = a.g.bw, bh = a.g.bh, fbw = bw / 2 + 1, ps = fbw * bh;
  const int lbw = log2_int(bw), lbh = log2_int(bh);
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  float2* buf = sm_big + w * kBigMax;
  float2* twr = sm_big + kBigWarps * kBigMax;
  float2* twc = twr + kBigMax / 2;
  load_twiddles(a.twr, a.twc, bw, bh, twr, twc);
  const int b = blockIdx.x;
  float2* F = a.work + (size_t)b * bh * bw;
  const size_t base = (size_t)b * ps;
  for (int i = threadIdx.x; i < ps; i += kBigThreads) {
    const int r = i / fbw, c = i - r * fbw;
    F[r * bw + c] = filter_bin(a, b, i, base + i);
  }
  __syncthreads();
  // Columns fbw..bw-1 first: each is the conjugate mirror of a column
  // 1..bw/2-1, read before those columns are transformed in place.
  for (int c = fbw + w; c < bw; c += kBigWarps) {
    for (int r = lane; r < bh; r += 32) {
      const float2 m = F[((bh - r) % bh) * bw + (bw - c)];
      buf[bit_reverse_rt(r, lbh)] = make_float2(m.x, -m.y);
    }
    __syncwarp();
    fft_warp(buf, bh, twc, true, lane);
    for (int r = lane; r < bh; r += 32) F[r * bw + c] = buf[r];
    __syncwarp();
  }
  __syncthreads();
  for (int c = w; c < fbw; c += kBigWarps) {
    for (int r = lane; r < bh; r += 32) buf[bit_reverse_rt(r, lbh)] = F[r * bw + c];
    __syncwarp();
    fft_warp(buf, bh, twc, true, lane);
    for (int r = lane; r < bh; r += 32) F[r * bw + c] = buf[r];
    __syncwarp();
  }
  __syncthreads();
  int bx, by, par;
  block_origin(a.g, b, bx, by, par);
  const float* win = par ? a.win_b : a.win_a;
  float* out = a.blocks + (size_t)b * bw * bh;
  for (int r = w; r < bh; r += kBigWarps) {
    for (int x = lane; x < bw; x += 32) buf[bit_reverse_rt(x, lbw)] = F[r * bw + x];
    __syncwarp();
    fft_warp(buf, bw, twr, true, lane);
    for (int x = lane; x < bw; x += 32) out[r * bw + x] = buf[x].x * win[r * bw + x];
    __syncwarp();
  }
}

constexpr size_t kBigSmem = sizeof(float2) * (kBigWarps * kBigMax + kBigMax);

}  // namespace

bool big_block(int bw, int bh) { return bw > 64 || bh > 64; }

cudaError_t launch_forward_big(const FwdArgs& a, cudaStream_t st) {
  if (a.g.bw > kBigMax || a.g.bh > kBigMax || !a.twr || !a.twc) return cudaErrorInvalidValue;
  if (a.g.nb == 0) return cudaSuccess;
  k_forward_big<<<a.g.nb, kBigThreads, kBigSmem, st>>>(a);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_inverse_big(const InvArgs& a, cudaStream_t st) {
  if (a.g.bw > kBigMax || a.g.bh > kBigMax || !a.twr || !a.twc || !a.work) return cudaErrorInvalidValue;
  if (a.g.nb == 0) return cudaSuccess;
  k_inverse_big<<<a.g.nb, kBigThreads, kBigSmem, st>>>(a);
  count_launch();
  return cudaGetLastError();
}

}  // namespace f3d
