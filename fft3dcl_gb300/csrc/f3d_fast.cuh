// f3d_fast.cuh -- building blocks of the fast form (packed real transforms
// in registers with FMA), shared by the per-block kernels (f3d_k_fast.cu)
// and the fused sweep kernel (f3d_k_sweep.cu).
//
// Spectra in HBM use the exact form's layout, float2 [nb][bh][fbw]: a thread
// that owns column c reads (r, c) while its neighbours read (r, c+1), so every
// warp access is contiguous. Transposes go through shared memory as
// column-major [fbw][bh+2] float2 tiles read and written 16 bytes at a time,
// which is free of bank conflicts.
#pragma once

#include "f3d_device.cuh"

// Unroll factor of the per-bin filter loop (pairs of bins): more bins'
// loads in flight against more registers.
#ifndef F3D_FILTER_UNROLL
#define F3D_FILTER_UNROLL 2
#endif
#define F3D_PRAGMA(x) _Pragma(#x)
#define F3D_UNROLL(n) F3D_PRAGMA(unroll n)

namespace f3d {

// Radix-2 DIT with FMA: twiddles (1,0) and (0,-1) (j = 0 and j = N/4) are
// applied without multiplications. Unnormalised in both directions. `tw`
// holds exp(-2 pi i k / (N*TWS)), read with stride TWS.
template <int N, int LEN, bool INV, int TWS = 1>
__device__ __forceinline__ void fft_fast_stage(float2 (&a)[N], const float2* tw) {
  constexpr int half = LEN / 2, step = N / LEN * TWS;
#pragma unroll
  for (int i = 0; i < N; i += LEN) {
#pragma unroll
    for (int j = 0; j < half; j++) {
      const float2 b = a[i + j + half];
      float2 t;
      if (j == 0) {
        t = b;
      } else if (j * step == N * TWS / 4) {
        t = INV ? make_float2(-b.y, b.x) : make_float2(b.y, -b.x);
      } else {
        const float2 w = tw[j * step];
        const float wy = INV ? -w.y : w.y;
        t.x = fmaf(w.x, b.x, -wy * b.y);
        t.y = fmaf(w.x, b.y, wy * b.x);
      }
      const float2 u = a[i + j];
      a[i + j] = make_float2(u.x + t.x, u.y + t.y);
      a[i + j + half] = make_float2(u.x - t.x, u.y - t.y);
    }
  }
  if constexpr (LEN < N) fft_fast_stage<N, LEN * 2, INV, TWS>(a, tw);
}

template <int N, bool INV, int TWS = 1>
__device__ __forceinline__ void fft_fast(float2 (&a)[N], const float2* tw) {
  constexpr int L = Log2<N>::v;
#pragma unroll
  for (int i = 0; i < N; i++) {
    const int r = bit_reverse(i, L);
    if (i < r) {
      const float2 t = a[i];
      a[i] = a[r];
      a[r] = t;
    }
  }
  fft_fast_stage<N, 2, INV, TWS>(a, tw);
}

template <int BW, int BH>
struct FCfg {
  static constexpr int FBW = BW / 2 + 1;
  static constexpr int NY = BW / 2;                      // Nyquist column
  static constexpr int PS = FBW * BH;
  static constexpr int TPB = (BW > BH ? BW : BH) / 2;    // <= 32: a block lives in one warp
  static constexpr int SB = BH + 2;                      // column stride of the transpose tile
  static constexpr int TS = BW + 1;                      // row stride of the input tile (floats)
  static constexpr int TILE_F2 = FBW * SB;               // transpose tile, float2
  static constexpr int IN_F2 = (BH * TS + 1) / 2;        // input tile, in float2 units
  static constexpr int SMEM_F2 = TILE_F2 > IN_F2 ? TILE_F2 : IN_F2;
};

// Column c, rows y and y+1 of a transpose tile, as one 16-byte access.
template <int SB>
__device__ __forceinline__ float4& tile_pair(float2* S, int c, int y) {
  return *reinterpret_cast<float4*>(S + c * SB + y);
}

// Tile position of row y of an inverted column: the column inverse runs as
// two half-length inverses over the even and odd inputs, and its outputs y
// and y + BH/2 land at positions 2y and 2y+1.
template <int BH>
__device__ __forceinline__ int yperm(int y) {
  return y < BH / 2 ? 2 * y : 2 * (y - BH / 2) + 1;
}

// Filter and invert block b. The TPB threads of the block (t = 0..TPB-1, all
// in one warp, all calling) share the transpose tile S. Thread t filters
// column t and a share of the Nyquist column, inverts column t (thread 0:
// columns 0 and bw/2 packed, from their Hermitian parts, which is what the
// real part of the reference's full complex inverse keeps), then inverts
// rows 2t and 2t+1, one after the other, each as a bw/2-point complex FFT of
// its even and odd samples. For each row y it calls emit(y, xy) with
// xy[n] = (x[2n], x[2n+1]), the unnormalised inverse (scale by 1/(bw*bh)).
// Row y's entries of the tile are S[c*SB + yperm(y)]. When emit runs, the
// thread has read everything it needs of them and no other thread touches
// them, so emit may store the row there (in pairs) without synchronisation.
// filtered() runs once the block's spectra have all been read.
template <int BW, int BH, int BM, class Emit, class Filtered>
__device__ __forceinline__ void inverse_block(const InvArgs& a, int b, int t, bool valid, float2* S,
                                              Emit&& emit, Filtered&& filtered) {
  using C = FCfg<BW, BH>;
  const size_t base = (size_t)b * C::PS;
  const bool cols = valid && t < C::NY;
  // Filter into the tile (two bins per 16-byte store); a partly unrolled loop
  // keeps a few bins' loads in flight without holding the column in registers.
  if (cols) {
    const float dc = block_dc(a, b);
    F3D_UNROLL(F3D_FILTER_UNROLL)
    for (int r = 0; r < BH; r += 2) {
      const float2 f0 = filter_bin_t<BM, true>(a, dc, r * C::FBW + t, base + r * C::FBW + t);
      const float2 f1 = filter_bin_t<BM, true>(a, dc, (r + 1) * C::FBW + t, base + (r + 1) * C::FBW + t);
      tile_pair<C::SB>(S, t, r) = make_float4(f0.x, f0.y, f1.x, f1.y);
    }
    for (int r = t; r < BH; r += C::NY)
      S[C::NY * C::SB + r] = filter_bin_t<BM, true>(a, dc, r * C::FBW + C::NY, base + r * C::FBW + C::NY);
  }
  filtered();
  __syncwarp();
  if (cols) {
    float2* col = S + t * C::SB;  // this thread's column; no other thread touches it now
    if (t == 0) {
      // Hermitian parts of columns 0 and bw/2, packed as F0 + i F_ny into
      // column 0; rows r and m = -r together (the part at m is the
      // conjugate of the one at r).
#pragma unroll
      for (int r = 0; r <= BH / 2; r++) {
        const int m = (BH - r) % BH;
        const float2 zr = col[r], zm = col[m];
        const float2 nr = S[C::NY * C::SB + r], nm = S[C::NY * C::SB + m];
        const float ar = 0.5f * (zr.x + zm.x), ai = 0.5f * (zr.y - zm.y);
        const float qr = 0.5f * (nr.x + nm.x), qi = 0.5f * (nr.y - nm.y);
        col[r] = make_float2(ar - qi, ai + qr);
        if (m != r) col[m] = make_float2(ar + qi, qr - ai);
      }
    }
    // Inverse of the column as two half-length inverses: E over the even
    // inputs (kept in the even slots), O over the odd ones, then
    // x[y] = E[y] + w^y O[y] at slot 2y, x[y + BH/2] = E[y] - w^y O[y] at
    // slot 2y+1 (w = e^{+2 pi i/BH}); see yperm.
    constexpr int H = BH / 2;
    {
      float2 e[H];
#pragma unroll
      for (int j = 0; j < H; j++) e[j] = col[2 * j];
      fft_fast<H, true, 2>(e, a.tw.col);
#pragma unroll
      for (int j = 0; j < H; j++) col[2 * j] = e[j];
    }
    float2 o[H];
#pragma unroll
    for (int j = 0; j < H; j++) o[j] = col[2 * j + 1];
    fft_fast<H, true, 2>(o, a.tw.col);
#pragma unroll
    for (int y = 0; y < H; y++) {
      const float2 e = col[2 * y];
      const float2 w = a.tw.col[y];  // e^{-2 pi i y/BH}; the conjugate is used
      const float px = fmaf(o[y].x, w.x, o[y].y * w.y), py = fmaf(o[y].y, w.x, -o[y].x * w.y);
      col[2 * y] = make_float2(e.x + px, e.y + py);
      col[2 * y + 1] = make_float2(e.x - px, e.y - py);
    }
    if (t == 0) {  // real inverses of columns 0 and bw/2
#pragma unroll
      for (int p = 0; p < BH; p++) {
        const float2 v = col[p];
        col[p] = make_float2(v.x, 0.0f);
        S[C::NY * C::SB + p] = make_float2(v.y, 0.0f);
      }
    }
  }
  __syncwarp();
  if (valid && t < BH / 2) {
    constexpr int M = BW / 2;
#pragma unroll
    for (int q = 0; q < 2; q++) {
      // Real row y from its half spectrum Y[0..M] (Y[0], Y[M] real): with
      // A = Y[k] + conj Y[M-k], B = (Y[k] - conj Y[M-k]) e^{+2 pi i k/bw},
      // the M-point inverse of A + iB is x[2n] + i x[2n+1].
      const int y = 2 * t + q, yp = yperm<BH>(y);
      float2 z2[M];
#pragma unroll
      for (int k = 0; k < M; k++) {
        const float2 yk = S[k * C::SB + yp], ym = S[(M - k) * C::SB + yp];
        const float ax = yk.x + ym.x, ay = yk.y - ym.y;
        const float bx = yk.x - ym.x, by = yk.y + ym.y;
        const float2 w = a.tw.row[k];  // e^{-2 pi i k/bw}; the conjugate is used
        const float px = fmaf(bx, w.x, by * w.y), py = fmaf(by, w.x, -bx * w.y);
        z2[k] = make_float2(ax - py, ay + px);
      }
      fft_fast<M, true, 2>(z2, a.tw.row);
      emit(y, z2);
    }
  }
  __syncwarp();  // S may be reused by the caller from here on
}

// Square blocks (N = 8, 16, 32): the same filter and inverse with N threads
// per block (one warp or part of one), so that each thread holds half as
// much and more warps fit on an SM.
//   filter   thread t = (c, h), c = t mod N/2, h = t div N/2: column c, rows
//            h*N/2 .. h*N/2 + N/2 - 1, and Nyquist row t;
//   columns  the pair (c, 0), (c, 1) inverts column c: the even inputs on
//            h = 0, the odd ones on h = 1, combined through a shuffle; the
//            Hermitian parts of columns 0 and N/2 are packed into column 0
//            first (thread r <= N/2 does rows r and -r);
//   rows     thread t inverts row t as an N/2-point complex FFT.
// Tile positions, emit and filtered() are those of inverse_block.
template <int N, int BM, class Emit, class Filtered>
__device__ __forceinline__ void inverse_block_sq(const InvArgs& a, int b, int t, bool valid, float2* S,
                                                 Emit&& emit, Filtered&& filtered) {
  using C = FCfg<N, N>;
  constexpr int NY = N / 2, H = N / 2, SB = C::SB, FBW = C::FBW;
  const size_t base = (size_t)b * C::PS;
  const int c = t % NY, h = t / NY;
  if (valid) {
    const float dc = block_dc(a, b);
    F3D_UNROLL(F3D_FILTER_UNROLL)
    for (int k = 0; k < H; k += 2) {
      const int r = h * H + k;
      const float2 f0 = filter_bin_t<BM, true>(a, dc, r * FBW + c, base + r * FBW + c);
      const float2 f1 = filter_bin_t<BM, true>(a, dc, (r + 1) * FBW + c, base + (r + 1) * FBW + c);
      tile_pair<SB>(S, c, r) = make_float4(f0.x, f0.y, f1.x, f1.y);
    }
    S[NY * SB + t] = filter_bin_t<BM, true>(a, dc, t * FBW + NY, base + t * FBW + NY);
  }
  filtered();
  __syncwarp();
  if (valid && t <= N / 2) {  // Hermitian parts of columns 0 and N/2, packed into column 0
    const int r = t, m = (N - t) % N;
    const float2 zr = S[r], zm = S[m];
    const float2 nr = S[NY * SB + r], nm = S[NY * SB + m];
    const float ar = 0.5f * (zr.x + zm.x), ai = 0.5f * (zr.y - zm.y);
    const float qr = 0.5f * (nr.x + nm.x), qi = 0.5f * (nr.y - nm.y);
    S[r] = make_float2(ar - qi, ai + qr);
    if (m != r) S[m] = make_float2(ar + qi, qr - ai);
  }
  __syncwarp();
  float2 e[H];
  if (valid) {
#pragma unroll
    for (int j = 0; j < H; j++) e[j] = S[c * SB + 2 * j + h];
    fft_fast<H, true, 2>(e, a.tw.col);
    if (h == 1) {
#pragma unroll
      for (int y = 0; y < H; y++) {  // e^{+2 pi i y/N} O[y]
        const float2 w = a.tw.col[y];
        e[y] = make_float2(fmaf(e[y].x, w.x, e[y].y * w.y), fmaf(e[y].y, w.x, -e[y].x * w.y));
      }
    }
  }
#pragma unroll
  for (int y = 0; y < H; y++) {
    const float ox = __shfl_xor_sync(0xffffffffu, e[y].x, NY);
    const float oy = __shfl_xor_sync(0xffffffffu, e[y].y, NY);
    // h = 0: x[y] = E + P at slot 2y; h = 1: x[y + N/2] = E - P at slot 2y+1
    const float2 x = h == 0 ? make_float2(e[y].x + ox, e[y].y + oy) : make_float2(ox - e[y].x, oy - e[y].y);
    if (valid) {
      if (c == 0) {  // real inverses of columns 0 and N/2
        S[2 * y + h] = make_float2(x.x, 0.0f);
        S[NY * SB + 2 * y + h] = make_float2(x.y, 0.0f);
      } else {
        S[c * SB + 2 * y + h] = x;
      }
    }
  }
  __syncwarp();
  if (valid) {
    const int yp = yperm<N>(t);
    float2 z2[H];
#pragma unroll
    for (int k = 0; k < H; k++) {
      const float2 yk = S[k * SB + yp], ym = S[(H - k) * SB + yp];
      const float ax = yk.x + ym.x, ay = yk.y - ym.y;
      const float bx = yk.x - ym.x, by = yk.y + ym.y;
      const float2 w = a.tw.row[k];
      const float px = fmaf(bx, w.x, by * w.y), py = fmaf(by, w.x, -bx * w.y);
      z2[k] = make_float2(ax - py, ay + px);
    }
    fft_fast<H, true, 2>(z2, a.tw.row);
    emit(t, z2);
  }
  __syncwarp();
}

// Bulk prefetch of `bytes` (a multiple of 16, 16-byte aligned) into L2.
__device__ __forceinline__ void prefetch_l2(const void* p, unsigned bytes) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(p), "r"(bytes) : "memory");
}

}  // namespace f3d
