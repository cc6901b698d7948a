// f3d_k_exact.cu -- exact-form kernels: the reference's radix-2 transforms in
// its own operation order, no fused multiply-add, so the engine's output has
// the same bits as the reference CPU backend.
//
// Compiled once per block width (-DF3D_BW=4|8|16|32|64) with --fmad=false;
// each object holds the kernels for every block height of that width.
//
// Thread mapping: TPB = max(bw, bh) threads own one block. The forward
// transform gives one thread per block row (row FFT held in registers), then
// one thread per kept column; the inverse one thread per column (Hermitian
// completion on the fly), then one thread per row. Shared memory carries the
// transposes; a CTA of 128 threads works on 128/TPB blocks.
// 64 x 64 blocks run their 64-point transforms on lane pairs instead
// (k_forward_exact64, k_inverse_exact64: 128 threads per block).
#include "f3d_device.cuh"

#ifndef F3D_BW
#error "F3D_BW must be defined"
#endif

namespace f3d {
namespace {

template <int BW, int BH>
struct Cfg {
  static constexpr int FBW = BW / 2 + 1;
  static constexpr int PS = FBW * BH;                 // bins per block
  static constexpr int TPB = BW > BH ? BW : BH;       // threads per block
  static constexpr int THREADS = TPB > 128 ? TPB : 128;
  static constexpr int BPC = THREADS / TPB;           // blocks per CTA
  static constexpr int TS = BW + 1;                   // padded row stride
  static constexpr int FWD_FLOATS = BH * TS + 2 * PS; // input tile + row spectra
  static constexpr int INV_FLOATS = 2 * PS + 2 * BH * TS;
  // Loads in flight per thread: the gather takes GB samples (and window
  // values) per round, the Kalman filter KB bins (spectrum, state, tables)
  // before any of their results is stored.
  static constexpr int GB = BW * BH / TPB < 16 ? BW * BH / TPB : 16;
  static constexpr int NJ = (PS + TPB - 1) / TPB;
  static constexpr int KB = NJ < 8 ? NJ : 8;
};

// One block: gather with mirror addressing, convert, subtract chroma
// centering, analysis window (src/cpu/reference.cpp:140-159); row FFTs then
// the fbw kept column FFTs (src/cpu/fft.cpp:68-86); store the half spectrum.
template <int BW, int BH>
__global__ void __launch_bounds__(Cfg<BW, BH>::THREADS)
    k_forward_exact(const __grid_constant__ FwdArgs a) {
  using C = Cfg<BW, BH>;
  extern __shared__ float4 smem4[];
  float* smem = reinterpret_cast<float*>(smem4);
  const int slot = threadIdx.x / C::TPB, t = threadIdx.x - slot * C::TPB;
  const int b = blockIdx.x * C::BPC + slot;
  const bool valid = b < a.g.nb;
  float* tile = smem + slot * C::FWD_FLOATS;
  float2* rows = reinterpret_cast<float2*>(tile + BH * C::TS);

  if (valid) {
    int bx, by, par;
    block_origin(a.g, b, bx, by, par);
    const bool inside = bx >= 0 && by >= 0 && bx + BW <= a.g.W && by + BH <= a.g.H;
    for (int i0 = 0; i0 < BW * BH; i0 += C::GB * C::TPB) {
      float v[C::GB], w[C::GB];
#pragma unroll
      for (int u = 0; u < C::GB; u++) {
        const int idx = i0 + t + u * C::TPB;
        if (idx >= BW * BH) continue;
        const int ly = idx / BW, lx = idx - ly * BW;
        const int y = inside ? by + ly : mirror_i(by + ly, a.g.H);
        const int x = inside ? bx + lx : mirror_i(bx + lx, a.g.W);
        v[u] = load_sample(a.src + (long long)y * a.pitch, x, a.fmt, a.norm);
        w[u] = a.win[idx];
      }
#pragma unroll
      for (int u = 0; u < C::GB; u++) {
        const int idx = i0 + t + u * C::TPB;
        if (idx >= BW * BH) continue;
        const int ly = idx / BW, lx = idx - ly * BW;
        const float c = v[u] - a.chroma_norm;
        tile[ly * C::TS + lx] = c * w[u];
      }
    }
  }
  __syncthreads();
  if (valid) {
    for (int r = t; r < BH; r += C::TPB) {
      float2 v[BW];
#pragma unroll
      for (int c = 0; c < BW; c++) v[c] = make_float2(tile[r * C::TS + c], 0.0f);
      fft_r2<BW, false>(v, a.tw.row);
#pragma unroll
      for (int c = 0; c < C::FBW; c++) rows[r * C::FBW + c] = v[c];
    }
  }
  __syncthreads();
  if (valid) {
    float2* out = a.spec + (size_t)b * C::PS;
    for (int c = t; c < C::FBW; c += C::TPB) {
      float2 v[BH];
#pragma unroll
      for (int r = 0; r < BH; r++) v[r] = rows[r * C::FBW + c];
      fft_r2<BH, false>(v, a.tw.col);
#pragma unroll
      for (int r = 0; r < BH; r++) out[r * C::FBW + c] = v[r];
    }
  }
}

// One block: temporal filter + sharpen per bin, Hermitian completion and
// column inverse FFTs, row inverse FFTs, real part times the synthesis
// window (src/cpu/reference.cpp:246-430, src/cpu/fft.cpp:88-119). KALMAN:
// the Kalman filter (bm 0), whose state loads of KB bins are issued before
// their updates are stored (the compiler cannot move a bin's loads above the
// previous bin's state stores); the other modes read bm at run time.
template <int BW, int BH, bool KALMAN>
__global__ void __launch_bounds__(Cfg<BW, BH>::THREADS)
    k_inverse_exact(const __grid_constant__ InvArgs a) {
  using C = Cfg<BW, BH>;
  extern __shared__ float4 smem4[];
  float* smem = reinterpret_cast<float*>(smem4);
  const int slot = threadIdx.x / C::TPB, t = threadIdx.x - slot * C::TPB;
  const int b = blockIdx.x * C::BPC + slot;
  const bool valid = b < a.g.nb;
  float2* F = reinterpret_cast<float2*>(smem + slot * C::INV_FLOATS);
  float2* G = F + C::PS;

  if (valid && KALMAN) {
    const size_t base = (size_t)b * C::PS;
    const float dc = block_dc(a, b);
    for (int j0 = 0; j0 < C::NJ; j0 += C::KB) {
      float2 sv[C::KB][4];
      KState ks[C::KB];
      BinTables tb[C::KB];
#pragma unroll
      for (int u = 0; u < C::KB; u++) {
        const int i = t + (j0 + u) * C::TPB;
        if (j0 + u >= C::NJ || i >= C::PS) continue;
        load_window<0>(a, base + i, sv[u]);
        ks[u] = load_kstate(a, base + i);
        tb[u] = bin_tables(a, i);
      }
#pragma unroll
      for (int u = 0; u < C::KB; u++) {
        const int i = t + (j0 + u) * C::TPB;
        if (j0 + u >= C::NJ || i >= C::PS) continue;
        F[i] = filter_vals_ks<0>(a, dc, tb[u], base + i, sv[u], ks[u]);
      }
    }
  } else if (valid) {
    const size_t base = (size_t)b * C::PS;
    const float dc = block_dc(a, b);
    const KState none{make_float2(0.0f, 0.0f), 0.0f, 0.0f};
    constexpr int KN = 4;  // bins whose window spectra are loaded together
    for (int j0 = 0; j0 < C::NJ; j0 += KN) {
      float2 sv[KN][4];
#pragma unroll
      for (int u = 0; u < KN; u++) {
        const int i = t + (j0 + u) * C::TPB;
        if (j0 + u < C::NJ && i < C::PS) load_window<kRuntimeBm>(a, base + i, sv[u]);
      }
#pragma unroll
      for (int u = 0; u < KN; u++) {
        const int i = t + (j0 + u) * C::TPB;
        if (j0 + u >= C::NJ || i >= C::PS) continue;
        F[i] = filter_vals_ks<kRuntimeBm>(a, dc, bin_tables(a, i), base + i, sv[u], none);
      }
    }
  }
  __syncthreads();
  if (valid) {
    for (int c = t; c < BW; c += C::TPB) {
      float2 v[BH];
#pragma unroll
      for (int r = 0; r < BH; r++) {
        if (c < C::FBW) {
          v[r] = F[r * C::FBW + c];
        } else {
          const float2 m = F[((BH - r) % BH) * C::FBW + (BW - c)];
          v[r] = make_float2(m.x, -m.y);
        }
      }
      fft_r2<BH, true>(v, a.tw.col);
#pragma unroll
      for (int r = 0; r < BH; r++) G[r * C::TS + c] = v[r];
    }
  }
  __syncthreads();
  if (valid) {
    int bx, by, par;
    block_origin(a.g, b, bx, by, par);
    const float* win = par ? a.win_b : a.win_a;
    float* out = a.blocks + (size_t)b * BW * BH;
    for (int r = t; r < BH; r += C::TPB) {
      float2 v[BW];
#pragma unroll
      for (int c = 0; c < BW; c++) v[c] = G[r * C::TS + c];
      fft_r2<BW, true>(v, a.tw.row);
#pragma unroll
      for (int c = 0; c < BW; c++) out[r * BW + c] = v[c].x * win[r * BW + c];
    }
  }
}

// ---- 64 x 64 blocks: each 64-point transform on a lane pair ----------------
//
// One thread per 64-point transform holds 128 registers of data and leaves
// 504 CTAs of two 720p blocks in two waves; a lane pair (lanes 2i, 2i+1)
// halves both. The bit-reversed array is split in halves: the even lane
// holds positions 0..31, the odd lane 32..63. Stages len = 2..32 stay inside
// a half (twiddles tw[j * 64 / len], as in the whole transform); the last
// stage pairs position j with j + 32: the odd lane forms t = w_j * a[j + 32],
// the lanes swap t and u = a[j] by one shuffle, and each forms its output,
// u + t or u - t. Every value is computed by the same operations as in
// fft_r2<64> (src/cpu/fft.cpp:28-58), so the bits are the same.

template <int LEN, bool INV>
__device__ __forceinline__ void half_stage64(float2 (&a)[32], const float2* tw) {
  constexpr int half = LEN / 2, step = 64 / LEN;
#pragma unroll
  for (int i = 0; i < 32; i += LEN) {
#pragma unroll
    for (int j = 0; j < half; j++) {
      const float2 b = a[i + j + half];
      float2 t;
      if (j == 0) {
        t = b;
      } else {
        const float2 w = tw[j * step];
        const float wy = INV ? -w.y : w.y;
        t.x = w.x * b.x - wy * b.y;
        t.y = w.x * b.y + wy * b.x;
      }
      const float2 u = a[i + j];
      a[i + j] = make_float2(u.x + t.x, u.y + t.y);
      a[i + j + half] = make_float2(u.x - t.x, u.y - t.y);
    }
  }
  if constexpr (LEN < 32) half_stage64<LEN * 2, INV>(a, tw);
}

// a: positions 32 * odd + p (p < 32) of the bit-reversed input; out: the
// transform's values 32 * odd + p. Every lane of the warp takes part.
template <bool INV>
__device__ __forceinline__ void fft64_pair(float2 (&a)[32], const float2* tw, bool odd) {
  half_stage64<2, INV>(a, tw);
#pragma unroll
  for (int j = 0; j < 32; j++) {
    const float2 x = a[j];
    float2 t = x;
    if (j > 0) {
      const float2 w = tw[j];
      const float wy = INV ? -w.y : w.y;
      t.x = w.x * x.x - wy * x.y;
      t.y = w.x * x.y + wy * x.x;
    }
    const float2 send = odd ? t : x;
    const float rx = __shfl_xor_sync(0xffffffffu, send.x, 1), ry = __shfl_xor_sync(0xffffffffu, send.y, 1);
    a[j] = odd ? make_float2(rx - t.x, ry - t.y) : make_float2(x.x + rx, x.y + ry);
  }
  if (INV) {
    const float invn = 1.0f / 64;
#pragma unroll
    for (int i = 0; i < 32; i++) a[i] = make_float2(a[i].x * invn, a[i].y * invn);
  }
}

constexpr int kPairThreads = 128;  // one 64 x 64 block per CTA
constexpr int kPairTS = 65;        // padded row stride (float or float2)

// Forward of one 64 x 64 block per CTA: gather, row transforms (pair p =
// row p), then the 33 kept columns (pair p = column p). The input tile and
// the row spectra share shared memory: every row is in registers before any
// row spectrum is written.
__global__ void __launch_bounds__(kPairThreads) k_forward_exact64(const __grid_constant__ FwdArgs a) {
  constexpr int FBW = 33;
  extern __shared__ float4 smem4[];
  float* tile = reinterpret_cast<float*>(smem4);    // [64][kPairTS]
  float2* rows = reinterpret_cast<float2*>(smem4);  // [64][FBW], after the row transforms
  const int t = threadIdx.x, p = t >> 1;
  const bool odd = t & 1;
  const int b = blockIdx.x;
  int bx, by, par;
  block_origin(a.g, b, bx, by, par);
  const bool inside = bx >= 0 && by >= 0 && bx + 64 <= a.g.W && by + 64 <= a.g.H;
  constexpr int GB = 16;
  for (int i0 = 0; i0 < 64 * 64; i0 += GB * kPairThreads) {
    float v[GB], w[GB];
#pragma unroll
    for (int u = 0; u < GB; u++) {
      const int idx = i0 + t + u * kPairThreads;
      const int ly = idx >> 6, lx = idx & 63;
      const int y = inside ? by + ly : mirror_i(by + ly, a.g.H);
      const int x = inside ? bx + lx : mirror_i(bx + lx, a.g.W);
      v[u] = load_sample(a.src + (long long)y * a.pitch, x, a.fmt, a.norm);
      w[u] = a.win[idx];
    }
#pragma unroll
    for (int u = 0; u < GB; u++) {
      const int idx = i0 + t + u * kPairThreads;
      const float c = v[u] - a.chroma_norm;
      tile[(idx >> 6) * kPairTS + (idx & 63)] = c * w[u];
    }
  }
  __syncthreads();
  float2 r[32];
#pragma unroll
  for (int q = 0; q < 32; q++) r[q] = make_float2(tile[p * kPairTS + bit_reverse(q, 6) + odd], 0.0f);
  __syncthreads();  // the tile is read: the row spectra may overwrite it
  fft64_pair<false>(r, a.tw.row, odd);
  if (!odd) {
#pragma unroll
    for (int c = 0; c < 32; c++) rows[p * FBW + c] = r[c];
  } else {
    rows[p * FBW + 32] = r[0];
  }
  __syncthreads();
  if (t < 2 * 48) {  // warps holding columns 0..32 (lanes of columns 33.. run along, store nothing)
    const int c = p < FBW ? p : 0;
#pragma unroll
    for (int q = 0; q < 32; q++) r[q] = rows[(bit_reverse(q, 6) + odd) * FBW + c];
    fft64_pair<false>(r, a.tw.col, odd);
    if (p < FBW) {
      float2* out = a.spec + (size_t)b * 64 * FBW + c;
#pragma unroll
      for (int q = 0; q < 32; q++) out[(32 * odd + q) * FBW] = r[q];
    }
  }
}

// Filter + inverse of one 64 x 64 block per CTA: the filtered half spectrum
// F, column transforms (pair p = column p, Hermitian completion on the fly)
// into G, which shares F's space once every column is in registers, then
// row transforms (pair p = row p) times the synthesis window.
template <bool KALMAN>
__global__ void __launch_bounds__(kPairThreads) k_inverse_exact64(const __grid_constant__ InvArgs a) {
  constexpr int FBW = 33, PS = 64 * FBW;
  extern __shared__ float4 smem4[];
  float2* F = reinterpret_cast<float2*>(smem4);  // [64][FBW]
  float2* G = F;                                 // [64][kPairTS], after the column reads
  const int t = threadIdx.x, p = t >> 1;
  const bool odd = t & 1;
  const int b = blockIdx.x;
  const size_t base = (size_t)b * PS;
  if (KALMAN) {
    const float dc = block_dc(a, b);
    constexpr int NJ = (PS + kPairThreads - 1) / kPairThreads, KB = 8;
    for (int j0 = 0; j0 < NJ; j0 += KB) {
      float2 sv[KB][4];
      KState ks[KB];
      BinTables tb[KB];
#pragma unroll
      for (int u = 0; u < KB; u++) {
        const int i = t + (j0 + u) * kPairThreads;
        if (j0 + u >= NJ || i >= PS) continue;
        load_window<0>(a, base + i, sv[u]);
        ks[u] = load_kstate(a, base + i);
        tb[u] = bin_tables(a, i);
      }
#pragma unroll
      for (int u = 0; u < KB; u++) {
        const int i = t + (j0 + u) * kPairThreads;
        if (j0 + u >= NJ || i >= PS) continue;
        F[i] = filter_vals_ks<0>(a, dc, tb[u], base + i, sv[u], ks[u]);
      }
    }
  } else {
    for (int i = t; i < PS; i += kPairThreads) F[i] = filter_bin(a, b, i, base + i);
  }
  __syncthreads();
  float2 r[32];
  {
    const int c = p;
#pragma unroll
    for (int q = 0; q < 32; q++) {
      const int row = bit_reverse(q, 6) + odd;
      if (c < FBW) {
        r[q] = F[row * FBW + c];
      } else {
        const float2 m = F[((64 - row) & 63) * FBW + (64 - c)];
        r[q] = make_float2(m.x, -m.y);
      }
    }
  }
  __syncthreads();  // F is read: G may overwrite it
  fft64_pair<true>(r, a.tw.col, odd);
#pragma unroll
  for (int q = 0; q < 32; q++) G[(32 * odd + q) * kPairTS + p] = r[q];
  __syncthreads();
#pragma unroll
  for (int q = 0; q < 32; q++) r[q] = G[p * kPairTS + bit_reverse(q, 6) + odd];
  fft64_pair<true>(r, a.tw.row, odd);
  int bx, by, par;
  block_origin(a.g, b, bx, by, par);
  const float* win = (par ? a.win_b : a.win_a) + p * 64 + 32 * odd;
  float* out = a.blocks + (size_t)b * 64 * 64 + p * 64 + 32 * odd;
#pragma unroll
  for (int q = 0; q < 32; q++) out[q] = r[q].x * win[q];
}

cudaError_t launch_fwd64(const FwdArgs& a, cudaStream_t st) {
  const size_t smem = sizeof(float2) * 64 * 33 > sizeof(float) * 64 * kPairTS ? sizeof(float2) * 64 * 33
                                                                               : sizeof(float) * 64 * kPairTS;
  if (a.g.nb == 0) return cudaSuccess;
  k_forward_exact64<<<a.g.nb, kPairThreads, smem, st>>>(a);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_inv64(const InvArgs& a, cudaStream_t st) {
  const size_t smem = sizeof(float2) * 64 * kPairTS;  // G, which covers F
  auto k = a.bm == 0 ? k_inverse_exact64<true> : k_inverse_exact64<false>;
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  if (a.g.nb == 0) return cudaSuccess;
  k<<<a.g.nb, kPairThreads, smem, st>>>(a);
  count_launch();
  return cudaGetLastError();
}

template <int BW, int BH>
cudaError_t launch_fwd(const FwdArgs& a, cudaStream_t st) {
  if constexpr (BW == 64 && BH == 64) {
    return launch_fwd64(a, st);
  } else {
    using C = Cfg<BW, BH>;
    const size_t smem = sizeof(float) * C::FWD_FLOATS * C::BPC;
    auto k = k_forward_exact<BW, BH>;
    if (smem > 48 * 1024) {
      cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e != cudaSuccess) return e;
    }
    const int grid = (a.g.nb + C::BPC - 1) / C::BPC;
    if (grid == 0) return cudaSuccess;
    k<<<grid, C::THREADS, smem, st>>>(a);
    count_launch();
    return cudaGetLastError();
  }
}

template <int BW, int BH>
cudaError_t launch_inv(const InvArgs& a, cudaStream_t st) {
  if constexpr (BW == 64 && BH == 64) {
    return launch_inv64(a, st);
  } else {
    using C = Cfg<BW, BH>;
    const size_t smem = sizeof(float) * C::INV_FLOATS * C::BPC;
    auto k = a.bm == 0 ? k_inverse_exact<BW, BH, true> : k_inverse_exact<BW, BH, false>;
    if (smem > 48 * 1024) {
      cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e != cudaSuccess) return e;
    }
    const int grid = (a.g.nb + C::BPC - 1) / C::BPC;
    if (grid == 0) return cudaSuccess;
    k<<<grid, C::THREADS, smem, st>>>(a);
    count_launch();
    return cudaGetLastError();
  }
}

}  // namespace

#define F3D_CAT2(a, b) a##b
#define F3D_CAT(a, b) F3D_CAT2(a, b)

cudaError_t F3D_CAT(launch_forward_exact_bw, F3D_BW)(const FwdArgs& a, cudaStream_t st) {
  switch (a.g.bh) {
  case 4: return launch_fwd<F3D_BW, 4>(a, st);
  case 8: return launch_fwd<F3D_BW, 8>(a, st);
  case 16: return launch_fwd<F3D_BW, 16>(a, st);
  case 32: return launch_fwd<F3D_BW, 32>(a, st);
  case 64: return launch_fwd<F3D_BW, 64>(a, st);
  default: return cudaErrorInvalidValue;
  }
}

cudaError_t F3D_CAT(launch_inverse_exact_bw, F3D_BW)(const InvArgs& a, cudaStream_t st) {
  switch (a.g.bh) {
  case 4: return launch_inv<F3D_BW, 4>(a, st);
  case 8: return launch_inv<F3D_BW, 8>(a, st);
  case 16: return launch_inv<F3D_BW, 16>(a, st);
  case 32: return launch_inv<F3D_BW, 32>(a, st);
  case 64: return launch_inv<F3D_BW, 64>(a, st);
  default: return cudaErrorInvalidValue;
  }
}

}  // namespace f3d
