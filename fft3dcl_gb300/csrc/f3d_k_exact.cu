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
    for (int i = t; i < C::PS; i += C::TPB) F[i] = filter_bin(a, b, i, base + i);
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

template <int BW, int BH>
cudaError_t launch_fwd(const FwdArgs& a, cudaStream_t st) {
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

template <int BW, int BH>
cudaError_t launch_inv(const InvArgs& a, cudaStream_t st) {
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
