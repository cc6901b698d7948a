// f3d_k_fast.cu -- fast form: packed real transforms in registers with FMA.
//
// Compiled with --fmad=true -ftz=true -prec-div=false -prec-sqrt=false: the
// per-bin filter (the same source as the exact form, f3d_device.cuh) then
// uses the hardware reciprocal and square-root approximations. Results stay
// within the engine's tolerance of the reference (+-1 LSB at 8 bit, +-4 LSB
// at 10 bit, 1e-4 for float output) instead of matching it bit for bit.
//
// Layout and building blocks: f3d_fast.cuh.
//
// Per block TPB = max(bw, bh)/2 threads (16 for 32x32, half a warp):
//  forward  - the block is gathered cooperatively (vector loads where the
//             rows are aligned), converted and windowed into shared memory;
//             thread t transforms rows 2t and 2t+1 as one complex FFT and
//             splits the two half spectra; thread t then transforms column t,
//             thread 0 columns 0 and bw/2 together (both are real).
//  inverse  - thread t filters column t (and a share of column bw/2) and
//             inverse-transforms it; thread 0 inverts columns 0 and bw/2
//             together after taking their Hermitian parts, which is what the
//             real part of the reference's full complex inverse keeps; thread t
//             then inverts rows 2t and 2t+1 from their Hermitian halves as one
//             complex FFT whose real and imaginary parts are the two rows.
#include "f3d_fast.cuh"

namespace f3d {
namespace {

constexpr int kThreads = 128;

template <int BW, int BH>
__global__ void __launch_bounds__(128) k_forward_fast(const __grid_constant__ FwdArgs a) {
  using C = FCfg<BW, BH>;
  constexpr int BPC = kThreads / C::TPB;
  extern __shared__ float4 smem4[];
  const int slot = threadIdx.x / C::TPB, t = threadIdx.x - slot * C::TPB;
  const int b = blockIdx.x * BPC + slot;
  const bool valid = b < a.g.nb;
  float2* S = reinterpret_cast<float2*>(smem4) + slot * C::SMEM_F2;
  float* tile = reinterpret_cast<float*>(S);  // input tile [BH][TS], aliased with S

  if (valid) {
    int bx, by, par;
    block_origin(a.g, b, bx, by, par);
    const bool inside = bx >= 0 && by >= 0 && bx + BW <= a.g.W && by + BH <= a.g.H;
    const int bps = a.fmt == FMT_U8 ? 1 : (a.fmt == FMT_U16 ? 2 : 4);
    const uintptr_t row0 = reinterpret_cast<uintptr_t>(a.src) + (long long)by * a.pitch + (long long)bx * bps;
    const bool vec = inside && ((row0 | (uintptr_t)a.pitch) & 15) == 0 && (BW * bps) % 16 == 0;
    if (vec) {
      // 16-byte loads: a row is BW*bps/16 chunks, the group covers them all.
      const int cpr = BW * bps / 16, spc = 16 / bps;
      for (int q = t; q < BH * cpr; q += C::TPB) {
        const int ly = q / cpr, ch = q - ly * cpr;
        const uint8_t* p = reinterpret_cast<const uint8_t*>(row0 + (long long)ly * a.pitch) + ch * 16;
        const uint4 u = *reinterpret_cast<const uint4*>(p);
        const uint32_t w4[4] = {u.x, u.y, u.z, u.w};
        float* dst = tile + ly * C::TS + ch * spc;
        const float* win = a.win + ly * BW + ch * spc;
        if (a.fmt == FMT_U8) {
#pragma unroll
          for (int k = 0; k < 16; k++)
            dst[k] = ((float)((w4[k >> 2] >> (8 * (k & 3))) & 0xffu) * (1.0f / 255.0f) - a.chroma_norm) * win[k];
        } else if (a.fmt == FMT_U16) {
#pragma unroll
          for (int k = 0; k < 8; k++)
            dst[k] = ((float)((w4[k >> 1] >> (16 * (k & 1))) & 0xffffu) * a.norm - a.chroma_norm) * win[k];
        } else {
#pragma unroll
          for (int k = 0; k < 4; k++) dst[k] = (__uint_as_float(w4[k]) - a.chroma_norm) * win[k];
        }
      }
    } else {
      for (int idx = t; idx < BW * BH; idx += C::TPB) {
        const int ly = idx / BW, lx = idx - ly * BW;
        const int y = inside ? by + ly : mirror_i(by + ly, a.g.H);
        const int x = inside ? bx + lx : mirror_i(bx + lx, a.g.W);
        tile[ly * C::TS + lx] =
            (load_sample(a.src + (long long)y * a.pitch, x, a.fmt, a.norm) - a.chroma_norm) * a.win[idx];
      }
    }
  }
  __syncwarp();
  float2 z[BW];
  const bool rows = valid && t < BH / 2;
  if (rows) {
#pragma unroll
    for (int c = 0; c < BW; c++) z[c] = make_float2(tile[(2 * t) * C::TS + c], tile[(2 * t + 1) * C::TS + c]);
  }
  __syncwarp();  // the tile is dead from here on; S reuses its storage
  if (rows) {
    fft_fast<BW, false>(z, a.tw.row);
    // Split Z = X_2t + i X_2t+1: X_2t[k] = (Z[k] + conj Z[-k])/2,
    // X_2t+1[k] = (Z[k] - conj Z[-k])/(2i).
#pragma unroll
    for (int k = 0; k <= C::NY; k++) {
      const float2 A = z[k], B = z[(BW - k) % BW];
      tile_pair<C::SB>(S, k, 2 * t) =
          make_float4(0.5f * (A.x + B.x), 0.5f * (A.y - B.y), 0.5f * (A.y + B.y), 0.5f * (B.x - A.x));
    }
  }
  __syncwarp();
  if (valid && t < C::NY) {
    float2 y[BH];
    if (t == 0) {  // columns 0 and bw/2 are real: transform them together
#pragma unroll
      for (int r = 0; r < BH; r += 2) {
        const float4 p0 = tile_pair<C::SB>(S, 0, r), pn = tile_pair<C::SB>(S, C::NY, r);
        y[r] = make_float2(p0.x, pn.x);
        y[r + 1] = make_float2(p0.z, pn.z);
      }
    } else {
#pragma unroll
      for (int r = 0; r < BH; r += 2) {
        const float4 p = tile_pair<C::SB>(S, t, r);
        y[r] = make_float2(p.x, p.y);
        y[r + 1] = make_float2(p.z, p.w);
      }
    }
    fft_fast<BH, false>(y, a.tw.col);
    float2* out = a.spec + (size_t)b * C::PS;
    if (t == 0) {
#pragma unroll
      for (int k = 0; k < BH; k++) {
        const float2 A = y[k], B = y[(BH - k) % BH];
        out[k * C::FBW] = make_float2(0.5f * (A.x + B.x), 0.5f * (A.y - B.y));
        out[k * C::FBW + C::NY] = make_float2(0.5f * (A.y + B.y), 0.5f * (B.x - A.x));
      }
    } else {
#pragma unroll
      for (int r = 0; r < BH; r++) out[r * C::FBW + t] = y[r];
    }
  }
}

template <int BW, int BH, int BM>
__global__ void __launch_bounds__(128) k_inverse_fast(const __grid_constant__ InvArgs a) {
  using C = FCfg<BW, BH>;
  constexpr int BPC = kThreads / C::TPB;
  extern __shared__ float4 smem4[];
  const int slot = threadIdx.x / C::TPB, t = threadIdx.x - slot * C::TPB;
  const int b = blockIdx.x * BPC + slot;
  const bool valid = b < a.g.nb;
  float2* S = reinterpret_cast<float2*>(smem4) + slot * C::SMEM_F2;
  int bx = 0, by = 0, par = 0;
  if (valid) block_origin(a.g, b, bx, by, par);
  const float* win = par ? a.win_b : a.win_a;
  float* out = a.blocks + (size_t)b * BW * BH;
  constexpr float inv_n = 1.0f / (BW * BH);
  inverse_block<BW, BH, BM>(a, b, t, valid, S, [&](int y, const float2(&xy)[BW / 2]) {
#pragma unroll
    for (int n = 0; n < BW / 2; n += 2) {
      const float4 wv = *reinterpret_cast<const float4*>(win + y * BW + 2 * n);
      *reinterpret_cast<float4*>(out + y * BW + 2 * n) =
          make_float4(xy[n].x * inv_n * wv.x, xy[n].y * inv_n * wv.y, xy[n + 1].x * inv_n * wv.z,
                      xy[n + 1].y * inv_n * wv.w);
    }
  }, [] {});
}

template <int BW, int BH>
cudaError_t launch_fwd(const FwdArgs& a, cudaStream_t st) {
  using C = FCfg<BW, BH>;
  constexpr int BPC = kThreads / C::TPB;
  const size_t smem = sizeof(float2) * C::SMEM_F2 * BPC;
  auto k = k_forward_fast<BW, BH>;
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  const int grid = (a.g.nb + BPC - 1) / BPC;
  if (grid == 0) return cudaSuccess;
  k<<<grid, kThreads, smem, st>>>(a);
  count_launch();
  return cudaGetLastError();
}

template <int BW, int BH, int BM>
cudaError_t launch_inv_bm(const InvArgs& a, cudaStream_t st) {
  using C = FCfg<BW, BH>;
  constexpr int BPC = kThreads / C::TPB;
  const size_t smem = sizeof(float2) * C::SMEM_F2 * BPC;
  auto k = k_inverse_fast<BW, BH, BM>;
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  const int grid = (a.g.nb + BPC - 1) / BPC;
  if (grid == 0) return cudaSuccess;
  k<<<grid, kThreads, smem, st>>>(a);
  count_launch();
  return cudaGetLastError();
}

template <int BW, int BH>
cudaError_t launch_inv(const InvArgs& a, cudaStream_t st) {
  switch (a.bm) {
  case -1: return launch_inv_bm<BW, BH, -1>(a, st);
  case 1: return launch_inv_bm<BW, BH, 1>(a, st);
  case 2: return launch_inv_bm<BW, BH, 2>(a, st);
  case 3: return launch_inv_bm<BW, BH, 3>(a, st);
  case 4: return launch_inv_bm<BW, BH, 4>(a, st);
  default: return cudaErrorNotSupported;  // Kalman runs the exact form
  }
}

template <int BW>
cudaError_t fwd_bh(const FwdArgs& a, cudaStream_t st) {
  switch (a.g.bh) {
  case 8: return launch_fwd<BW, 8>(a, st);
  case 16: return launch_fwd<BW, 16>(a, st);
  case 32: return launch_fwd<BW, 32>(a, st);
  case 64: return launch_fwd<BW, 64>(a, st);
  default: return cudaErrorInvalidValue;
  }
}

template <int BW>
cudaError_t inv_bh(const InvArgs& a, cudaStream_t st) {
  switch (a.g.bh) {
  case 8: return launch_inv<BW, 8>(a, st);
  case 16: return launch_inv<BW, 16>(a, st);
  case 32: return launch_inv<BW, 32>(a, st);
  case 64: return launch_inv<BW, 64>(a, st);
  default: return cudaErrorInvalidValue;
  }
}

}  // namespace

cudaError_t launch_forward_fast(const FwdArgs& a, cudaStream_t st) {
  switch (a.g.bw) {
  case 8: return fwd_bh<8>(a, st);
  case 16: return fwd_bh<16>(a, st);
  case 32: return fwd_bh<32>(a, st);
  case 64: return fwd_bh<64>(a, st);
  default: return cudaErrorInvalidValue;
  }
}

cudaError_t launch_inverse_fast(const InvArgs& a, cudaStream_t st) {
  switch (a.g.bw) {
  case 8: return inv_bh<8>(a, st);
  case 16: return inv_bh<16>(a, st);
  case 32: return inv_bh<32>(a, st);
  case 64: return inv_bh<64>(a, st);
  default: return cudaErrorInvalidValue;
  }
}

}  // namespace f3d
