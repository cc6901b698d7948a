// f3d_k_common.cu -- overlap-add + sample packing, and the launch dispatch.
// Compiled with --fmad=false (the packing must round like the reference).
#include "f3d_device.cuh"

#include <atomic>

namespace f3d {

static std::atomic<unsigned long long> g_launch_count{0};
void count_launch() { g_launch_count.fetch_add(1, std::memory_order_relaxed); }
unsigned long long launch_count() { return g_launch_count.load(std::memory_order_relaxed); }

namespace {

__device__ __forceinline__ int floor_div(int a, int b) {
  int q = a / b;
  return (a % b != 0 && ((a < 0) != (b < 0))) ? q - 1 : q;
}

// One output sample per thread: sum of the covering windowed blocks in
// ascending block order starting from 0 (src/cpu/reference.cpp:415-430, the
// same order as src/cl/kernels.h:409-435), plus chroma centering once
// (:433-436), then packed to the plane's sample format (:107-138).
__global__ void __launch_bounds__(256) k_ola(const __grid_constant__ OlaArgs a) {
  const int x = blockIdx.x * 32 + (threadIdx.x & 31);
  const int y = blockIdx.y * 8 + (threadIdx.x >> 5);
  const Geo& g = a.g;
  if (x >= g.W || y >= g.H) return;
  const int bsz = g.bw * g.bh;
  float sum = 0.0f;
  if (g.mode == 1) {
    int n0 = floor_div(x - g.xoff - g.bw, g.xstep) + 1;
    int n1 = floor_div(x - g.xoff, g.xstep);
    int m0 = floor_div(y - g.yoff - g.bh, g.ystep) + 1;
    int m1 = floor_div(y - g.yoff, g.ystep);
    if (n0 < 0) n0 = 0;
    if (m0 < 0) m0 = 0;
    if (n1 > g.ncols - 1) n1 = g.ncols - 1;
    if (m1 > g.nrows - 1) m1 = g.nrows - 1;
    // The step is at least half the block (the overlap is at most half of
    // it), so at most 2 x 2 blocks cover a sample: their values are loaded
    // together, then added in block order.
    float v[2][2] = {{0.0f, 0.0f}, {0.0f, 0.0f}};
#pragma unroll
    for (int i = 0; i < 2; i++) {
      const int m = m0 + i;
      if (m > m1) continue;
      const int ly = y - (g.yoff + m * g.ystep);
#pragma unroll
      for (int j = 0; j < 2; j++) {
        const int n = n0 + j;
        if (n > n1) continue;
        const int lx = x - (g.xoff + n * g.xstep);
        v[i][j] = a.blocks[(size_t)(m * g.ncols + n) * bsz + ly * g.bw + lx];
      }
    }
#pragma unroll
    for (int i = 0; i < 2; i++)
#pragma unroll
      for (int j = 0; j < 2; j++)
        if (m0 + i <= m1 && n0 + j <= n1) sum += v[i][j];
  } else {
    const int per = g.ncols * g.nrows;
    for (int grid = 0; grid < 2; grid++) {
      const int ox = grid ? g.bw / 2 : 0, oy = grid ? g.bh / 2 : 0;
      const int n = (x + ox) / g.bw, m = (y + oy) / g.bh;
      if (n < g.ncols && m < g.nrows) {
        const int lx = x + ox - n * g.bw, ly = y + oy - m * g.bh;
        sum += a.blocks[(size_t)(grid * per + m * g.ncols + n) * bsz + ly * g.bw + lx];
      }
    }
  }
  if (a.chroma_norm != 0.0f) sum += a.chroma_norm;
  store_sample(a.dst + (long long)y * a.pitch, x, sum, a.fmt, a.inv_norm, a.max_pix);
}

}  // namespace

cudaError_t launch_ola(const OlaArgs& a, cudaStream_t st) {
  if (a.g.W <= 0 || a.g.H <= 0) return cudaSuccess;
  dim3 grid((a.g.W + 31) / 32, (a.g.H + 7) / 8);
  k_ola<<<grid, 256, 0, st>>>(a);
  count_launch();
  return cudaGetLastError();
}

static bool pow2_in(int v, int lo, int hi) { return v >= lo && v <= hi && (v & (v - 1)) == 0; }

bool form_supported(int form, int bw, int bh) {
  if (form == F3D_FORM_EXACT) return pow2_in(bw, 4, 512) && pow2_in(bh, 4, 512);
  if (form == F3D_FORM_FAST) return pow2_in(bw, 8, 64) && pow2_in(bh, 8, 64);
  if (form == F3D_FORM_TC) return bw == bh && (bw == 16 || bw == 32);
  return false;
}

cudaError_t launch_forward(int form, const FwdArgs& a, cudaStream_t st) {
  if (form == F3D_FORM_FAST) return launch_forward_fast(a, st);
  if (form != F3D_FORM_EXACT) return cudaErrorNotSupported;
  if (big_block(a.g.bw, a.g.bh)) return launch_forward_big(a, st);
  switch (a.g.bw) {
  case 4: return launch_forward_exact_bw4(a, st);
  case 8: return launch_forward_exact_bw8(a, st);
  case 16: return launch_forward_exact_bw16(a, st);
  case 32: return launch_forward_exact_bw32(a, st);
  case 64: return launch_forward_exact_bw64(a, st);
  default: return cudaErrorInvalidValue;
  }
}

cudaError_t launch_filter_inverse(int form, const InvArgs& a, cudaStream_t st) {
  if (form == F3D_FORM_FAST) return launch_inverse_fast(a, st);
  if (form != F3D_FORM_EXACT) return cudaErrorNotSupported;
  if (big_block(a.g.bw, a.g.bh)) return launch_inverse_big(a, st);
  switch (a.g.bw) {
  case 4: return launch_inverse_exact_bw4(a, st);
  case 8: return launch_inverse_exact_bw8(a, st);
  case 16: return launch_inverse_exact_bw16(a, st);
  case 32: return launch_inverse_exact_bw32(a, st);
  case 64: return launch_inverse_exact_bw64(a, st);
  default: return cudaErrorInvalidValue;
  }
}

}  // namespace f3d
