// f3d_k_sweep.cu -- fused filter + inverse + overlap-add + packing (fast
// form) for mode 1 with half overlap, the geometry of every default and
// benchmark configuration.
//
// Cells: the plane is cut into cells of cw x ch = (bw/2) x (bh/2) samples;
// block (m, n) covers cell rows m-1, m and cell columns n-1, n, so cell (i, j)
// is the sum of four quadrants, taken in the reference's block order
// (src/cpu/reference.cpp:415-430):
//   ((q(i,j) + q(i,j+1)) + q(i+1,j)) + q(i+1,j+1)
// where q(m,n) is the part of block (m, n)'s windowed inverse over the cell.
// With half overlap every cell inside the plane has all four blocks.
//
// A CTA of F3D_SWEEP_THREADS threads holds threads/bw block slots (one
// thread per block row); it owns a strip of TJ = slots-1 cells (slot s
// computes block column J0+s, the last slot the strip's right neighbour
// column) and a segment [M0, M1) of block rows. For
// each block row m it filters and inverts the row's blocks into shared
// memory, then
//   - finishes cell row m-1 from the partial sums P (q(m-1,j) + q(m-1,j+1))
//     plus the top halves of row m, and writes it, packed, to the plane;
//   - starts cell row m: P = bottom halves of row m.
// The first cell row of a segment (row M0-1) and its last (M1-1) are shared
// with the neighbouring segments: their quadrants go to seam buffers and
// k_seam_merge finishes them in the same order. The next row's window
// spectra can be bulk-prefetched into L2 while row m is processed (off by
// default: with one wave of CTAs each holding a row, the prefetched rows
// exceed what L2 keeps and the extra traffic costs more than it hides).
#include "f3d_batch_plan.hpp"
#include "f3d_fast.cuh"

#include <algorithm>

namespace f3d {
namespace {

// CTA size and resident CTAs per SM of the sweep (register budget =
// 65536 / (threads * CTAs)).
#ifndef F3D_SWEEP_THREADS
#define F3D_SWEEP_THREADS 256
#endif
#ifndef F3D_SWEEP_MINB
#define F3D_SWEEP_MINB 3
#endif
constexpr int kSweepThreads = F3D_SWEEP_THREADS;

template <int BW, int BH>
struct SCfg {
  using C = FCfg<BW, BH>;
  static constexpr int TPB = BW;  // square blocks: inverse_block_sq, one thread per row
  static constexpr int SLOTS = kSweepThreads / TPB;
  static constexpr int TJ = SLOTS - 1;             // cells per strip
  static constexpr int CW = BW / 2, CH = BH / 2;   // cell size
  static constexpr int QK = CW / 4;                // float4 chunks per cell row
  static constexpr size_t SMEM = sizeof(float2) * C::SMEM_F2 * SLOTS + sizeof(float) * TJ * CH * CW;
};

// Samples x..x+3 (x even) of row y of a block's windowed inverse, stored in
// its tile as pairs: (x, x+1) at Q[(x/2)*SB + yperm(y)].
template <int SB, int BH>
__device__ __forceinline__ float4 qload(const float2* Q, int y, int x) {
  const int yp = yperm<BH>(y);
  const float2 lo = Q[(x / 2) * SB + yp], hi = Q[(x / 2 + 1) * SB + yp];
  return make_float4(lo.x, lo.y, hi.x, hi.y);
}

__device__ __forceinline__ float4 add4(float4 a, float4 b) {
  return make_float4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w);
}

// Four output samples at x..x+3 of row y (bounds-checked against the plane).
__device__ __forceinline__ void store4(const SweepArgs& sa, int y, int x, float4 v) {
  if (y >= sa.inv.g.H) return;
  uint8_t* row = sa.dst + (long long)y * sa.pitch;
  const float e[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
  for (int k = 0; k < 4; k++) {
    if (x + k >= sa.inv.g.W) break;
    float s = e[k];
    if (sa.chroma_norm != 0.0f) s += sa.chroma_norm;
    store_sample(row, x + k, s, sa.fmt, sa.inv_norm, sa.max_pix);
  }
}

// CTA `cta` (strip, segment) of plane sa's sweep.
template <int BW, int BH, int BM>
__device__ __forceinline__ void sweep_fast_cta(const SweepArgs& sa, int cta) {
  using S_ = SCfg<BW, BH>;
  using C = FCfg<BW, BH>;
  constexpr int TPB = S_::TPB, TJ = S_::TJ, CW = S_::CW, CH = S_::CH, QK = S_::QK;
  constexpr int NWIN = BM >= 2 ? BM : 1;
  const InvArgs& a = sa.inv;
  extern __shared__ float4 smem4[];
  float2* slots = reinterpret_cast<float2*>(smem4);
  float4* P = reinterpret_cast<float4*>(slots + S_::SLOTS * C::SMEM_F2);  // [TJ][CH][QK]
  const int slot = threadIdx.x / TPB, t = threadIdx.x - slot * TPB;
  float2* S = slots + slot * C::SMEM_F2;
  const int strip = cta % sa.strips, seg = cta / sa.strips;
  const int J0 = strip * TJ;
  const int nrow = sa.cells_y + 1;  // block rows 0..cells_y are needed
  const int M0 = (int)((long long)seg * nrow / sa.segs);
  const int M1 = (int)((long long)(seg + 1) * nrow / sa.segs);
  const int n = J0 + slot;
  const bool col_ok = n <= sa.cells_x;  // block columns 0..cells_x are needed
  const int ncell = min(TJ, sa.cells_x - J0);
  constexpr float inv_n = 1.0f / (BW * BH);

  // L2 prefetch of one block's window spectra (one thread per slot).
  auto prefetch_block = [&](int bb) {
#pragma unroll
    for (int k = 0; k < NWIN; k++) prefetch_l2(a.s[k] + (size_t)bb * C::PS, C::PS * sizeof(float2));
  };
  if (sa.prefetch && t == 0 && col_ok && M0 < M1) prefetch_block(M0 * a.g.ncols + n);
  for (int m = M0; m < M1; m++) {
    const int b = m * a.g.ncols + n;
    const bool pf_next = t == 0 && col_ok && m + 1 < M1;
    if (sa.prefetch == 1 && pf_next) prefetch_block(b + a.g.ncols);
    // Windowed rows go back into the tile as sample pairs: (x, x+1) of row y
    // at S[(x/2)*SB + yperm(y)] (see inverse_block).
    const float* win = (n & 1) ? a.win_b : a.win_a;
    inverse_block_sq<BW, BM>(a, b, t, col_ok, S, [&](int y, const float2(&xy)[BW / 2]) {
#pragma unroll
      for (int k = 0; k < BW / 2; k++) {
        const float2 wv = *reinterpret_cast<const float2*>(win + y * BW + 2 * k);
        S[k * C::SB + yperm<BH>(y)] = make_float2(xy[k].x * inv_n * wv.x, xy[k].y * inv_n * wv.y);
      }
    }, [&] {
      // Row m's spectra are read by now: fetch row m+1 while the transforms
      // and the cell sums of row m run.
      if (sa.prefetch == 2 && pf_next) prefetch_block(b + a.g.ncols);
    });
    __syncthreads();
    const bool emit = m > M0;                       // cell row m-1 finishes here
    const bool seam_top = m == M0 && M0 > 0;        // cell row M0-1: quadrants 3, 4 to the seam
    const bool seam_bot = m == M1 - 1 && seg < sa.segs - 1;  // cell row M1-1: quadrants 1, 2
    for (int it = threadIdx.x; it < CH * TJ * QK; it += kSweepThreads) {
      const int yy = it / (TJ * QK);
      const int rem = it - yy * (TJ * QK);
      const int jj = rem / QK, k = rem - jj * QK;
      if (jj >= ncell) continue;
      const float2* Qa = slots + jj * C::SMEM_F2;
      const float2* Qb = slots + (jj + 1) * C::SMEM_F2;
      const float4 q10 = qload<C::SB, BH>(Qa, yy, CW + 4 * k);  // block (m, j) top right
      const float4 q11 = qload<C::SB, BH>(Qb, yy, 4 * k);       // block (m, j+1) top left
      float4& p = P[(jj * CH + yy) * QK + k];
      const int x = (J0 + jj) * CW + 4 * k;
      if (emit) {
        store4(sa, (m - 1) * CH + yy, x, add4(add4(p, q10), q11));
      } else if (seam_top) {
        float* t0 = sa.seam_t + ((size_t)((seg - 1) * 2) * CH + yy) * sa.seam_w + x;
        float* t1 = sa.seam_t + ((size_t)((seg - 1) * 2 + 1) * CH + yy) * sa.seam_w + x;
        *reinterpret_cast<float4*>(t0) = q10;
        *reinterpret_cast<float4*>(t1) = q11;
      }
      p = add4(qload<C::SB, BH>(Qa, CH + yy, CW + 4 * k), qload<C::SB, BH>(Qb, CH + yy, 4 * k));  // row m bottom halves
      if (seam_bot) *reinterpret_cast<float4*>(sa.seam_b + ((size_t)seg * CH + yy) * sa.seam_w + x) = p;
    }
    __syncthreads();
  }
}

template <int BW, int BH, int BM>
__global__ void __launch_bounds__(kSweepThreads, F3D_SWEEP_MINB) k_sweep_fast(const __grid_constant__ SweepArgs sa) {
  sweep_fast_cta<BW, BH, BM>(sa, blockIdx.x);
}

// The sweeps of a batch of planes in one launch: the CTAs of a run of
// planes of one geometry (consecutive outputs of a plane) are interleaved,
// so that the window spectra they share are read from L2 the second time.
template <int BW, int BH, int BM>
__global__ void __launch_bounds__(kSweepThreads, F3D_SWEEP_MINB)
    k_sweep_fast_batch(const __grid_constant__ SweepBatch B) {
  int p = 0;
  while (p + 1 < B.n && (int)blockIdx.x >= B.cta0[p + 1]) p++;
  const int r0 = B.run[p], rl = B.rlen[r0];
  const int local = (int)blockIdx.x - B.cta0[r0];
  sweep_fast_cta<BW, BH, BM>(B.p[r0 + local % rl], local / rl);
}

// Finishes the seam cell rows: ((q1 + q2) + q3) + q4 per sample, packed.
__global__ void __launch_bounds__(256) k_seam_merge(const __grid_constant__ SweepArgs sa, int ch) {
  const int x = blockIdx.x * 256 + threadIdx.x;
  const int yy = blockIdx.y, k = blockIdx.z;  // seam k: cell row M1(k) - 1
  if (x >= sa.inv.g.W) return;
  const int nrow = sa.cells_y + 1;
  const int m1 = (int)((long long)(k + 1) * nrow / sa.segs);
  const int y = (m1 - 1) * ch + yy;
  if (y >= sa.inv.g.H) return;
  const size_t o = ((size_t)k * ch + yy) * sa.seam_w + x;
  const size_t ot = ((size_t)(k * 2) * ch + yy) * sa.seam_w + x;
  float v = sa.seam_b[o] + sa.seam_t[ot];
  v = v + sa.seam_t[ot + (size_t)ch * sa.seam_w];
  if (sa.chroma_norm != 0.0f) v += sa.chroma_norm;
  store_sample(sa.dst + (long long)y * sa.pitch, x, v, sa.fmt, sa.inv_norm, sa.max_pix);
}

template <int BW, int BH, int BM>
cudaError_t launch_bm(const SweepArgs& a, cudaStream_t st, cudaEvent_t mark) {
  using S_ = SCfg<BW, BH>;
  auto k = k_sweep_fast<BW, BH, BM>;
  static_assert(S_::SMEM * F3D_SWEEP_MINB <= 227 * 1024, "CTAs per SM");
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)S_::SMEM);
  if (e != cudaSuccess) return e;
  k<<<a.strips * a.segs, kSweepThreads, S_::SMEM, st>>>(a);
  count_launch();
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  if (mark) cudaEventRecord(mark, st);
  return launch_seam_merge(a, st);
}

template <int BW, int BH, int BM>
cudaError_t launch_batch_bm(const SweepBatch& Bs, int n, cudaStream_t st) {
  using S_ = SCfg<BW, BH>;
  auto k = k_sweep_fast_batch<BW, BH, BM>;
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)S_::SMEM);
  if (e != cudaSuccess) return e;
  if (Bs.cta0[n] == 0) return cudaSuccess;
  k<<<Bs.cta0[n], kSweepThreads, S_::SMEM, st>>>(Bs);
  count_launch();
  return cudaGetLastError();
}

template <int BW, int BH>
cudaError_t launch_batch_size(const SweepBatch& Bs, int n, cudaStream_t st) {
  switch (Bs.p[0].inv.bm) {
  case -1: return launch_batch_bm<BW, BH, -1>(Bs, n, st);
  case 1: return launch_batch_bm<BW, BH, 1>(Bs, n, st);
  case 2: return launch_batch_bm<BW, BH, 2>(Bs, n, st);
  case 3: return launch_batch_bm<BW, BH, 3>(Bs, n, st);
  case 4: return launch_batch_bm<BW, BH, 4>(Bs, n, st);
  default: return cudaErrorNotSupported;
  }
}

template <int BW, int BH>
cudaError_t launch_size(const SweepArgs& a, cudaStream_t st, cudaEvent_t mark) {
  switch (a.inv.bm) {
  case -1: return launch_bm<BW, BH, -1>(a, st, mark);
  case 1: return launch_bm<BW, BH, 1>(a, st, mark);
  case 2: return launch_bm<BW, BH, 2>(a, st, mark);
  case 3: return launch_bm<BW, BH, 3>(a, st, mark);
  case 4: return launch_bm<BW, BH, 4>(a, st, mark);
  default: return cudaErrorNotSupported;
  }
}

}  // namespace

cudaError_t launch_sweep_fast_batch(const SweepArgs* planes, int n, cudaStream_t st, cudaEvent_t mark) {
  SweepBatch Bf, Bs, Bm;
  if (!sweep_batches(planes, n, Bf, Bs, Bm, false))
    return n < 1 || n > kMaxBatch ? cudaErrorInvalidValue : cudaErrorNotSupported;
  int maxw = 0;
  for (int i = 0; i < n; i++) maxw = std::max(maxw, planes[i].inv.g.W);
  cudaError_t e;
  switch (planes[0].inv.g.bw) {
  case 8: e = launch_batch_size<8, 8>(Bs, n, st); break;
  case 16: e = launch_batch_size<16, 16>(Bs, n, st); break;
  case 32: e = launch_batch_size<32, 32>(Bs, n, st); break;
  default: return cudaErrorNotSupported;
  }
  if (e != cudaSuccess) return e;
  if (mark) cudaEventRecord(mark, st);
  return launch_seam_merge_batch(Bm, n, maxw, planes[0].inv.g.bh / 2, st);
}

cudaError_t launch_seam_merge(const SweepArgs& a, cudaStream_t st) {
  if (a.segs < 2) return cudaSuccess;
  dim3 grid((a.inv.g.W + 255) / 256, a.inv.g.bh / 2, a.segs - 1);
  k_seam_merge<<<grid, 256, 0, st>>>(a, a.inv.g.bh / 2);
  count_launch();
  return cudaGetLastError();
}

bool sweep_supported(int form, const Geo& g, int bm) {
  if (bm == 0 || g.mode != 1) return false;
  if (form == F3D_FORM_TC) {
    if (!tc_supported(g.mode, g.bw, g.bh, bm)) return false;
  } else if (form != F3D_FORM_FAST || g.bw != g.bh || (g.bw != 8 && g.bw != 16 && g.bw != 32)) {
    return false;
  }
  return g.xoff == -g.bw / 2 && g.xstep == g.bw / 2 && g.yoff == -g.bh / 2 && g.ystep == g.bh / 2;
}

void sweep_plan(int form, const Geo& g, int sm_count, int* strips, int* segs) {
  const int tj = form == F3D_FORM_TC ? tc_sweep_cells(g.bw) : kSweepThreads / g.bw - 1;
  const int per_sm = form == F3D_FORM_TC ? kTcSweepCtasPerSm : F3D_SWEEP_MINB;
  const int cells_x = (g.W + g.bw / 2 - 1) / (g.bw / 2);
  const int cells_y = (g.H + g.bh / 2 - 1) / (g.bh / 2);
  *strips = (cells_x + tj - 1) / tj;
  // At most one wave of resident CTAs (a partial second wave would double the
  // time), segments of at least two block rows.
  int s = per_sm * sm_count / *strips;
  const int maxseg = (cells_y + 1) / 2;
  if (s > maxseg) s = maxseg;
  *segs = s < 1 ? 1 : s;
}

size_t sweep_seam_floats(const Geo& g, int segs) {
  const int cells_x = (g.W + g.bw / 2 - 1) / (g.bw / 2);
  return (size_t)(segs > 1 ? segs - 1 : 0) * 3 * (g.bh / 2) * (size_t)cells_x * (g.bw / 2);
}

cudaError_t launch_sweep(int form, const SweepArgs& a, cudaStream_t st, cudaEvent_t mark) {
  if (!sweep_supported(form, a.inv.g, a.inv.bm)) return cudaErrorNotSupported;
  if (form == F3D_FORM_TC) return launch_sweep_tc(a, st, mark);
  switch (a.inv.g.bw) {
  case 8: return launch_size<8, 8>(a, st, mark);
  case 16: return launch_size<16, 16>(a, st, mark);
  case 32: return launch_size<32, 32>(a, st, mark);
  default: return cudaErrorNotSupported;
  }
}

}  // namespace f3d
