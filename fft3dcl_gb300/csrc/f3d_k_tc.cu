// f3d_k_tc.cu -- the tensor-core form: 2D block DFTs as dense DFT-matrix
// products on the fifth-generation tensor cores (tcgen05), fp16 operands
// split into hi + lo parts with fp32 accumulation in tensor memory.
//
// Forward transform of an n x n real block X (n = 32) with separable
// analysis window wx[x] * wy[y] (src/cpu/tables.cpp:21-105), folded into the
// DFT matrices:
//   step 1 (rows):    Z[y][j] = sum_x X[y][x] * B1[j][x], the n real outputs
//                     j = (Re Z0, Re Z(n/2), Re Z1, Im Z1, .., Im Z(n/2-1)) of
//                     each row's real DFT;
//   step 2 (columns): for each packed column k' = 0..n/2-1 (k' = 0 carries
//                     Z0 + i Z(n/2)), Y[ky][k'] = sum_y e^(-2 pi i ky y/n)
//                     wy[y] Z[y][k'] as a real 2n x 2n matrix B2 acting on
//                     interleaved (re, im) pairs;
//   unpacking:        Y0 = (P + conj P(-ky))/2, Y(n/2) = (P - conj P(-ky))/2i
//                     for the packed column P.
// This equals fft2dRealForward of the windowed block (src/cpu/fft.cpp:68-86,
// src/cpu/reference.cpp:140-170) up to fp32 rounding. The chroma offset is
// removed in the spectrum (c * DFT(window)), the sample scale (1/255,
// 2^(16-bits)/65535) applied to the output.
//
// Tiling: a group of G = 8 blocks; step 1 runs as two M = 128 tiles (rows =
// 4 blocks x 32 rows, N = 32, K = 32), step 2 as one M = 128 tile (rows = 8
// blocks x 16 packed columns, N = 64, K = 64). Operands hi/lo: step 1 uses
// X exactly (integer samples of up to 11 bits are exact in fp16) times
// B1hi + B1lo, or Xhi*B1hi + Xhi*B1lo + Xlo*B1hi; step 2 Ahi*Bhi + Ahi*Blo +
// Alo*Bhi. The spectra of a group (8 x 4352 bytes, contiguous in HBM) leave
// shared memory by one bulk copy.
#include "f3d_batch_plan.hpp"
#include "f3d_device.cuh"
#include "f3d_tc.cuh"

#include <algorithm>
#include <cmath>
#include <cstring>

namespace f3d {
namespace {

constexpr double kPiD = 3.14159265358979323846;

// Byte offsets of the table sections for n x n blocks.
template <int N>
struct TcTab {
  static constexpr int FBW = N / 2 + 1;
  static constexpr uint32_t B1HI = 0, B1LO = B1HI + N * N * 2;
  static constexpr uint32_t B2HI = B1LO + N * N * 2, B2LO = B2HI + 8 * N * N;
  static constexpr uint32_t WSPEC = B2LO + 8 * N * N;  // float2 [N][FBW]
  static constexpr uint32_t C2HI = WSPEC + N * FBW * 8, C2LO = C2HI + 8 * N * N;
  // Row inverses with the even (A) and odd (B) synthesis x-windows.
  static constexpr uint32_t C1AHI = C2LO + 8 * N * N, C1ALO = C1AHI + N * N * 2;
  static constexpr uint32_t C1BHI = C1ALO + N * N * 2, C1BLO = C1BHI + N * N * 2;
  static constexpr uint32_t TOTAL = C1BLO + N * N * 2;
  static_assert(WSPEC % 16 == 0 && C2HI % 16 == 0 && C1AHI % 16 == 0, "16-byte sections");
};

// Scale of the filtered spectrum before its hi/lo split in the inverse
// (keeps the column sums inside fp16 range), undone with the inverse's
// 1/n^2 when the blocks are added up.
constexpr float kInvPre = 1.0f / 16.0f;

// Kernel configuration for n x n blocks.
template <int N>
struct TcCfg {
  static constexpr int NY = N / 2, FBW = NY + 1, PS = N * FBW;
  static constexpr int G = 128 / NY;       // blocks per group (step-2 tile rows: G x NY)
  static constexpr int BPT1 = 128 / N;     // blocks per step-1 tile (rows: BPT1 x N)
  static constexpr int T1 = G / BPT1;      // step-1 tiles per group
  static constexpr int K1 = N, N1 = N;     // step 1: K = x, N = packed outputs
  static constexpr int K2 = 2 * N, N2 = 2 * N;
  static constexpr uint32_t A1_BYTES = 128 * K1 * 2, A2_BYTES = 128 * K2 * 2;
  static constexpr uint32_t B1_BYTES = N1 * K1 * 2, B2_BYTES = N2 * K2 * 2;
  static constexpr uint32_t TMEM_COLS = 128;
  static constexpr uint32_t D1_COL = 0, D2_COL = 64;
  static_assert(N == 16 || N == 32, "the tensor-core form is built for 16 x 16 and 32 x 32 blocks");
  static_assert(T1 * N1 <= (int)D2_COL && D2_COL + N2 <= (int)TMEM_COLS, "tensor memory columns");
};

// The step-2 operand (128 rows, K2 = 2N fp16 columns; the column inverse's
// operand tile too): SWIZZLE_128B for N = 32 (rows of 128 bytes), the
// interleaved core-matrix layout for N = 16 (rows of 64 bytes).
template <int N>
__host__ __device__ constexpr uint32_t a2_off(int row, int k) {
  return N == 32 ? tc::off_sw128(row, k) : tc::off_il(row, k, 2 * N);
}
// Descriptor of K-step ks (16 columns) of a step-2 operand at base.
template <int N>
__device__ __forceinline__ uint64_t a2_desc(uint32_t base, int ks) {
  if constexpr (N == 32) return tc::sdesc(base + ks * 32, 16, 1024, tc::LAYOUT_SW128);
  else return tc::sdesc(base + ks * 256, 128, (2 * N / 8) * 128, tc::LAYOUT_INTERLEAVE);
}

constexpr int kTcThreads = 256;
// Filter-kernel variants: CTAs per SM (minb) and filter_batch(minb), the
// blocks of a group whose spectra loads are in flight together; fewer CTAs
// leave registers for deeper batches.
__host__ __device__ constexpr int filter_batch(int minb) { return minb >= 5 ? 1 : 2; }
constexpr uint64_t kWaitNs = 1000000000ull;  // one second

// ---- forward ---------------------------------------------------------------

// Shared memory of the forward kernel (offsets from a 1024-aligned base).
// A1 and A2 are live at the same time (the next group's step-1 operand is
// deposited while step 2 of the current group runs). The staging area of a
// group's spectra shares A2's space: it is written once step 2 has read A2,
// and its bulk store has drained before the next group writes A2. Without the
// split (integer samples of up to 11 bits) A1 holds only the hi parts: 73 KB,
// three CTAs per SM; with the split 88 KB, two.
template <int N, bool SPLIT>
struct FwdSmem {
  using C = TcCfg<N>;
  static constexpr uint32_t A1_TILE = (SPLIT ? 2 : 1) * C::A1_BYTES;  // hi[, lo] of one step-1 tile
  static constexpr uint32_t STAGE_BYTES = C::G * C::PS * 8;           // float2 [G][N][FBW]
  static constexpr uint32_t B2 = 0;                       // hi, lo
  static constexpr uint32_t B1 = B2 + 2 * C::B2_BYTES;    // hi, lo
  static constexpr uint32_t A2 = (B1 + 2 * C::B1_BYTES + 1023) / 1024 * 1024;  // hi, lo (SWIZZLE_128B)
  static constexpr uint32_t STAGE = A2;
  static constexpr uint32_t A1 = A2 + (2 * C::A2_BYTES > STAGE_BYTES ? 2 * C::A2_BYTES : STAGE_BYTES);
  static constexpr uint32_t BAR = A1 + C::T1 * A1_TILE;   // [tile][hi, lo]
  static constexpr uint32_t TSLOT = BAR + 16;
  static constexpr uint32_t BYTES = TSLOT + 16 + 1024;    // + alignment slack
  static_assert(STAGE % 16 == 0 && A1 % 128 == 0 && BAR % 16 == 0, "bulk-copy and operand alignment");
};
// CTAs per SM of the forward kernel: the launch bound, and what fits.
constexpr int kFwdMaxCtasPerSm = 3;

// Gather of a group's samples: task q covers 16 source bytes (16/BPS samples)
// of row y of block bl. The raw bytes are fetched into registers one group
// ahead, so that their loads are in flight while the tensor cores work on the
// current group, and deposited into the step-1 operand as fp16.
template <int N, int BPS>
struct Gather {
  static constexpr int S = 16 / BPS;                   // samples per task
  static constexpr int TPR = N / S;                    // tasks per block row
  static constexpr int TASKS = TcCfg<N>::G * N * TPR;
  static constexpr int TPT = TASKS / kTcThreads;       // tasks per thread
  static_assert(TASKS % kTcThreads == 0 && S >= 4, "task split");
};

template <int N, int BPS>
__device__ __forceinline__ void fetch(const TcFwdArgs& a, int b0, int nvalid, uint4 (&r)[Gather<N, BPS>::TPT]) {
  using Gt = Gather<N, BPS>;
  // The group's blocks are consecutive in the mode-1 grid (the only mode of
  // this form): one division for the first, a carry into the next block row
  // for the others.
  const int m0 = b0 / a.g.ncols, n0 = b0 - m0 * a.g.ncols;
#pragma unroll
  for (int i = 0; i < Gt::TPT; i++) {
    const int q = threadIdx.x + i * kTcThreads;
    const int c = q % Gt::TPR, ry = q / Gt::TPR;
    const int bl = ry / N, y = ry - bl * N;
    r[i] = make_uint4(0u, 0u, 0u, 0u);
    if (bl >= nvalid) continue;
    int n = n0 + bl, m = m0;
    while (n >= a.g.ncols) {
      n -= a.g.ncols;
      m++;
    }
    const int bx = a.g.xoff + n * a.g.xstep, by = a.g.yoff + m * a.g.ystep;
    if (bx >= 0 && by >= 0 && bx + N <= a.g.W && by + N <= a.g.H) {
      const uint8_t* p = a.src + (long long)(by + y) * a.pitch + (long long)bx * BPS + 16 * c;
      if ((reinterpret_cast<uintptr_t>(p) & 15) == 0) {
        r[i] = __ldg(reinterpret_cast<const uint4*>(p));
        continue;
      }
    }
    // Mirrored or unaligned: one sample at a time (src/cpu/reference.cpp:10-17).
    const uint8_t* row = a.src + (long long)mirror_i(by + y, a.g.H) * a.pitch;
    uint32_t w[4] = {0u, 0u, 0u, 0u};
#pragma unroll
    for (int k = 0; k < Gt::S; k++) {
      const int x = mirror_i(bx + c * Gt::S + k, a.g.W);
      uint32_t v;
      if (BPS == 1) v = row[x];
      else if (BPS == 2) v = reinterpret_cast<const uint16_t*>(row)[x];
      else v = reinterpret_cast<const uint32_t*>(row)[x];
      w[(k * BPS) / 4] |= v << (8 * ((k * BPS) % 4));
    }
    r[i] = make_uint4(w[0], w[1], w[2], w[3]);
  }
}

// Raw bytes -> fp16 (hi, and lo on the split path) in A1[tile][part]: rows
// (block % BPT1, y), K = x.
template <int N, int BPS, bool SPLIT>
__device__ __forceinline__ void deposit(const TcFwdArgs& a, uint8_t* a1, const uint4 (&r)[Gather<N, BPS>::TPT]) {
  using Gt = Gather<N, BPS>;
  using C = TcCfg<N>;
  const bool split = SPLIT && a.split;
  // Integer samples below 1024 become fp16 exactly by exponent bias: 0x6400
  // is 1024.0, and its ten mantissa bits hold the sample, so (0x6400 | v) -
  // 1024 = v, two instructions per pair. Samples of 1024 and above (11-bit
  // clips) take the conversion through fp32.
  bool small = BPS == 1;
  if (BPS == 2 && !split) {
    uint32_t hi_bits = 0u;
#pragma unroll
    for (int i = 0; i < Gt::TPT; i++) hi_bits |= r[i].x | r[i].y | r[i].z | r[i].w;
    small = (hi_bits & 0xFC00FC00u) == 0u;
  }
  const __half2 k1024 = __halves2half2(__ushort_as_half(0x6400), __ushort_as_half(0x6400));
#pragma unroll
  for (int i = 0; i < Gt::TPT; i++) {
    const int q = threadIdx.x + i * kTcThreads;
    const int c = q % Gt::TPR, ry = q / Gt::TPR;
    const int bl = ry / N, y = ry - bl * N;
    const int tile = bl / C::BPT1, row = (bl % C::BPT1) * N + y;
    const uint32_t w[4] = {r[i].x, r[i].y, r[i].z, r[i].w};
    uint32_t h[Gt::S / 2], l[Gt::S / 2];
    if (BPS <= 2 && small) {
#pragma unroll
      for (int k = 0; k < Gt::S / 2; k++) {
        // The pair (sample 2k, sample 2k+1) with 0x64 as each one's high byte.
        const uint32_t biased = BPS == 1 ? __byte_perm(w[k >> 1], 0x64646464u, (k & 1) ? 0x4342u : 0x4140u)
                                         : (w[k] | 0x64006400u);
        const __half2 hv = __hsub2(*reinterpret_cast<const __half2*>(&biased), k1024);
        h[k] = *reinterpret_cast<const uint32_t*>(&hv);
        l[k] = 0u;
      }
    } else {
      float v[Gt::S];
#pragma unroll
      for (int k = 0; k < Gt::S; k++) {
        if (BPS == 1) v[k] = (float)((w[k >> 2] >> (8 * (k & 3))) & 0xffu);
        else if (BPS == 2) v[k] = (float)((w[k >> 1] >> (16 * (k & 1))) & 0xffffu) * (split ? a.norm : 1.0f);
        else v[k] = __uint_as_float(w[k]);
      }
#pragma unroll
      for (int k = 0; k < Gt::S / 2; k++) tc::split_pair(v[2 * k], v[2 * k + 1], h[k], l[k]);
    }
    uint8_t* t0 = a1 + tile * FwdSmem<N, SPLIT>::A1_TILE;
    const int x0 = c * Gt::S;
    if (Gt::S >= 8) {
#pragma unroll
      for (int j = 0; j < Gt::S / 8; j++) {
        const uint32_t o = tc::off_il(row, x0 + 8 * j, C::K1);
        *reinterpret_cast<uint4*>(t0 + o) = make_uint4(h[4 * j], h[4 * j + 1], h[4 * j + 2], h[4 * j + 3]);
        if (split)
          *reinterpret_cast<uint4*>(t0 + C::A1_BYTES + o) = make_uint4(l[4 * j], l[4 * j + 1], l[4 * j + 2], l[4 * j + 3]);
      }
    } else {
      const uint32_t o = tc::off_il(row, x0, C::K1);
      *reinterpret_cast<uint2*>(t0 + o) = make_uint2(h[0], h[1]);
      if (split) *reinterpret_cast<uint2*>(t0 + C::A1_BYTES + o) = make_uint2(l[0], l[1]);
    }
  }
}

// Plane of a batch that item idx (a CTA, or a forward block group) belongs to.
template <class Batch>
__device__ __forceinline__ int plane_of(const Batch& b, const int (&prefix)[kMaxBatch + 1], int idx) {
  int p = 0;
  while (p + 1 < b.n && idx >= prefix[p + 1]) p++;
  return p;
}

template <int N, int BPS, bool SPLIT>
__global__ void __launch_bounds__(kTcThreads, kFwdMaxCtasPerSm) k_forward_tc(const __grid_constant__ TcFwdBatch B) {
  using C = TcCfg<N>;
  using L = FwdSmem<N, SPLIT>;
  using T = TcTab<N>;
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t* sm = smem_raw + ((1024u - (tc::smem_u32(smem_raw) & 1023u)) & 1023u);
  const uint32_t sbase = tc::smem_u32(sm);
  uint64_t* bar = reinterpret_cast<uint64_t*>(sm + L::BAR);
  uint32_t* tslot = reinterpret_cast<uint32_t*>(sm + L::TSLOT);
  float2* stage = reinterpret_cast<float2*>(sm + L::STAGE);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

  // Constant operands (the same for every plane of a batch): B2 (hi, lo) and
  // B1 (hi, lo) are contiguous in the table.
  {
    const uint4* src2 = reinterpret_cast<const uint4*>(B.p[0].tab + T::B2HI);
    uint4* dst2 = reinterpret_cast<uint4*>(sm + L::B2);
    for (int i = tid; i < (int)(2 * C::B2_BYTES / 16); i += kTcThreads) dst2[i] = src2[i];
    const uint4* src1 = reinterpret_cast<const uint4*>(B.p[0].tab + T::B1HI);
    uint4* dst1 = reinterpret_cast<uint4*>(sm + L::B1);
    for (int i = tid; i < (int)(2 * C::B1_BYTES / 16); i += kTcThreads) dst1[i] = src1[i];
  }
  if (warp == 0) {
    tc::tmem_alloc(tslot, C::TMEM_COLS);
    tc::tmem_relinquish();
  }
  if (tid == 0) {
    tc::mbar_init(&bar[0], 1);
    tc::mbar_init(&bar[1], 1);
    tc::fence_mbar_init();
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = *tslot;
  const int ngroups = B.grp0[B.n];
  uint32_t phase = 0;
  uint4 raw[Gather<N, BPS>::TPT];
  // Raw samples of batch group g (the block group g - grp0[p] of plane p).
  auto fetch_group = [&](int g) {
    const int p = plane_of(B, B.grp0, g);
    const TcFwdArgs& ap = B.p[p];
    const int b = (g - B.grp0[p]) * C::G;
    fetch<N, BPS>(ap, b, min(C::G, ap.g.nb - b), raw);
  };
  // Group g (its samples in raw) into A1, the loads of the CTA's group after
  // it started, then step 1 on the tensor cores: D1[tile] = A1 * B1^T, two or
  // three passes, committed to bar[0]. A1 and D1 must be free: no step 1 in
  // flight, D1 read out.
  auto begin_group = [&](int g) {
    const TcFwdArgs& ap = B.p[plane_of(B, B.grp0, g)];
    deposit<N, BPS, SPLIT>(ap, sm + L::A1, raw);
    if (g + (int)gridDim.x < ngroups) fetch_group(g + gridDim.x);
    tc::fence_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    if (tid == 0) {
      tc::fence_after_sync();
      constexpr uint32_t id1 = tc::idesc_f16(128, C::N1);
      const uint32_t sbo = (C::K1 / 8) * 128;
      for (int t = 0; t < C::T1; t++) {
        const uint32_t a_hi = sbase + L::A1 + t * L::A1_TILE, a_lo = a_hi + C::A1_BYTES;
        const uint32_t d = tmem + C::D1_COL + t * C::N1;
        for (int ks = 0; ks < C::K1 / 16; ks++) {
          const uint64_t ah = tc::sdesc(a_hi + ks * 256, 128, sbo, tc::LAYOUT_INTERLEAVE);
          const uint64_t bh = tc::sdesc(sbase + L::B1 + ks * 256, 128, sbo, tc::LAYOUT_INTERLEAVE);
          const uint64_t bl = tc::sdesc(sbase + L::B1 + C::B1_BYTES + ks * 256, 128, sbo, tc::LAYOUT_INTERLEAVE);
          tc::mma_f16(d, ah, bh, id1, ks > 0);
          tc::mma_f16(d, ah, bl, id1, 1);
          if (SPLIT && ap.split)
            tc::mma_f16(d, tc::sdesc(a_lo + ks * 256, 128, sbo, tc::LAYOUT_INTERLEAVE), bh, id1, 1);
        }
      }
      tc::mma_commit(&bar[0]);
    }
  };
  if ((int)blockIdx.x < ngroups) {
    fetch_group(blockIdx.x);
    begin_group(blockIdx.x);
  }

  // Per group: step 1 was issued one iteration earlier; step 2 runs while
  // the next group's samples are deposited and its step 1 issued; the
  // spectra are staged and leave by one bulk copy, which drains while the
  // next group goes through steps 1 to 5.
  for (int grp = blockIdx.x; grp < ngroups; grp += gridDim.x) {
    const int pl = plane_of(B, B.grp0, grp);
    const TcFwdArgs& a = B.p[pl];
    const int b0 = (grp - B.grp0[pl]) * C::G;
    const int nvalid = min(C::G, a.g.nb - b0);
    // The previous group's bulk store must have read the staging area, which
    // shares A2's space (written next). Every thread takes the same branch: a
    // wait that gave up anywhere ends the sweep of groups for the whole CTA.
    if (tid == 0) tc::bulk_wait_read();
    if (!__syncthreads_and(tc::mbar_wait(&bar[0], phase, kWaitNs))) {
      if (tid == 0) atomicOr(a.err, kErrWaitForward);
      break;
    }
    tc::fence_after_sync();

    // 3. D1 -> A2 (hi, lo): row (block, k'), K = 2y + (re, im).
    {
      const int t = warp >> 2, s = warp & 3;
      const int r1 = 32 * s + lane;
      const int bl = t * C::BPT1 + r1 / N, y = r1 % N;
      float v[C::N1];
      tc::tmem_ld<C::N1>(tmem + ((uint32_t)(32 * s) << 16) + C::D1_COL + t * C::N1, v);
#pragma unroll
      for (int kp = 0; kp < C::NY; kp++) {
        uint32_t hi, lo;
        tc::split_pair(v[2 * kp], v[2 * kp + 1], hi, lo);
        const uint32_t o = a2_off<N>(bl * C::NY + kp, 2 * y);
        *reinterpret_cast<uint32_t*>(sm + L::A2 + o) = hi;
        *reinterpret_cast<uint32_t*>(sm + L::A2 + C::A2_BYTES + o) = lo;
      }
    }
    tc::fence_async_smem();
    tc::fence_before_sync();
    __syncthreads();

    // 4. Step 2: D2 = A2 * B2^T, three passes.
    if (tid == 0) {
      tc::fence_after_sync();
      constexpr uint32_t id2 = tc::idesc_f16(128, C::N2);
      const uint32_t sbo_b = (C::K2 / 8) * 128;
      const uint32_t d = tmem + C::D2_COL;
      for (int ks = 0; ks < C::K2 / 16; ks++) {
        const uint64_t ah = a2_desc<N>(sbase + L::A2, ks);
        const uint64_t al = a2_desc<N>(sbase + L::A2 + C::A2_BYTES, ks);
        const uint64_t bh = tc::sdesc(sbase + L::B2 + ks * 256, 128, sbo_b, tc::LAYOUT_INTERLEAVE);
        const uint64_t bl = tc::sdesc(sbase + L::B2 + C::B2_BYTES + ks * 256, 128, sbo_b, tc::LAYOUT_INTERLEAVE);
        tc::mma_f16(d, ah, bh, id2, ks > 0);
        tc::mma_f16(d, ah, bl, id2, 1);
        tc::mma_f16(d, al, bh, id2, 1);
      }
      tc::mma_commit(&bar[1]);
    }

    // 5. The next group's operand and step 1 (every warp has read D1 above).
    if (grp + (int)gridDim.x < ngroups) begin_group(grp + gridDim.x);

    // Step 2 done: A2's space is free for the staging area.
    if (!__syncthreads_and(tc::mbar_wait(&bar[1], phase, kWaitNs))) {
      if (tid == 0) atomicOr(a.err, kErrWaitForward);
      break;
    }
    phase ^= 1;
    tc::fence_after_sync();

    // 6. D2 -> staging [block][ky][kx], scaled; column 0 holds the packed P.
    {
      const int s = warp & 3, h = warp >> 2;
      const int r2 = 32 * s + lane;
      const int bl = r2 / C::NY, kp = r2 % C::NY;
      float v[N];  // half of the N2 = 2N columns: NY values of ky, (re, im)
      tc::tmem_ld<N>(tmem + ((uint32_t)(32 * s) << 16) + C::D2_COL + N * h, v);
      float2* o = stage + bl * C::PS + kp;
#pragma unroll
      for (int j = 0; j < C::NY; j++) {
        const int ky = C::NY * h + j;
        o[ky * C::FBW] = make_float2(v[2 * j] * a.out_scale, v[2 * j + 1] * a.out_scale);
      }
    }
    __syncthreads();

    // 7. Unpack columns 0 and n/2; chroma offset.
    {
      const int bl = tid / N, ky = tid % N;
      float2* blk = stage + bl * C::PS;
      const float2 P = blk[ky * C::FBW], Q = blk[((N - ky) % N) * C::FBW];
      __syncwarp();
      // Both halves of a pair (ky, n-ky) sit in the same warp (N <= 32).
      blk[ky * C::FBW] = make_float2(0.5f * (P.x + Q.x), 0.5f * (P.y - Q.y));
      blk[ky * C::FBW + C::NY] = make_float2(0.5f * (P.y + Q.y), 0.5f * (Q.x - P.x));
      if (a.chroma_norm != 0.0f) {
        const float2* ws = reinterpret_cast<const float2*>(a.tab + T::WSPEC) + ky * C::FBW;
        for (int kx = 0; kx < C::FBW; kx++) {
          const float2 w = ws[kx];
          float2& z = blk[ky * C::FBW + kx];
          z.x -= a.chroma_norm * w.x;
          z.y -= a.chroma_norm * w.y;
        }
      }
    }
    // Half storage: the staged spectra narrowed to fp16 pairs in place (all
    // values read before any is written).
    if (a.half) {
      constexpr int PER = C::G * C::PS / kTcThreads;
      static_assert(C::G * C::PS % kTcThreads == 0, "staged values per thread");
      float2 r[PER];
      __syncthreads();
#pragma unroll
      for (int i = 0; i < PER; i++) r[i] = stage[tid + kTcThreads * i];
      __syncthreads();
      __half2* hs = reinterpret_cast<__half2*>(stage);
#pragma unroll
      for (int i = 0; i < PER; i++) hs[tid + kTcThreads * i] = __float22half2_rn(r[i]);
    }
    tc::fence_async_smem();
    __syncthreads();

    // 8. One bulk copy of the group's spectra to HBM.
    if (tid == 0 && nvalid > 0) {
      if (a.half)
        tc::bulk_store(reinterpret_cast<__half2*>(a.spec) + (size_t)b0 * C::PS, stage, (uint32_t)(nvalid * C::PS * 4));
      else
        tc::bulk_store(a.spec + (size_t)b0 * C::PS, stage, (uint32_t)(nvalid * C::PS * 8));
      tc::bulk_commit();
    }
  }
  if (tid == 0) tc::bulk_wait();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  if (warp == 0) tc::tmem_dealloc(tmem, C::TMEM_COLS);
}

// ---- sweep: filter, then inverse + overlap-add -------------------------------
//
// The tensor-core counterpart of the fast-form sweep (f3d_k_sweep.cu). The
// plane is cut into strips of TJ = 7 cells; the group of a strip in block row
// m is block columns J0..J0+7 (the last one the strip's right neighbour).
//
// k_filter_tc, one CTA per (row, strip) group:
//   F: the temporal filter (filter_vals, fast form) of the group's 8 x 544
//      bins, contiguous in HBM, into shared memory;
//   R: rows (k', block) of the column-inverse operand, k' = 0 packing the
//      Hermitian parts of columns 0 and n/2 as H0 + i H(n/2), scaled by
//      kInvPre and split hi/lo, written to HBM as the exact shared-memory
//      image (SWIZZLE_128B) the inverse kernel loads with one bulk copy.
// With no tensor-memory phases to wait for, it runs at five CTAs per SM.
//
// k_sweep_tc, one CTA per (strip, segment of block rows), per row:
//   the operand tile arrives by bulk copy (issued while the previous row's
//   transforms ran);
//   step 2': V[y][k'] = sum_ky e^(2 pi i ky y/n) sy[y] F[ky][k'] (tensor cores);
//   V: V into the row-inverse operand, rows (y, block slot) of two tiles
//      that hold the even and the odd block columns;
//   step 1': out[y][x] = sum_j V'[y][j] C1[x][j] with the even or odd
//      synthesis x-window (tensor cores), i.e. fft2dRealInverseHalf
//      (src/cpu/fft.cpp:88-119) times the synthesis window;
//   O: overlap-add from tensor memory into the cell partial sums in the
//      reference's block order (src/cpu/reference.cpp:415-436), finished cell
//      rows packed straight to the output plane; segment seams as in the
//      fast-form sweep.
template <int N>
struct SwpCfg {
  using C = TcCfg<N>;
  static constexpr int TJ = C::G - 1;        // cells per strip
  static constexpr int CH = N / 2, CW = N / 2;
  // Filtered-bin stride per block (float2), padded: in R a half-warp reads
  // the same bin of 8 blocks for 2 k', which fall in 16 distinct bank pairs
  // when FS / 2 is odd.
  static constexpr int FS = C::PS + 2;
  static_assert(FS % 4 == 2, "R-phase loads free of bank conflicts");
  static constexpr int PR = CW + 4;          // partial-sum row stride (floats), padded
  static constexpr int PC = CH * PR + 4;     // partial-sum cell stride (floats), padded
  static constexpr uint32_t TILE = 2 * C::A2_BYTES;                  // operand image: hi, lo
  // Inverse kernel shared memory.
  static constexpr uint32_t C2 = 0;                                  // hi, lo
  static constexpr uint32_t C1 = C2 + 2 * C::B2_BYTES;               // A hi, A lo, B hi, B lo
  static constexpr uint32_t A2 = (C1 + 4 * C::B1_BYTES + 1023) / 1024 * 1024;  // hi, lo (SWIZZLE_128B)
  // A1 shares A2's space: step 2' has read the operand tile before V writes
  // A1, and the next tile is loaded once step 1' has read A1. Three CTAs fit
  // on an SM.
  static constexpr uint32_t A1 = A2;                                 // [tile][hi, lo] (INTERLEAVE)
  // The second tile starts 64 B further than its hi + lo: in V the lanes of
  // the two tiles store to the same offsets, which then fall in different
  // banks.
  static constexpr uint32_t A1_STRIDE = 2 * C::A1_BYTES + 64;
  static constexpr uint32_t P = A2 + (C::T1 - 1) * A1_STRIDE + 2 * C::A1_BYTES;  // [2][TJ][PC] floats
  static constexpr uint32_t BAR = P + 2 * TJ * PC * 4;               // operand load, step 2', step 1'
  static constexpr uint32_t TSLOT = BAR + 24;
  static constexpr uint32_t BYTES = TSLOT + 8 + 1024;
  // Filter kernel shared memory.
  static constexpr uint32_t F_DC = C::G * FS * 8;
  static constexpr uint32_t F_BYTES = F_DC + C::G * 4;
  static_assert(C::T1 == 2, "one tile per block-column parity");
  static_assert(P >= A2 + TILE, "the operand tile fits below the partial sums");
  static_assert(A1_STRIDE % 16 == 0, "operand start addresses are 16-byte aligned");
  static_assert(BAR % 8 == 0 && P % 16 == 0, "alignment");
};

// Scale of a block sample after step 1': the inverse's 1/n^2 and kInvPre.
template <int N>
__host__ __device__ constexpr float out_scale() {
  return 1.0f / (kInvPre * N * N);
}

// Packs and stores samples x0 .. x0+W-1 (W = 8 or 16) of plane row y
// (bounds-checked), with 8- and 16-byte stores where the run is inside the
// plane and aligned.
template <int W>
__device__ __forceinline__ void emit_run(const SweepArgs& sa, int y, int x0, const float (&v)[W]) {
  static_assert(W == 8 || W == 16, "run width");
  if (y >= sa.inv.g.H) return;
  uint8_t* row = sa.dst + (long long)y * sa.pitch;
  const bool full = x0 + W <= sa.inv.g.W;
  if (full && sa.fmt == FMT_U16 && ((reinterpret_cast<uintptr_t>(row) + 2 * x0) & 15) == 0) {
    uint32_t w[W / 2];
#pragma unroll
    for (int k = 0; k < W / 2; k++)
      w[k] = pack_u16(v[2 * k] + sa.chroma_norm, sa.inv_norm, sa.max_pix) |
             (pack_u16(v[2 * k + 1] + sa.chroma_norm, sa.inv_norm, sa.max_pix) << 16);
    uint4* p = reinterpret_cast<uint4*>(row + 2 * x0);
#pragma unroll
    for (int k = 0; k < W / 8; k++) p[k] = make_uint4(w[4 * k], w[4 * k + 1], w[4 * k + 2], w[4 * k + 3]);
    return;
  }
  if (full && sa.fmt == FMT_U8 && ((reinterpret_cast<uintptr_t>(row) + x0) & (W - 1)) == 0) {
    uint32_t w[W / 4];
#pragma unroll
    for (int k = 0; k < W / 4; k++)
      w[k] = pack_u8(v[4 * k] + sa.chroma_norm) | (pack_u8(v[4 * k + 1] + sa.chroma_norm) << 8) |
             (pack_u8(v[4 * k + 2] + sa.chroma_norm) << 16) | (pack_u8(v[4 * k + 3] + sa.chroma_norm) << 24);
    if constexpr (W == 16) *reinterpret_cast<uint4*>(row + x0) = make_uint4(w[0], w[1], w[2], w[3]);
    else *reinterpret_cast<uint2*>(row + x0) = make_uint2(w[0], w[1]);
    return;
  }
#pragma unroll
  for (int k = 0; k < W; k++) {
    if (x0 + k >= sa.inv.g.W) break;
    float s = v[k];
    if (sa.chroma_norm != 0.0f) s += sa.chroma_norm;
    store_sample(row, x0 + k, s, sa.fmt, sa.inv_norm, sa.max_pix);
  }
}

// Bin j of a spectrum stored as float2 or, with half storage, as __half2.
template <bool HALF>
__device__ __forceinline__ float2 spec_at(const float2* s, size_t j) {
  if constexpr (HALF) return __half22float2(reinterpret_cast<const __half2*>(s)[j]);
  else return s[j];
}

// R. Row (k', block), K = 2 ky + (re, im) of the operand image of a group
// from its filtered bins fbuf[block][bin], in 16-byte chunks of 4 ky, into
// img. prev (optional) also receives block 0, as the previous strip's block
// 7; with skip_last the group's block 7 is not written (the next strip
// writes it).
template <int N>
__device__ __forceinline__ void tile_rows(uint8_t* img, uint8_t* prev, bool skip_last, const float2* fbuf,
                                          int tid) {
  using C = TcCfg<N>;
  using S = SwpCfg<N>;
  const int r2 = tid & 127, h = tid >> 7;
  const int kp = r2 / C::G, bl = r2 % C::G;
  if (bl == C::G - 1 && skip_last) return;
  const float2* fb = fbuf + bl * S::FS;
#pragma unroll
  for (int cq = 0; cq < C::NY / 4; cq++) {
    uint32_t hi[4], lo[4];
#pragma unroll
    for (int u = 0; u < 4; u++) {
      const int ky = C::NY * h + 4 * cq + u;
      float2 z;
      if (kp == 0) {
        const int kym = (N - ky) & (N - 1);
        const float2 f0 = fb[ky * C::FBW], f0m = fb[kym * C::FBW];
        const float2 fn = fb[ky * C::FBW + C::NY], fnm = fb[kym * C::FBW + C::NY];
        const float h0x = 0.5f * (f0.x + f0m.x), h0y = 0.5f * (f0.y - f0m.y);
        const float hnx = 0.5f * (fn.x + fnm.x), hny = 0.5f * (fn.y - fnm.y);
        z = make_float2(h0x - hny, h0y + hnx);
      } else {
        z = fb[ky * C::FBW + kp];
      }
      tc::split_pair(z.x * kInvPre, z.y * kInvPre, hi[u], lo[u]);
    }
    const uint32_t o = a2_off<N>(r2, 2 * (C::NY * h + 4 * cq));
    *reinterpret_cast<uint4*>(img + o) = make_uint4(hi[0], hi[1], hi[2], hi[3]);
    *reinterpret_cast<uint4*>(img + C::A2_BYTES + o) = make_uint4(lo[0], lo[1], lo[2], lo[3]);
    if (bl == 0 && prev) {
      const uint32_t op = a2_off<N>(r2 + C::G - 1, 2 * (C::NY * h + 4 * cq));
      *reinterpret_cast<uint4*>(prev + op) = make_uint4(hi[0], hi[1], hi[2], hi[3]);
      *reinterpret_cast<uint4*>(prev + C::A2_BYTES + op) = make_uint4(lo[0], lo[1], lo[2], lo[3]);
    }
  }
}

// The operand image of group (m, strip) in HBM: block 0 also goes to the
// previous strip's tile as its block 7; this tile's block 7 comes from the
// next strip.
template <int N>
__device__ __forceinline__ void operand_tile(const SweepArgs& sa, int m, int strip, const float2* fbuf, int tid) {
  using S = SwpCfg<N>;
  uint8_t* img = sa.img + ((size_t)m * sa.strips + strip) * S::TILE;
  tile_rows<N>(img, strip > 0 ? img - S::TILE : nullptr, strip != sa.strips - 1, fbuf, tid);
}

// Start of a group's filter: its window spectra begin moving into L2 as
// whole runs (of shifted windows, only the newest frame: the others are an
// earlier output's), and the current frame's DC of each block (the degrid
// correction's scale) goes to dcs. gb0: the group's first bin; nvbin: the
// bins filtered.
template <int N, int NF, bool HALF>
__device__ __forceinline__ void group_start(const SweepArgs& sa, size_t gb0, int nvbin, bool shifted, int m, int J0,
                                            float* dcs, int tid) {
  using C = TcCfg<N>;
  const InvArgs& a = sa.inv;
  constexpr uint32_t BIN_BYTES = HALF ? 4 : 8;
  const bool pull = !shifted || tid == NF - 1;
  if (tid < NF && nvbin > 0 && pull)
    tc::prefetch_l2(reinterpret_cast<const uint8_t*>(a.s[tid]) + gb0 * BIN_BYTES, (uint32_t)(nvbin * BIN_BYTES));
  if (tid < C::G) {
    const int n = J0 + tid;
    dcs[tid] = (a.dg && n <= sa.cells_x && n < a.g.ncols)
                   ? spec_at<HALF>(a.s[a.cur], (size_t)(m * a.g.ncols + n) * C::PS).x
                   : 0.0f;
  }
}

// F. The temporal filter (filter_vals, fast form) of a group's nvb blocks
// into fbuf[block][bin] (blocks nvb.. get zeros). Thread t filters bin
// li = t + 256 r (r < NL) of every block of the group, the bin's tables read
// once for all blocks, then tail item q: bin NL * 256 + e % TAIL of block
// e / TAIL, e = t + 256 q. The spectra loads of BATCH blocks are issued
// together; every index is the thread's base plus a constant.
template <int N, int BM, int BATCH, bool HALF>
__device__ __forceinline__ void filter_group(const InvArgs& a, size_t gb0, int nvb, const float* dcs, float2* fbuf,
                                             int tid) {
  using C = TcCfg<N>;
  using S = SwpCfg<N>;
  constexpr int NF = BM >= 2 ? BM : 1;
  constexpr int NL = C::PS / kTcThreads;
  constexpr int TAIL = C::PS - NL * kTcThreads;
  constexpr int NT = TAIL * C::G / kTcThreads;
  static_assert((TAIL * C::G) % kTcThreads == 0, "tail bins per thread");
  static_assert(C::G % BATCH == 0, "load batches");
  const size_t gt = gb0 + tid;
  if constexpr (NL > 0) {
    BinTables tb[NL];
#pragma unroll
    for (int r = 0; r < NL; r++) tb[r] = bin_tables(a, tid + kTcThreads * r);
#pragma unroll
    for (int b0 = 0; b0 < C::G; b0 += BATCH) {
      float2 sv[BATCH][NL][4];
#pragma unroll
      for (int u = 0; u < BATCH; u++) {
        if (b0 + u >= nvb) continue;
#pragma unroll
        for (int r = 0; r < NL; r++)
#pragma unroll
          for (int k = 0; k < NF; k++)
            sv[u][r][k] = spec_at<HALF>(a.s[k], gt + (size_t)(b0 + u) * C::PS + kTcThreads * r);
      }
#pragma unroll
      for (int u = 0; u < BATCH; u++) {
        const int b = b0 + u;
        const float dc = dcs[b];
#pragma unroll
        for (int r = 0; r < NL; r++) {
          const int li = tid + kTcThreads * r;
          float2 f = make_float2(0.0f, 0.0f);
          if (b < nvb) f = filter_vals_t<BM, true>(a, dc, tb[r], gb0 + (size_t)b * C::PS + li, sv[u][r]);
          fbuf[b * S::FS + li] = f;
        }
      }
    }
  }
#pragma unroll
  for (int q = 0; q < NT; q++) {
    const int e = tid + kTcThreads * q;
    const int b = e / TAIL, li = NL * kTcThreads + e % TAIL;
    float2 f = make_float2(0.0f, 0.0f);
    if (b < nvb) {
      float2 sv[4];
#pragma unroll
      for (int k = 0; k < NF; k++) sv[k] = spec_at<HALF>(a.s[k], gb0 + (size_t)b * C::PS + li);
      f = filter_vals_t<BM, true>(a, dcs[b], bin_tables(a, li), gb0 + (size_t)b * C::PS + li, sv);
    }
    fbuf[b * S::FS + li] = f;
  }
}

template <int N, int BM, int MINB, bool HALF>
__global__ void __launch_bounds__(kTcThreads, MINB) k_filter_tc(const __grid_constant__ SweepBatch B) {
  using C = TcCfg<N>;
  using S = SwpCfg<N>;
  // A run of planes of one geometry (e.g. consecutive frames of a plane)
  // runs the same group of each of its planes back to back, so that the
  // window spectra they share are read from L2 the second time.
  const int r0 = B.run[plane_of(B, B.cta0, blockIdx.x)];
  const int rl = B.rlen[r0];
  const int local = (int)blockIdx.x - B.cta0[r0];
  const int pl = r0 + local % rl;
  const SweepArgs& sa = B.p[pl];
  const int cta = local / rl;
  const InvArgs& a = sa.inv;
  extern __shared__ __align__(16) uint8_t smem_f[];
  float2* fbuf = reinterpret_cast<float2*>(smem_f);
  float* dcs = reinterpret_cast<float*>(smem_f + S::F_DC);
  const int tid = threadIdx.x;
  const int strip = cta % sa.strips, m = cta / sa.strips;
  const int J0 = strip * S::TJ;
  const int ncols = a.g.ncols;
  // A tile's eighth block is the next strip's first: that strip filters it
  // and writes it into both tiles, so each block is filtered once. The last
  // strip filters its own eighth block.
  const bool last_strip = strip == sa.strips - 1;
  const int own = last_strip ? C::G : C::G - 1;
  const int nvb = max(0, min(own, min(sa.cells_x + 1, ncols) - J0));  // blocks filtered here
  constexpr int NF = BM >= 2 ? BM : 1;  // window frames read
  const size_t gb0 = ((size_t)m * ncols + J0) * C::PS;
  group_start<N, NF, HALF>(sa, gb0, nvb * C::PS, (B.shifted >> pl) & 1, m, J0, dcs, tid);
  __syncthreads();
  filter_group<N, BM, filter_batch(MINB), HALF>(a, gb0, nvb, dcs, fbuf, tid);
  __syncthreads();
  operand_tile<N>(sa, m, strip, fbuf, tid);
}

// Shared-memory and barrier state of the inverse phases of one CTA.
struct InvState {
  uint8_t* sm;
  uint32_t sbase;
  uint64_t* bar;  // [1] column-inverse products, [2] row-inverse products
  uint32_t tmem;
  uint32_t phase;
  float* P_old;   // cell partial sums of block row m - 1 (finished by this row's top halves)
  float* P_new;   // cell partial sums of block row m
};

// The inverse of block row m once its operand tile is in shared memory (A2):
// step 2' (column inverse, tensor cores), V, step 1' (row inverse with the
// synthesis windows, tensor cores), then `after` (the tile's space is free
// again), then O (overlap-add in the reference's block order, finished cell
// rows packed to the output, segment seams). Returns false when a wait gave
// up (the error word has its bit); every thread of the CTA returns the same.
template <int N, class After>
__device__ __forceinline__ bool inverse_row(const SweepArgs& sa, InvState& st, int m, int M0, int M1, int seg, int J0,
                                            int ncell, After after) {
  using C = TcCfg<N>;
  using S = SwpCfg<N>;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  uint8_t* sm = st.sm;
  const uint32_t sbase = st.sbase;
  uint64_t* bar = st.bar;
  const uint32_t tmem = st.tmem;
  if (tid == 0) {
    tc::fence_after_sync();
    constexpr uint32_t id2 = tc::idesc_f16(128, C::N2);
    const uint32_t sbo_b = (C::K2 / 8) * 128;
    const uint32_t d = tmem + C::D2_COL;
    for (int ks = 0; ks < C::K2 / 16; ks++) {
      const uint64_t ah = a2_desc<N>(sbase + S::A2, ks);
      const uint64_t al = a2_desc<N>(sbase + S::A2 + C::A2_BYTES, ks);
      const uint64_t bh = tc::sdesc(sbase + S::C2 + ks * 256, 128, sbo_b, tc::LAYOUT_INTERLEAVE);
      const uint64_t bl = tc::sdesc(sbase + S::C2 + C::B2_BYTES + ks * 256, 128, sbo_b, tc::LAYOUT_INTERLEAVE);
      tc::mma_f16(d, ah, bh, id2, ks > 0);
      tc::mma_f16(d, ah, bl, id2, 1);
      tc::mma_f16(d, al, bh, id2, 1);
    }
    tc::mma_commit(&bar[1]);
  }
  if (!__syncthreads_and(tc::mbar_wait(&bar[1], st.phase, kWaitNs))) {
    if (tid == 0) atomicOr(sa.err, kErrWaitColumn);
    return false;
  }
  tc::fence_after_sync();

  // V. Row-inverse operand: tile = parity of the block column, row (y, slot).
  {
    const int s = warp & 3, h = warp >> 2;
    const int r2 = 32 * s + lane;
    const int kp = r2 / C::G, bl = r2 % C::G;
    const int tile = (J0 + bl) & 1, slot = bl >> 1;
    uint8_t* t0 = sm + S::A1 + tile * S::A1_STRIDE;
    float v[N];  // half of the N2 = 2N columns: NY values of y, (re, im)
    tc::tmem_ld<N>(tmem + ((uint32_t)(32 * s) << 16) + C::D2_COL + N * h, v);
#pragma unroll
    for (int j = 0; j < C::NY; j++) {
      const int y = C::NY * h + j;
      uint32_t hi, lo;
      tc::split_pair(v[2 * j], v[2 * j + 1], hi, lo);
      const uint32_t o = tc::off_il((C::G / 2) * y + slot, 2 * kp, C::K1);
      *reinterpret_cast<uint32_t*>(t0 + o) = hi;
      *reinterpret_cast<uint32_t*>(t0 + C::A1_BYTES + o) = lo;
    }
  }
  tc::fence_async_smem();
  tc::fence_before_sync();
  __syncthreads();

  // Step 1' on the tensor cores: D1[tile] = A1[tile] * C1(tile)^T.
  if (tid == 0) {
    tc::fence_after_sync();
    constexpr uint32_t id1 = tc::idesc_f16(128, C::N1);
    const uint32_t sbo = (C::K1 / 8) * 128;
    for (int t = 0; t < C::T1; t++) {
      const uint32_t a_hi = sbase + S::A1 + t * S::A1_STRIDE, a_lo = a_hi + C::A1_BYTES;
      const uint32_t b_hi = sbase + S::C1 + t * 2 * C::B1_BYTES, b_lo = b_hi + C::B1_BYTES;
      const uint32_t d = tmem + C::D1_COL + t * C::N1;
      for (int ks = 0; ks < C::K1 / 16; ks++) {
        const uint64_t ah = tc::sdesc(a_hi + ks * 256, 128, sbo, tc::LAYOUT_INTERLEAVE);
        const uint64_t al = tc::sdesc(a_lo + ks * 256, 128, sbo, tc::LAYOUT_INTERLEAVE);
        const uint64_t bh = tc::sdesc(b_hi + ks * 256, 128, sbo, tc::LAYOUT_INTERLEAVE);
        const uint64_t bl = tc::sdesc(b_lo + ks * 256, 128, sbo, tc::LAYOUT_INTERLEAVE);
        tc::mma_f16(d, ah, bh, id1, ks > 0);
        tc::mma_f16(d, ah, bl, id1, 1);
        tc::mma_f16(d, al, bh, id1, 1);
      }
    }
    tc::mma_commit(&bar[2]);
  }
  if (!__syncthreads_and(tc::mbar_wait(&bar[2], st.phase, kWaitNs))) {
    if (tid == 0) atomicOr(sa.err, kErrWaitRow);
    return false;
  }
  st.phase ^= 1;
  tc::fence_after_sync();
  after();

  // O. Overlap-add. Thread: block row y of block bl; y < n/2 finishes cell
  // row m-1 (P_old), y >= n/2 starts cell row m (P_new).
  float* P_old = st.P_old;
  float* P_new = st.P_new;
  {
    const int t = warp >> 2, s = warp & 3;
    const int r = 32 * s + lane;
    const int y = r / (C::G / 2), slot = r % (C::G / 2);
    const int bl = 2 * slot + ((t ^ J0) & 1);
    float v[N];
    tc::tmem_ld<N>(tmem + ((uint32_t)(32 * s) << 16) + C::D1_COL + t * C::N1, v);
#pragma unroll
    for (int x = 0; x < N; x++) v[x] *= out_scale<N>();
    const bool top = y < S::CH;
    const int yy = top ? y : y - S::CH;
    const bool right_ok = bl < ncell;                // right half -> cell bl
    const bool left_ok = bl >= 1 && bl - 1 < ncell;  // left half -> cell bl-1
    const bool seam_top = m == M0;                   // cell row m-1 is another segment's (or none)
    if (top) {
      if (seam_top) {
        if (M0 > 0 && right_ok) {
          float* t0 = sa.seam_t + ((size_t)((seg - 1) * 2) * S::CH + yy) * sa.seam_w + (J0 + bl) * S::CW;
#pragma unroll
          for (int x = 0; x < S::CW; x += 4)
            *reinterpret_cast<float4*>(t0 + x) = make_float4(v[S::CW + x], v[S::CW + x + 1], v[S::CW + x + 2], v[S::CW + x + 3]);
        }
      } else if (right_ok) {
        float* p = P_old + bl * S::PC + yy * S::PR;
#pragma unroll
        for (int x = 0; x < S::CW; x += 4) {
          float4 q = *reinterpret_cast<float4*>(p + x);
          q.x += v[S::CW + x], q.y += v[S::CW + x + 1], q.z += v[S::CW + x + 2], q.w += v[S::CW + x + 3];
          *reinterpret_cast<float4*>(p + x) = q;
        }
      }
    } else if (right_ok) {
      float* p = P_new + bl * S::PC + yy * S::PR;
#pragma unroll
      for (int x = 0; x < S::CW; x += 4)
        *reinterpret_cast<float4*>(p + x) = make_float4(v[S::CW + x], v[S::CW + x + 1], v[S::CW + x + 2], v[S::CW + x + 3]);
    }
    __syncthreads();
    if (top) {
      if (seam_top) {
        if (M0 > 0 && left_ok) {
          float* t1 = sa.seam_t + ((size_t)((seg - 1) * 2 + 1) * S::CH + yy) * sa.seam_w + (J0 + bl - 1) * S::CW;
#pragma unroll
          for (int x = 0; x < S::CW; x += 4)
            *reinterpret_cast<float4*>(t1 + x) = make_float4(v[x], v[x + 1], v[x + 2], v[x + 3]);
        }
      } else if (left_ok) {
        const float* p = P_old + (bl - 1) * S::PC + yy * S::PR;
        float o[S::CW];
#pragma unroll
        for (int x = 0; x < S::CW; x += 4) {
          const float4 q = *reinterpret_cast<const float4*>(p + x);
          o[x] = q.x + v[x], o[x + 1] = q.y + v[x + 1], o[x + 2] = q.z + v[x + 2], o[x + 3] = q.w + v[x + 3];
        }
        emit_run<S::CW>(sa, (m - 1) * S::CH + yy, (J0 + bl - 1) * S::CW, o);
      }
    } else if (left_ok) {
      float* p = P_new + (bl - 1) * S::PC + yy * S::PR;
      const bool seam_bot = m == M1 - 1 && seg < sa.segs - 1;
      float* sb = sa.seam_b + ((size_t)seg * S::CH + yy) * sa.seam_w + (J0 + bl - 1) * S::CW;
#pragma unroll
      for (int x = 0; x < S::CW; x += 4) {
        float4 q = *reinterpret_cast<float4*>(p + x);
        q.x += v[x], q.y += v[x + 1], q.z += v[x + 2], q.w += v[x + 3];
        if (seam_bot) *reinterpret_cast<float4*>(sb + x) = q;
        else *reinterpret_cast<float4*>(p + x) = q;
      }
    }
  }
  st.P_old = P_new;
  st.P_new = P_old;
  tc::fence_before_sync();
  __syncthreads();
  return true;
}

// Constant operands of the inverse (C2 hi, lo, then C1 A hi, lo, B hi, lo)
// into shared memory, tensor memory and the barriers.
template <int N>
__device__ __forceinline__ void inverse_setup(const SweepArgs& sa, uint8_t* sm, uint64_t* bar, uint32_t* tslot) {
  using C = TcCfg<N>;
  using S = SwpCfg<N>;
  using T = TcTab<N>;
  const int tid = threadIdx.x;
  const uint4* src2 = reinterpret_cast<const uint4*>(sa.tab + T::C2HI);
  uint4* dst2 = reinterpret_cast<uint4*>(sm + S::C2);
  for (int i = tid; i < (int)(2 * C::B2_BYTES / 16); i += kTcThreads) dst2[i] = src2[i];
  const uint4* src1 = reinterpret_cast<const uint4*>(sa.tab + T::C1AHI);
  uint4* dst1 = reinterpret_cast<uint4*>(sm + S::C1);
  for (int i = tid; i < (int)(4 * C::B1_BYTES / 16); i += kTcThreads) dst1[i] = src1[i];
  if ((tid >> 5) == 0) {
    tc::tmem_alloc(tslot, C::TMEM_COLS);
    tc::tmem_relinquish();
  }
  if (tid == 0) {
    for (int i = 0; i < 3; i++) tc::mbar_init(&bar[i], 1);
    tc::fence_mbar_init();
  }
}

template <int N>
__global__ void __launch_bounds__(kTcThreads, kTcSweepCtasPerSm) k_sweep_tc(const __grid_constant__ SweepBatch B) {
  using C = TcCfg<N>;
  using S = SwpCfg<N>;
  static_assert(sizeof(B) <= 32000, "kernel parameter space");
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t* sm = smem_raw + ((1024u - (tc::smem_u32(smem_raw) & 1023u)) & 1023u);
  uint64_t* bar = reinterpret_cast<uint64_t*>(sm + S::BAR);  // [0] operand load, [1] step 2', [2] step 1'
  uint32_t* tslot = reinterpret_cast<uint32_t*>(sm + S::TSLOT);
  const int tid = threadIdx.x, warp = tid >> 5;

  const int pl = plane_of(B, B.cta0, blockIdx.x);
  const SweepArgs& sa = B.p[pl];
  const int cta = blockIdx.x - B.cta0[pl];
  const int strip = cta % sa.strips, seg = cta / sa.strips;
  const int J0 = strip * S::TJ;
  const int nrow = sa.cells_y + 1;
  const int M0 = (int)((long long)seg * nrow / sa.segs);
  const int M1 = (int)((long long)(seg + 1) * nrow / sa.segs);
  const int ncell = min(S::TJ, sa.cells_x - J0);
  auto tile_of = [&](int m) { return sa.img + ((size_t)m * sa.strips + strip) * S::TILE; };

  inverse_setup<N>(sa, sm, bar, tslot);
  if (tid == 0) {
    tc::fence_async_smem();
    if (M0 < M1) {
      tc::mbar_expect_tx(&bar[0], S::TILE);
      // A test of the bounded wait leaves this copy out: nothing is then in
      // flight on the barrier, the wait below gives up and the CTA leaves.
      if (!(sa.test_skip && cta == 0)) tc::bulk_load(sm + S::A2, tile_of(M0), S::TILE, &bar[0]);
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  InvState st{sm, tc::smem_u32(sm), bar, *tslot, 0u, reinterpret_cast<float*>(sm + S::P),
              reinterpret_cast<float*>(sm + S::P) + S::TJ * S::PC};

  for (int m = M0; m < M1; m++) {
    // The operand tile of row m arrives by bulk copy (issued while the
    // previous row's overlap-add ran).
    if (!__syncthreads_and(tc::mbar_wait(&bar[0], st.phase, kWaitNs))) {
      if (tid == 0) atomicOr(sa.err, kErrWaitTile);
      break;
    }
    // A1 (the operand tile's space) is consumed once step 1' is done: the
    // next row's tile starts moving in while the overlap-add runs.
    const bool ok = inverse_row<N>(sa, st, m, M0, M1, seg, J0, ncell, [&] {
      if (tid == 0 && m + 1 < M1) {
        tc::mbar_expect_tx(&bar[0], S::TILE);
        tc::bulk_load(sm + S::A2, tile_of(m + 1), S::TILE, &bar[0]);
      }
    });
    if (!ok) break;
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  if (warp == 0) tc::tmem_dealloc(st.tmem, C::TMEM_COLS);
}

template <class K>
cudaError_t prepare(K k, size_t smem) {
  return cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
}

int sm_count() {
  int dev = 0, n = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
  return n > 0 ? n : 1;
}

// Host-side fp16 hi/lo split of a double.
void split_h(double v, __half& hi, __half& lo) {
  hi = __float2half_rn((float)v);
  lo = __float2half_rn((float)(v - (double)__half2float(hi)));
}
void put_pair(std::vector<uint8_t>& t, uint32_t hi_base, uint32_t lo_base, uint32_t off, double v) {
  __half h, l;
  split_h(v, h, l);
  std::memcpy(t.data() + hi_base + off, &h, 2);
  std::memcpy(t.data() + lo_base + off, &l, 2);
}

template <int N>
std::vector<uint8_t> tables_n(const std::vector<double>& wx, const std::vector<double>& wy,
                              const std::vector<double>& sxa, const std::vector<double>& sxb,
                              const std::vector<double>& sy) {
  using T = TcTab<N>;
  constexpr int NY = N / 2, FBW = NY + 1;
  std::vector<uint8_t> t(T::TOTAL, 0);
  auto cs = [](int k, int x, double& c, double& s) {
    const double th = 2.0 * kPiD * (double)((k * x) % N) / N;
    c = std::cos(th);
    s = std::sin(th);
  };
  // Packed real row transform coefficient j at x: 1, (-1)^x, cos, -sin.
  auto row_coef = [&](int j, int x) {
    if (j == 0) return 1.0;
    if (j == 1) return (x & 1) ? -1.0 : 1.0;
    double c, s;
    cs(j / 2, x, c, s);
    return (j & 1) ? -s : c;
  };
  // B1 [j][x]: packed real row DFT, analysis x-window folded in.
  for (int j = 0; j < N; j++)
    for (int x = 0; x < N; x++) put_pair(t, T::B1HI, T::B1LO, tc::off_il(j, x, N), row_coef(j, x) * wx[x]);
  // B2 [2ky+ro][2y+ri]: complex column DFT, analysis y-window folded in.
  for (int ky = 0; ky < N; ky++)
    for (int y = 0; y < N; y++) {
      double c, s;
      cs(ky, y, c, s);
      const double w = wy[y];
      put_pair(t, T::B2HI, T::B2LO, tc::off_il(2 * ky, 2 * y, 2 * N), w * c);
      put_pair(t, T::B2HI, T::B2LO, tc::off_il(2 * ky, 2 * y + 1, 2 * N), w * s);
      put_pair(t, T::B2HI, T::B2LO, tc::off_il(2 * ky + 1, 2 * y, 2 * N), -w * s);
      put_pair(t, T::B2HI, T::B2LO, tc::off_il(2 * ky + 1, 2 * y + 1, 2 * N), w * c);
    }
  // Spectrum of the analysis window (the chroma offset's contribution): the
  // window is separable, so it is the product of the two axes' DFTs.
  std::vector<double> ayr(N), ayi(N), axr(FBW), axi(FBW);
  for (int k = 0; k < N; k++)
    for (int j = 0; j < N; j++) {
      double c, s;
      cs(k, j, c, s);
      ayr[k] += wy[j] * c;
      ayi[k] -= wy[j] * s;
      if (k < FBW) {
        axr[k] += wx[j] * c;
        axi[k] -= wx[j] * s;
      }
    }
  for (int ky = 0; ky < N; ky++)
    for (int kx = 0; kx < FBW; kx++) {
      const float f[2] = {(float)(ayr[ky] * axr[kx] - ayi[ky] * axi[kx]),
                          (float)(ayr[ky] * axi[kx] + ayi[ky] * axr[kx])};
      std::memcpy(t.data() + T::WSPEC + (ky * FBW + kx) * 8, f, 8);
    }
  // C2 [2y+ro][2ky+ri]: complex column inverse DFT (unnormalised), synthesis
  // y-window folded in.
  for (int y = 0; y < N; y++)
    for (int ky = 0; ky < N; ky++) {
      double c, s;
      cs(ky, y, c, s);
      const double w = sy[y];
      put_pair(t, T::C2HI, T::C2LO, tc::off_il(2 * y, 2 * ky, 2 * N), w * c);
      put_pair(t, T::C2HI, T::C2LO, tc::off_il(2 * y, 2 * ky + 1, 2 * N), -w * s);
      put_pair(t, T::C2HI, T::C2LO, tc::off_il(2 * y + 1, 2 * ky, 2 * N), w * s);
      put_pair(t, T::C2HI, T::C2LO, tc::off_il(2 * y + 1, 2 * ky + 1, 2 * N), w * c);
    }
  // C1 [x][j]: real row inverse from the packed half spectrum (twice the
  // cos/sin terms: the mirrored columns), synthesis x-window folded in.
  for (int x = 0; x < N; x++)
    for (int j = 0; j < N; j++) {
      const double v = j < 2 ? row_coef(j, x) : 2.0 * row_coef(j, x);
      put_pair(t, T::C1AHI, T::C1ALO, tc::off_il(x, j, N), v * sxa[x]);
      put_pair(t, T::C1BHI, T::C1BLO, tc::off_il(x, j, N), v * sxb[x]);
    }
  return t;
}

}  // namespace

bool tc_supported(int mode, int bw, int bh, int bm) {
  return mode == 1 && bw == bh && (bw == 16 || bw == 32) && bm != 0;
}

int tc_group_blocks(int n) { return 128 / (n / 2); }
int tc_sweep_cells(int n) { return tc_group_blocks(n) - 1; }

static_assert(TcCfg<32>::G == 8 && TcCfg<16>::G == 16, "forward group sizes of the batch plan");

std::vector<uint8_t> tc_tables(int n, const std::vector<double>& wx, const std::vector<double>& wy,
                               const std::vector<double>& sxa, const std::vector<double>& sxb,
                               const std::vector<double>& sy) {
  for (const auto* v : {&wx, &wy, &sxa, &sxb, &sy})
    if ((int)v->size() != n) return {};
  if (n == 32) return tables_n<32>(wx, wy, sxa, sxb, sy);
  if (n == 16) return tables_n<16>(wx, wy, sxa, sxb, sy);
  return {};
}

namespace {

template <int N>
cudaError_t launch_forward_n(const TcFwdBatch& B, const TcFwdArgs* planes, int n, const TcTune& t,
                             cudaStream_t st) {
  // The split kernel (hi + lo step-1 operand) also takes planes that need no
  // split; it fits two CTAs per SM, the other three.
  bool split = false;
  for (int i = 0; i < n; i++) split = split || planes[i].split;
  const int fmt = planes[0].fmt;
  if (fmt == FMT_U8 && split) return cudaErrorNotSupported;
  auto k = fmt == FMT_U8 ? k_forward_tc<N, 1, false>
           : fmt == FMT_U16 ? (split ? k_forward_tc<N, 2, true> : k_forward_tc<N, 2, false>)
                            : k_forward_tc<N, 4, true>;
  const size_t smem = split ? FwdSmem<N, true>::BYTES : FwdSmem<N, false>::BYTES;
  cudaError_t attr = prepare(k, smem);
  if (attr != cudaSuccess) return attr;
  const int ngroups = B.grp0[n];
  if (ngroups == 0) return cudaSuccess;
  const int per_sm = std::max(1, std::min(t.fwd_ctas_per_sm, split ? 2 : kFwdMaxCtasPerSm));
  static_assert(kFwdMaxCtasPerSm * (FwdSmem<N, false>::BYTES + 1024) <= 228 * 1024, "CTAs per SM");
  static_assert(2 * (FwdSmem<N, true>::BYTES + 1024) <= 228 * 1024, "CTAs per SM");
  const int grid = std::min(ngroups, per_sm * sm_count());
  k<<<grid, kTcThreads, smem, st>>>(B);
  count_launch();
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_forward_tc_batch(const TcFwdArgs* planes, int n, const TcTune& t, cudaStream_t st) {
  TcFwdBatch B;
  if (!forward_batch(planes, n, B)) return n < 1 || n > kMaxBatch ? cudaErrorInvalidValue : cudaErrorNotSupported;
  return planes[0].g.bw == 16 ? launch_forward_n<16>(B, planes, n, t, st) : launch_forward_n<32>(B, planes, n, t, st);
}

cudaError_t launch_forward_tc(const TcFwdArgs& a, cudaStream_t st) { return launch_forward_tc_batch(&a, 1, TcTune{}, st); }

template <int N, int BM, int MINB, bool HALF>
cudaError_t launch_filter_bm(const SweepBatch& B, cudaStream_t st) {
  constexpr size_t smem = SwpCfg<N>::F_BYTES;
  auto k = k_filter_tc<N, BM, MINB, HALF>;
  cudaError_t e = prepare(k, smem);
  if (e != cudaSuccess) return e;
  if (B.cta0[B.n] == 0) return cudaSuccess;
  k<<<B.cta0[B.n], kTcThreads, smem, st>>>(B);
  count_launch();
  return cudaGetLastError();
}

template <int N, int MINB, bool HALF>
cudaError_t launch_filter_h(const SweepBatch& B, int bm, cudaStream_t st) {
  switch (bm) {
  case -1: return launch_filter_bm<N, -1, MINB, HALF>(B, st);
  case 1: return launch_filter_bm<N, 1, MINB, HALF>(B, st);
  case 2: return launch_filter_bm<N, 2, MINB, HALF>(B, st);
  case 3: return launch_filter_bm<N, 3, MINB, HALF>(B, st);
  case 4: return launch_filter_bm<N, 4, MINB, HALF>(B, st);
  default: return cudaErrorNotSupported;
  }
}

// The planes of a batch store their spectra alike, fp32 or fp16 (sweep_batches checks).
template <int N, int MINB>
cudaError_t launch_filter(const SweepBatch& B, int bm, cudaStream_t st) {
  return B.p[0].inv.half ? launch_filter_h<N, MINB, true>(B, bm, st) : launch_filter_h<N, MINB, false>(B, bm, st);
}

// Finishes the seam cell rows of every plane of the batch: blockIdx.z runs
// over all planes' seams (prefix in cta0), the sum as in k_seam_merge
// (f3d_k_sweep.cu): ((q1 + q2) + q3) + q4, packed.
__global__ void __launch_bounds__(256) k_seam_merge_batch(const __grid_constant__ SweepBatch B, int ch) {
  const int pl = plane_of(B, B.cta0, blockIdx.z);
  const SweepArgs& sa = B.p[pl];
  const int k = blockIdx.z - B.cta0[pl];
  const int x = blockIdx.x * 256 + threadIdx.x;
  const int yy = blockIdx.y;
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

namespace {

template <int N>
cudaError_t launch_sweep_n(const SweepBatch& Bf, const SweepBatch& B, const SweepBatch& Bm, int n, int maxw,
                           const TcTune& t, cudaStream_t st, cudaEvent_t mark, cudaEvent_t after_filter) {
  using S = SwpCfg<N>;
  const int bm = B.p[0].inv.bm;
  constexpr size_t smem = S::BYTES;
  static_assert(kTcSweepCtasPerSm * (S::BYTES + 1024) <= 228 * 1024, "CTAs per SM");
  // Filter: one CTA per (row, strip) group of every plane.
  cudaError_t e = t.filter_minb == 3   ? launch_filter<N, 3>(Bf, bm, st)
                  : t.filter_minb == 4 ? launch_filter<N, 4>(Bf, bm, st)
                                       : launch_filter<N, 5>(Bf, bm, st);
  if (e != cudaSuccess) return e;
  if (mark) cudaEventRecord(mark, st);
  if (after_filter && (e = cudaEventRecord(after_filter, st)) != cudaSuccess) return e;
  // Inverse + overlap-add: one CTA per (strip, segment) of every plane.
  e = prepare(k_sweep_tc<N>, smem);
  if (e != cudaSuccess) return e;
  k_sweep_tc<N><<<B.cta0[n], kTcThreads, smem, st>>>(B);
  count_launch();
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  // Seam rows of all planes.
  if (Bm.cta0[n] == 0) return cudaSuccess;
  dim3 grid((maxw + 255) / 256, S::CH, Bm.cta0[n]);
  k_seam_merge_batch<<<grid, 256, 0, st>>>(Bm, S::CH);
  count_launch();
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_seam_merge_batch(const SweepBatch& Bm, int n, int maxw, int ch, cudaStream_t st) {
  if (Bm.cta0[n] == 0) return cudaSuccess;
  dim3 grid((maxw + 255) / 256, ch, Bm.cta0[n]);
  k_seam_merge_batch<<<grid, 256, 0, st>>>(Bm, ch);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_sweep_tc_batch(const SweepArgs* planes, int n, const TcTune& t, cudaStream_t st,
                                  cudaEvent_t mark, cudaEvent_t after_filter) {
  SweepBatch Bf, B, Bm;
  if (!sweep_batches(planes, n, Bf, B, Bm)) return n < 1 || n > kMaxBatch ? cudaErrorInvalidValue : cudaErrorNotSupported;
  int maxw = 0;
  for (int i = 0; i < n; i++) maxw = std::max(maxw, planes[i].inv.g.W);
  static_assert(SwpCfg<32>::TJ == 7 && SwpCfg<16>::TJ == 15, "cells per strip");
  return planes[0].inv.g.bw == 16 ? launch_sweep_n<16>(Bf, B, Bm, n, maxw, t, st, mark, after_filter)
                                  : launch_sweep_n<32>(Bf, B, Bm, n, maxw, t, st, mark, after_filter);
}

cudaError_t launch_sweep_tc(const SweepArgs& a, cudaStream_t st, cudaEvent_t mark) {
  return launch_sweep_tc_batch(&a, 1, TcTune{}, st, mark);
}

namespace {
template <int N, int MINB, bool HALF>
bool is_filter_h(const void* f) {
  return f == (const void*)k_filter_tc<N, -1, MINB, HALF> || f == (const void*)k_filter_tc<N, 1, MINB, HALF> ||
         f == (const void*)k_filter_tc<N, 2, MINB, HALF> || f == (const void*)k_filter_tc<N, 3, MINB, HALF> ||
         f == (const void*)k_filter_tc<N, 4, MINB, HALF>;
}
template <int N>
bool is_filter(const void* f) {
  return is_filter_h<N, 3, false>(f) || is_filter_h<N, 3, true>(f) || is_filter_h<N, 4, false>(f) ||
         is_filter_h<N, 4, true>(f) || is_filter_h<N, 5, false>(f) || is_filter_h<N, 5, true>(f);
}
template <int N>
bool is_forward(const void* f) {
  return f == (const void*)k_forward_tc<N, 1, false> || f == (const void*)k_forward_tc<N, 2, false> ||
         f == (const void*)k_forward_tc<N, 2, true> || f == (const void*)k_forward_tc<N, 4, true>;
}
}  // namespace

cudaError_t tc_graph_update(cudaGraphExec_t exec, cudaGraph_t graph, const TcFwdArgs* fwd, int nf,
                            const SweepArgs* sw, int ns) {
  TcFwdBatch Bw{};
  SweepBatch Bf, Bs, Bm;
  if (nf > 0 && !forward_batch(fwd, nf, Bw)) return cudaErrorNotSupported;
  if (ns > 0 && !sweep_batches(sw, ns, Bf, Bs, Bm)) return cudaErrorNotSupported;
  size_t cnt = 0;
  cudaError_t e = cudaGraphGetNodes(graph, nullptr, &cnt);
  if (e != cudaSuccess) return e;
  std::vector<cudaGraphNode_t> nodes(cnt);
  if ((e = cudaGraphGetNodes(graph, nodes.data(), &cnt)) != cudaSuccess) return e;
  int ch = (ns > 0 ? sw[0].inv.g.bh : 32) / 2;
  for (cudaGraphNode_t node : nodes) {
    cudaGraphNodeType ty;
    if ((e = cudaGraphNodeGetType(node, &ty)) != cudaSuccess) return e;
    if (ty != cudaGraphNodeTypeKernel) continue;
    cudaKernelNodeParams kp{};
    if ((e = cudaGraphKernelNodeGetParams(node, &kp)) != cudaSuccess) return e;
    void* args[2] = {nullptr, &ch};
    const void* f = kp.func;
    if (is_forward<32>(f) || is_forward<16>(f))
      args[0] = &Bw;
    else if (is_filter<32>(f) || is_filter<16>(f))
      args[0] = &Bf;
    else if (f == (const void*)k_sweep_tc<32> || f == (const void*)k_sweep_tc<16>)
      args[0] = &Bs;
    else if (f == (const void*)k_seam_merge_batch)
      args[0] = &Bm;
    else
      return cudaErrorInvalidValue;
    kp.kernelParams = args;
    kp.extra = nullptr;
    if ((e = cudaGraphExecKernelNodeSetParams(exec, node, &kp)) != cudaSuccess) return e;
  }
  return cudaSuccess;
}

size_t tc_image_bytes(const Geo& g, int strips) {
  const int cells_y = (g.H + g.bh / 2 - 1) / (g.bh / 2);
  const size_t tile = g.bw == 16 ? SwpCfg<16>::TILE : SwpCfg<32>::TILE;
  return (size_t)(cells_y + 1) * strips * tile;
}

}  // namespace f3d
