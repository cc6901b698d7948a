// f3d_kernels.hpp -- launch interface between the engine (host C++) and the
// CUDA kernels. Plain structs passed by value as __grid_constant__ kernel
// parameters, so tables that every thread reads with compile-time indices
// (the FFT twiddles) sit in the constant bank.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <vector>

namespace f3d {

// Plane geometry and block grid as the kernels see it.
struct Geo {
  int W, H;          // plane size in samples
  int bw, bh, fbw;   // block size, kept spectrum columns (bw/2+1)
  int nb;            // blocks in the plane
  int mode;          // 0: two offset grids, 1: overlapped grid
  int ncols, nrows;  // mode 1: blocks per row / rows; mode 0: nx, ny per grid
  int xoff, xstep, yoff, ystep;
};

// Sample formats of the raw planes.
enum Fmt : int { FMT_F32 = 0, FMT_U8 = 8, FMT_U16 = 16 };

// FFT twiddles of the reference plans (double -> float), N/2 entries each,
// for the row (bw) and column (bh) lengths up to 64 (larger blocks read them
// from device tables, FwdArgs/InvArgs::twr, twc).
struct Twiddles {
  float2 row[32];
  float2 col[32];
};

struct FwdArgs {
  Geo g;
  Twiddles tw;
  const uint8_t* src;  // plane in device memory
  long long pitch;     // bytes between rows
  int fmt;
  float norm;          // 16-bit: 2^(16-bits)/65535
  float chroma_norm;   // subtracted before windowing (mode-1 chroma)
  const float* win;    // analysis window, bw*bh
  float2* spec;        // out: nb x bh x fbw half spectra
  const float2* twr;   // blocks above 64: device twiddles, bw/2 and bh/2 entries
  const float2* twc;
};

struct InvArgs {
  Geo g;
  Twiddles tw;
  const float2* s[4];  // window spectra in temporal order (__half2 pairs when half)
  int half;            // spectra stored as fp16 pairs (tensor-core filter only)
  int cur;             // index of the current frame in s
  int bm;              // temporal mode -1..4
  int dg, pat, shp;    // degrid, sigma pattern, sharpen on
  int kalman_init;     // bt=0: first frame, state starts from s[0]
  const float2* gs;    // degrid sample, bh x fbw
  const float* pattern;
  const float* sharpen;
  float2* klast;       // Kalman state, nb x bh x fbw
  float* kcov;
  float* kproc;
  const float* win_a;  // synthesis window of even-parity blocks (mode 0: analysis window)
  const float* win_b;  // synthesis window of odd-parity blocks
  float* blocks;       // out: nb x bh x bw windowed blocks
  float sigma_x, sigma_y, beta_x, beta, ssmin, ssmax, kalman_cn, kr2;
  const float2* twr;   // blocks above 64: device twiddles, bw/2 and bh/2 entries,
  const float2* twc;   //   and nb x bh x bw complex work space
  float2* work;
};

struct OlaArgs {
  Geo g;
  const float* blocks;
  uint8_t* dst;
  long long pitch;
  int fmt;
  float chroma_norm, inv_norm, max_pix;
};

// Fused filter + inverse + overlap-add + packing for mode 1 with half
// overlap (bw = 2 ow, bh = 2 oh), the "sweep": the plane is cut into cells of
// (bw/2) x (bh/2) samples, each covered by exactly four blocks. A CTA owns a
// strip of cells and a range of block rows (a segment); it sweeps down the
// block rows, adding each row's windowed blocks to the cells in shared
// memory in the reference's block order, and writes finished cells straight
// to the output plane. Cell rows on the boundary between two segments are
// finished by a merge pass from the seam buffers.
struct SweepArgs {
  InvArgs inv;
  uint8_t* dst;          // output plane
  long long pitch;
  int fmt;
  float chroma_norm, inv_norm, max_pix;
  int cells_x, cells_y;  // cells covering the plane
  int strips, segs;      // CTA (strip, segment) grid
  int seam_w;            // floats per seam row (cells_x * bw/2)
  int prefetch;          // L2 prefetch of the next block row: 0 off, 1 at row start, 2 after the filter
  float* seam_b;         // [segs-1][bh/2][seam_w]: first two quadrants of each seam cell, summed
  float* seam_t;         // [segs-1][2][bh/2][seam_w]: third and fourth quadrants
  const uint8_t* tab;    // tensor-core form: device copy of tc_tables()
  int* err;              // tensor-core form: bits set when a wait gives up (kErrWait*)
  uint8_t* img;          // tensor-core form: filtered column-inverse operands, one tile per (row, strip)
  int test_skip;         // tests only: the plane's first CTA skips its first operand-tile copy
};

// Bits of the tensor-core kernels' error word: which wait gave up.
enum : int {
  kErrWaitForward = 1,  // forward: a group's tensor-core steps
  kErrWaitTile = 2,     // inverse: the operand tile copy
  kErrWaitColumn = 4,   // inverse: the column-inverse products
  kErrWaitRow = 8       // inverse: the row-inverse products
};

// Whether the sweep handles this geometry and form; its CTA grid; the seam
// scratch it needs (floats); and the launches (sweep, then merge).
bool sweep_supported(int form, const Geo& g, int bm);
void sweep_plan(int form, const Geo& g, int sm_count, int* strips, int* segs);
size_t sweep_seam_floats(const Geo& g, int segs);
// `mark` (optional) is recorded after the first kernel: the fast-form sweep,
// or the tensor-core filter kernel.
cudaError_t launch_sweep(int form, const SweepArgs& a, cudaStream_t st, cudaEvent_t mark = nullptr);

// Kernel launches; each returns the launch error. `form` is F3D_FORM_*.
cudaError_t launch_forward(int form, const FwdArgs& a, cudaStream_t st);
cudaError_t launch_filter_inverse(int form, const InvArgs& a, cudaStream_t st);
cudaError_t launch_ola(const OlaArgs& a, cudaStream_t st);
// True when kernels of this form exist for this block size.
bool form_supported(int form, int bw, int bh);

// Exact-form launchers, one translation unit per block width.
#define F3D_DECLARE_EXACT(BW)                                                        \
  cudaError_t launch_forward_exact_bw##BW(const FwdArgs& a, cudaStream_t st);        \
  cudaError_t launch_inverse_exact_bw##BW(const InvArgs& a, cudaStream_t st);
F3D_DECLARE_EXACT(4)
F3D_DECLARE_EXACT(8)
F3D_DECLARE_EXACT(16)
F3D_DECLARE_EXACT(32)
F3D_DECLARE_EXACT(64)
#undef F3D_DECLARE_EXACT

// Exact form for blocks above 64 (f3d_k_big.cu): one CTA per block,
// transforms through global memory.
bool big_block(int bw, int bh);
cudaError_t launch_forward_big(const FwdArgs& a, cudaStream_t st);
cudaError_t launch_inverse_big(const InvArgs& a, cudaStream_t st);

// Fast-form launchers (f3d_k_fast.cu).
cudaError_t launch_forward_fast(const FwdArgs& a, cudaStream_t st);
cudaError_t launch_inverse_fast(const InvArgs& a, cudaStream_t st);

// Tensor-core form (f3d_k_tc.cu): block transforms as DFT-matrix products on
// the tensor cores, fp16 operands split into hi + lo parts, fp32
// accumulation in tensor memory. Mode 1, square 16x16 or 32x32 blocks.
struct TcFwdArgs {
  Geo g;
  const uint8_t* src;  // plane in device memory
  long long pitch;
  int fmt;
  int split;           // 0: integer samples enter as fp16 exactly (8..11 bits); 1: hi + lo parts
  float norm;          // 16-bit normalisation (split path)
  float out_scale;     // applied to the spectra: 1/255 or norm on the integer path, 1 on the split path
  float chroma_norm;
  const uint8_t* tab;  // device copy of tc_tables()
  float2* spec;        // out: nb x bh x fbw half spectra (__half2 pairs when half)
  int half;            // store the spectra as fp16 pairs
  int* err;            // kErrWaitForward set when a tensor-core wait gives up
};
bool tc_supported(int mode, int bw, int bh, int bm);
// DFT matrices (fp16 hi/lo, in the kernels' shared-memory operand layout)
// with the separable mode-1 windows folded in, and the analysis window's
// spectrum, for n x n blocks: analysis wx[x] * wy[y], synthesis sxa[x] *
// sy[y] (even block columns) and sxb[x] * sy[y] (odd).
std::vector<uint8_t> tc_tables(int n, const std::vector<double>& wx, const std::vector<double>& wy,
                               const std::vector<double>& sxa, const std::vector<double>& sxb,
                               const std::vector<double>& sy);
cudaError_t launch_forward_tc(const TcFwdArgs& a, cudaStream_t st);

// Batches: up to kMaxBatch planes with the same block geometry, windows,
// temporal mode and sample format in one launch of each kernel (the planes
// of a YUV frame, or planes of several streams). A CTA finds its plane from
// the prefix of per-plane CTA (forward: block-group) counts. Passed by value
// as kernel parameters, so a captured CUDA graph is re-pointed at the next
// frame's buffers by updating its kernel nodes' parameters. At 16 planes a
// SweepBatch is about 13.5 KB: above the classic 4 KB parameter limit, within
// the 32 KB that CUDA 12.1+ allows for __grid_constant__ parameters.
constexpr int kMaxBatch = 16;
struct TcFwdBatch {
  int n;
  int grp0[kMaxBatch + 1];
  TcFwdArgs p[kMaxBatch];
};
struct SweepBatch {
  int n;
  int cta0[kMaxBatch + 1];
  // Filter: runs of consecutive planes of one geometry. run[i] is the first
  // plane of plane i's run, rlen[r] the length of the run starting at r; the
  // run's CTAs interleave its planes (CTA j of the run: group j / rlen of
  // plane r + j % rlen).
  int run[kMaxBatch];
  int rlen[kMaxBatch];
  int shifted;  // filter: bit i set when plane i's window is plane i-1's (same run) moved on by one frame
  SweepArgs p[kMaxBatch];
};
// Launch shape of the tensor-core kernels, picked by the autotuner.
struct TcTune {
  int fwd_ctas_per_sm = 3;  // persistent forward grid: CTAs per SM (1 to 3; 2 at most with the split)
  int filter_minb = 5;      // filter kernel variant: 5, 4 or 3 CTAs per SM (spectra loads of 1, 2, 2 blocks in flight)
};
cudaError_t launch_forward_tc_batch(const TcFwdArgs* planes, int n, const TcTune& t, cudaStream_t st);
// mark and after_filter (either may be null) are recorded on st between the
// filter and the inverse kernels.
cudaError_t launch_sweep_tc_batch(const SweepArgs* planes, int n, const TcTune& t, cudaStream_t st,
                                  cudaEvent_t mark, cudaEvent_t after_filter = nullptr);
// Re-points the kernel nodes of a graph captured from launch_forward_tc_batch
// (nf planes, 0: none) + launch_sweep_tc_batch (ns planes) at new plane
// arguments of the same shapes.
cudaError_t tc_graph_update(cudaGraphExec_t exec, cudaGraph_t graph, const TcFwdArgs* fwd, int nf,
                            const SweepArgs* sw, int ns);
// Tensor-core sweep: cells per strip, CTAs per SM, and the launches (filter,
// inverse + overlap-add, seam merge of f3d_k_sweep.cu).
int tc_sweep_cells(int n);  // 7 for 32 x 32 blocks, 15 for 16 x 16
constexpr int kTcSweepCtasPerSm = 3;
cudaError_t launch_sweep_tc(const SweepArgs& a, cudaStream_t st, cudaEvent_t mark);
// The fast form's fused sweeps of n planes (8x8 to 32x32 blocks, one
// temporal mode) in one launch, then their seam rows in one more; `mark` is
// recorded between the two.
cudaError_t launch_sweep_fast_batch(const SweepArgs* planes, int n, cudaStream_t st, cudaEvent_t mark);
cudaError_t launch_seam_merge_batch(const SweepBatch& Bm, int n, int maxw, int ch, cudaStream_t st);
// Bytes of SweepArgs::img for this geometry and strip count.
size_t tc_image_bytes(const Geo& g, int strips);
cudaError_t launch_seam_merge(const SweepArgs& a, cudaStream_t st);

// Counts one kernel launch made by this library (all engines, all threads).
void count_launch();

} // namespace f3d
