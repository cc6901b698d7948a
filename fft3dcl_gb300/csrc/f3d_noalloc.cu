// f3d_noalloc.cu -- f3d_denoise_noalloc: one frame through the exact-form
// kernels with every intermediate in a static device array, for callers that
// cannot call cudaMalloc (hosts that hand out a fixed device-memory budget up
// front, real-time threads that must not take cudaMalloc/cudaFree's
// device-wide synchronisation).
//
// Scratch layout (one call): [tables][window spectra x nwin][windowed blocks],
// each region 256-byte aligned. Every byte the kernels read is written
// earlier in the same call and on the same stream (tables by the table
// kernel, spectra by the forward kernel, blocks by the inverse kernel), so
// nothing needs clearing between calls.
//
// The tables are built on the host by the engine's own builders
// (f3d_host.hpp) into stack storage and reach the device as parameters of
// k_noalloc_tables: the launch copies them, so no host buffer has to outlive
// the call and calls share no host staging.
#include "f3d_host.hpp"
#include "f3d_kernels.hpp"

#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <mutex>

namespace f3d {
void set_last_error(const char* msg);
}

namespace {

using namespace f3d;

// Held by every GPU that loads this library, until the process exits.
static __device__ __align__(256) unsigned char g_noalloc_scratch[F3D_NOALLOC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
constexpr int kMaxDim = 64;               // block sizes of this entry point
constexpr int kMaxBins = (kMaxDim / 2 + 1) * kMaxDim;
constexpr size_t kAlign = 256;

// Host tables of one call, in their device order:
// [win_ana | syn_a | syn_b | pattern | sharpen | gs].
constexpr int kMaxTabFloats = 3 * kMaxDim * kMaxDim + 4 * kMaxBins;

// One piece of the tables as a kernel parameter, within CUDA's 32 KB of
// kernel parameters.
constexpr int kPieceFloats = 7680;
struct TablePiece {
  float* dst;
  int n;
  float v[kPieceFloats];
};
static_assert(sizeof(TablePiece) <= 31 * 1024, "kernel parameter space");

__global__ void k_noalloc_tables(const __grid_constant__ TablePiece p) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < p.n; i += gridDim.x * blockDim.x) p.dst[i] = p.v[i];
}

// Device address of the scratch array, looked up with cudaGetSymbolAddress
// once per device and CUDA context, with that device current. The context is
// part of the key: after cudaDeviceReset the runtime creates a new primary
// context, in which the array has a new address.
using CtxGetCurrent = int (*)(void**);  // cuCtxGetCurrent
struct ScratchAddr {
  void* ctx = nullptr;
  unsigned char* ptr = nullptr;
};
std::mutex g_mtx;  // guards g_addr and g_ctx_get_current
ScratchAddr g_addr[kMaxDevices];
CtxGetCurrent g_ctx_get_current = nullptr;

size_t round_up(size_t v) { return (v + kAlign - 1) / kAlign * kAlign; }

int fail(int code, const char* msg) {
  set_last_error(msg);
  return code;
}

void* current_context() {
  void* ctx = nullptr;
  if (g_ctx_get_current) g_ctx_get_current(&ctx);
  return ctx;
}

int scratch_on_current_device(unsigned char** out) {
  int dev = 0;
  cudaError_t ce = cudaGetDevice(&dev);
  if (ce != cudaSuccess) return fail(F3D_E_CUDA, "FFT3DCL: no current CUDA device for the no-alloc call");
  if (dev < 0 || dev >= kMaxDevices) return fail(F3D_E_UNSUPPORTED, "FFT3DCL: device ordinal above 63");
  std::lock_guard<std::mutex> lock(g_mtx);
  if (!g_ctx_get_current) {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q{};
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &fn, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      g_ctx_get_current = reinterpret_cast<CtxGetCurrent>(fn);
    cudaGetLastError();
  }
  ScratchAddr& a = g_addr[dev];
  void* ctx = current_context();
  // A thread that has not used the runtime yet has no current context: the
  // lookup below binds the device's context, and the key is taken after it.
  if (!a.ptr || !ctx || ctx != a.ctx) {
    void* p = nullptr;
    ce = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (ce != cudaSuccess || !p) {
      char msg[200];
      std::snprintf(msg, sizeof msg, "FFT3DCL: cudaGetSymbolAddress of the no-alloc scratch failed: %s",
                    cudaGetErrorString(ce));
      cudaGetLastError();
      return fail(F3D_E_CUDA, msg);
    }
    a.ptr = static_cast<unsigned char*>(p);
    a.ctx = current_context();
  }
  *out = a.ptr;
  return F3D_OK;
}

// Host tables of one call into t (kMaxTabFloats floats, the caller's stack).
void build_tables_into(const f3d_internal_params& ip, const float* tw_row, const float* tw_col, float* t) {
  const int bwbh = ip.bw * ip.bh, ps = (ip.bw / 2 + 1) * ip.bh;
  float* ana = t;
  float* sa = ana + bwbh;
  float* sb = sa + bwbh;
  float* pat = sb + bwbh;
  float* shp = pat + ps;
  float* gs = shp + ps;
  std::memset(t, 0, sizeof(float) * (3 * (size_t)bwbh + 4 * (size_t)ps));
  if (ip.mode == 0) {
    window_mode0_into(ip.bw, ip.bh, ana);
  } else {
    double ax[kMaxDim], ay[kMaxDim], sxa[kMaxDim], sxb[kMaxDim], sy[kMaxDim];
    mode1_axes_into(ip.bw, ip.bh, ip.ow, ip.oh, ip.wintype, ax, ay, sxa, sxb, sy);
    windows_mode1_into(ip.bw, ip.bh, ax, ay, sxa, sxb, sy, ana, sa, sb);
  }
  if (ip.use_pattern)
    sigma_pattern_into(ip.bw, ip.bh, ip.bt, ip.sigma * 255.0f, ip.sigma2, ip.sigma3, ip.sigma4, pat);
  if (ip.sharpen_on) sharpen_lut_into(ip.bw, ip.bh, ip.sharpen, ip.svr, ip.scutoff, shp);
  if (ip.degrid_on) degrid_sample_into(ip.bw, ip.bh, ip.degrid, ana, tw_row, tw_col, gs);
}

}  // namespace

extern "C" int f3d_denoise_noalloc(const f3d_script_params* sp, const f3d_plane_geom* geom,
                                   const void* const* dev_window, int nwin, size_t src_pitch, void* dev_dst,
                                   size_t dst_pitch, void* stream) {
  if (!sp || !geom || !dev_window || !dev_dst) return fail(F3D_E_PARAM, "FFT3DCL: null argument");
  const f3d_plane_geom& g = *geom;
  if (g.width <= 0 || g.height <= 0) return fail(F3D_E_PARAM, "FFT3DCL: plane size must be positive");
  if (g.sample_type == 1 ? g.bits != 32 : (g.bits < 8 || g.bits > 16))
    return fail(F3D_E_PARAM, "FFT3DCL: integer bit depths 8-16 and 32-bit float only");
  f3d_internal_params ip;
  std::string err;  // stays empty (no allocation) unless validation fails
  if (!validate_params(*sp, g.width, g.height, g.bits, ip, &err)) return fail(F3D_E_PARAM, err.c_str());
  if (ip.bm == 0)
    return fail(F3D_E_UNSUPPORTED, "FFT3DCL: the no-alloc call has no state across frames; Kalman (bt=0) "
                                   "needs an engine");
  if (ip.bw > kMaxDim || ip.bh > kMaxDim || !form_supported(F3D_FORM_EXACT, ip.bw, ip.bh))
    return fail(F3D_E_UNSUPPORTED, "FFT3DCL: the no-alloc call takes block sizes 4..64");
  const int need = ip.bm >= 2 ? ip.bt : 1;
  if (nwin != need) {
    char msg[120];
    std::snprintf(msg, sizeof msg, "FFT3DCL: the no-alloc call needs %d window frame(s), got %d", need, nwin);
    return fail(F3D_E_PARAM, msg);
  }
  const int bps = g.sample_type == 1 ? 4 : (g.bits <= 8 ? 1 : 2);
  if (src_pitch < (size_t)g.width * bps || dst_pitch < (size_t)g.width * bps)
    return fail(F3D_E_PARAM, "FFT3DCL: pitch too small");

  const Grid grid = make_grid(ip);
  const int fbw = ip.bw / 2 + 1, ps = fbw * ip.bh, bwbh = ip.bw * ip.bh;
  const size_t tab_floats = 3 * (size_t)bwbh + 4 * (size_t)ps;
  const size_t off_spec = round_up(tab_floats * sizeof(float));
  const size_t spec_bytes = round_up(sizeof(float2) * (size_t)grid.nb * ps);
  const size_t off_blocks = off_spec + spec_bytes * need;
  const size_t total = off_blocks + round_up(sizeof(float) * (size_t)grid.nb * bwbh);
  if (total > F3D_NOALLOC_SCRATCH_BYTES) {
    char msg[200];
    std::snprintf(msg, sizeof msg,
                  "FFT3DCL: a %dx%d plane with %dx%d blocks and %d window frame(s) needs %zu bytes of scratch; "
                  "the no-alloc limit is %zu bytes",
                  g.width, g.height, ip.bw, ip.bh, need, total, (size_t)F3D_NOALLOC_SCRATCH_BYTES);
    return fail(F3D_E_UNSUPPORTED, msg);
  }

  unsigned char* base = nullptr;
  int rc = scratch_on_current_device(&base);
  if (rc != F3D_OK) return rc;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  cudaError_t ce = cudaSuccess;

  // Tables on the host (stack storage only), then into the head of the
  // scratch array through the parameters of the table kernel.
  Twiddles tw{};
  twiddles_into(ip.bw, reinterpret_cast<float*>(tw.row));
  twiddles_into(ip.bh, reinterpret_cast<float*>(tw.col));
  float tabs[kMaxTabFloats];
  build_tables_into(ip, reinterpret_cast<const float*>(tw.row), reinterpret_cast<const float*>(tw.col), tabs);
  for (size_t off = 0; off < tab_floats; off += kPieceFloats) {
    TablePiece piece;
    piece.dst = reinterpret_cast<float*>(base) + off;
    piece.n = (int)(tab_floats - off < (size_t)kPieceFloats ? tab_floats - off : (size_t)kPieceFloats);
    std::memcpy(piece.v, tabs + off, sizeof(float) * piece.n);
    k_noalloc_tables<<<8, 256, 0, st>>>(piece);
    count_launch();
    ce = cudaGetLastError();
    if (ce != cudaSuccess) return fail(F3D_E_CUDA, "FFT3DCL: table launch of the no-alloc call failed");
  }
  float* d_ana = reinterpret_cast<float*>(base);
  float* d_sa = d_ana + bwbh;
  float* d_sb = d_sa + bwbh;
  float* d_pat = d_sb + bwbh;
  float* d_shp = d_pat + ps;
  float2* d_gs = reinterpret_cast<float2*>(d_shp + ps);

  Geo geo{};
  geo.W = g.width;
  geo.H = g.height;
  geo.bw = ip.bw;
  geo.bh = ip.bh;
  geo.fbw = fbw;
  geo.nb = grid.nb;
  geo.mode = grid.mode;
  geo.ncols = grid.ncols;
  geo.nrows = grid.nrows;
  geo.xoff = grid.xoff;
  geo.xstep = grid.xstep;
  geo.yoff = grid.yoff;
  geo.ystep = grid.ystep;
  const int fmt = g.sample_type == 1 ? FMT_F32 : (g.bits <= 8 ? FMT_U8 : FMT_U16);
  const float norm = fmt == FMT_U16 ? (float)(1u << (16 - g.bits)) / 65535.0f : 1.0f;
  const float inv_norm = fmt == FMT_U16 ? 1.0f / (float)(1u << (16 - g.bits)) : 1.0f;
  const float max_pix = fmt == FMT_U16 ? (float)((1u << g.bits) - 1) : 0.0f;
  const float cnorm = chroma_norm(ip, g);

  float2* spec[4] = {nullptr, nullptr, nullptr, nullptr};
  for (int i = 0; i < need; i++) {
    spec[i] = reinterpret_cast<float2*>(base + off_spec + spec_bytes * i);
    FwdArgs a{};
    a.g = geo;
    a.tw = tw;
    a.src = static_cast<const uint8_t*>(dev_window[i]);
    a.pitch = (long long)src_pitch;
    a.fmt = fmt;
    a.norm = norm;
    a.chroma_norm = cnorm;
    a.win = d_ana;
    a.spec = spec[i];
    ce = launch_forward(F3D_FORM_EXACT, a, st);
    if (ce != cudaSuccess) return fail(F3D_E_CUDA, "FFT3DCL: forward launch of the no-alloc call failed");
  }
  float* d_blocks = reinterpret_cast<float*>(base + off_blocks);
  InvArgs v{};
  v.g = geo;
  v.tw = tw;
  for (int i = 0; i < 4; i++) v.s[i] = spec[i < need ? i : 0];
  v.cur = ip.bm >= 2 ? ip.current : 0;
  v.bm = ip.bm;
  v.dg = ip.degrid_on;
  v.pat = ip.use_pattern;
  v.shp = ip.sharpen_on;
  v.kalman_init = 0;
  v.gs = d_gs;
  v.pattern = d_pat;
  v.sharpen = d_shp;
  v.win_a = grid.mode == 1 ? d_sa : d_ana;
  v.win_b = grid.mode == 1 ? d_sb : d_ana;
  v.blocks = d_blocks;
  v.sigma_x = ip.beta * ip.wiener_s;
  v.sigma_y = ip.wiener_s;
  v.beta_x = ip.beta_x;
  v.beta = ip.beta;
  v.ssmin = ip.ssmin;
  v.ssmax = ip.ssmax;
  v.kalman_cn = ip.kalman_cn;
  v.kr2 = ip.kratio * ip.kratio;
  ce = launch_filter_inverse(F3D_FORM_EXACT, v, st);
  if (ce != cudaSuccess) return fail(F3D_E_CUDA, "FFT3DCL: filter/inverse launch of the no-alloc call failed");
  OlaArgs o{};
  o.g = geo;
  o.blocks = d_blocks;
  o.dst = static_cast<uint8_t*>(dev_dst);
  o.pitch = (long long)dst_pitch;
  o.fmt = fmt;
  o.chroma_norm = cnorm;
  o.inv_norm = inv_norm;
  o.max_pix = max_pix;
  ce = launch_ola(o, st);
  if (ce != cudaSuccess) return fail(F3D_E_CUDA, "FFT3DCL: overlap-add launch of the no-alloc call failed");
  return F3D_OK;
}
