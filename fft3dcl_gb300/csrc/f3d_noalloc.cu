// f3d_noalloc.cu -- f3d_denoise_noalloc: one frame through the exact-form
// kernels with every intermediate in a static device array, for callers that
// cannot call cudaMalloc (graph capture, fixed device-memory budgets,
// real-time threads that must not take cudaMalloc's device-wide sync).
//
// Scratch layout (one call): [tables][window spectra x nwin][windowed blocks],
// each region 256-byte aligned. Every byte the kernels read is written
// earlier in the same call (tables by the upload, spectra by the forward
// kernel, blocks by the inverse kernel), so nothing needs clearing between
// calls.
#include "f3d_host.hpp"
#include "f3d_kernels.hpp"

#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <mutex>

namespace f3d {
void set_last_error(const char* msg);
}

namespace {

using namespace f3d;

// Held by every GPU that loads this library, until the process exits.
static __device__ __align__(256) unsigned char g_noalloc_scratch[F3D_NOALLOC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
constexpr int kMaxDim = 64;               // block sizes of the GPU path
constexpr int kMaxBins = (kMaxDim / 2 + 1) * kMaxDim;
constexpr size_t kAlign = 256;

std::mutex g_mtx;                          // guards the set-up and the host table staging
unsigned char* g_scratch_ptr[kMaxDevices]; // device address of the array, per device

// Host staging of the tables, in the order they are laid out on the device.
struct HostTables {
  float win[3 * kMaxDim * kMaxDim];  // analysis, synthesis A, synthesis B
  float pattern[kMaxBins];
  float sharpen[kMaxBins];
  float gs[2 * kMaxBins];            // degrid sample, interleaved re, im
};
HostTables g_host;

size_t round_up(size_t v) { return (v + kAlign - 1) / kAlign * kAlign; }

int fail(int code, const char* msg) {
  set_last_error(msg);
  return code;
}

// The table formulas below are the engine's (f3d_host.hpp, which restates
// src/cpu/tables.cpp, src/cpu/fft.cpp:8-58 and src/cpu/reference.cpp:51-57,
// 172-198) with stack storage instead of vectors; the GPU test of this entry
// point checks that its output has the engine's bits.

void twiddles_into(int n, float2* tw) {
  for (int k = 0; k < n / 2; k++) {
    double a = -2.0 * 3.14159265358979323846 * k / n;
    tw[k] = make_float2((float)std::cos(a), (float)std::sin(a));
  }
}

void window_mode0_into(int bw, int bh, float* w) {
  int off = 0;
  for (double n1 = -bh / 2.0 + 0.5; n1 < bh / 2.0; n1++) {
    double cosy = std::cos(n1 * kPi / bh);
    for (double n2 = -bw / 2.0 + 0.5; n2 < bw / 2.0; n2++) {
      double cosx = std::cos(n2 * kPi / bw);
      w[off++] = (float)std::sqrt(0.5 * (cosx * cosx + cosy * cosy));
    }
  }
}

void ramps(int o, int wintype, double* wan, double* wsyn) {
  for (int i = 0; i < o; i++) {
    const double hc = std::cos(kPi * (i - o + 0.5) / (o * 2.0));
    if (wintype == 1) {
      wan[i] = std::sqrt(hc);
      wsyn[i] = wan[i] * wan[i] * wan[i];
    } else if (wintype == 2) {
      wan[i] = 1.0;
      wsyn[i] = hc;
      wsyn[i] *= wsyn[i];
    } else {
      wan[i] = hc;
      wsyn[i] = wan[i];
    }
  }
}

void windows_mode1_into(int bw, int bh, int ow, int oh, int wintype, float* A, float* synA, float* synB) {
  double wanx[kMaxDim], wsynx[kMaxDim], wany[kMaxDim], wsyny[kMaxDim];
  double wxA[kMaxDim], wxSA[kMaxDim], wxSB[kMaxDim], wyA[kMaxDim], wySA[kMaxDim];
  ramps(ow, wintype, wanx, wsynx);
  ramps(oh, wintype, wany, wsyny);
  for (int lx = 0; lx < bw; lx++) {
    if (lx < ow) {
      wxA[lx] = wanx[lx];
      wxSA[lx] = wsynx[lx];
      wxSB[lx] = wsynx[(ow - 1) - lx];
    } else if (lx < bw - ow) {
      wxA[lx] = wxSA[lx] = wxSB[lx] = 1.0;
    } else {
      const int x = lx - (bw - ow);
      wxA[lx] = wanx[(ow - 1) - x];
      wxSA[lx] = wsynx[(ow - 1) - x];
      wxSB[lx] = wsynx[x];
    }
  }
  for (int ly = 0; ly < bh; ly++) {
    if (ly < oh) {
      wyA[ly] = wany[ly];
      wySA[ly] = wsyny[ly];
    } else if (ly < bh - oh) {
      wyA[ly] = wySA[ly] = 1.0;
    } else {
      wyA[ly] = wany[bh - 1 - ly];
      wySA[ly] = wsyny[bh - 1 - ly];
    }
  }
  for (int ly = 0; ly < bh; ly++)
    for (int lx = 0; lx < bw; lx++) {
      A[ly * bw + lx] = (float)(wxA[lx] * wyA[ly]);
      synA[ly * bw + lx] = (float)(wxSA[lx] * wySA[ly]);
      const int sx = (lx + bw - ow) % bw;  // odd-parity window sampled (bw-ow) right
      synB[ly * bw + lx] = (float)(wxSB[sx] * wySA[ly]);
    }
}

void pattern_into(int bw, int bh, int bt, float sigma, float sigma2, float sigma3, float sigma4, float* pat) {
  const int fbw = bw / 2 + 1;
  auto scale = [&](float s) {
    double v = s / 255.0;
    return (float)(v * v * bt * bw * bh);
  };
  float s = scale(sigma), s2 = scale(sigma2), s3 = scale(sigma3), s4 = scale(sigma4);
  float ft2 = (float)(std::sqrt(0.5) / 2.0);
  float ft3 = (float)(std::sqrt(0.5) / 4.0);
  for (int h = 0; h < bh; h++) {
    float fy = (bh - 2.0f * std::fabs(h - bh / 2.0f)) / bh;
    for (int w = 0; w < fbw; w++) {
      float fx = w * 1.0f / fbw;
      float f = std::sqrt((fx * fx + fy * fy) * 0.5f);
      float p;
      if (f < ft3)
        p = s4 + (s3 - s4) * f / ft3;
      else if (f < ft2)
        p = s3 + (s2 - s3) * (f - ft3) / (ft2 - ft3);
      else
        p = s + (s2 - s) * (1.0f - f) / (1.0f - ft2);
      pat[h * fbw + w] = p;
    }
  }
}

void sharpen_into(int bw, int bh, float strength, float svr, float scutoff, float* lut) {
  const int fbw = bw / 2 + 1;
  for (int j = 0; j < bh; j++) {
    int dj = j >= bh / 2 ? bh - j : j;
    float d2v = (float)(dj * dj) * (svr * svr) / ((bh / 2.0f) * (bh / 2.0f));
    for (int i = 0; i < fbw; i++) {
      float d2 = d2v + (float)(i * i) / ((bw / 2.0f) * (bw / 2.0f));
      lut[j * fbw + i] = strength * (1.0f - std::exp(-d2 / (2.0f * scutoff * scutoff)));
    }
  }
}

// Radix-2 DIT of n interleaved complex values, forward (src/cpu/fft.cpp:28-58).
void fft_forward(int n, const float2* tw, const float* in, float* out) {
  float a[2 * kMaxDim];
  int bits = 0;
  while ((1 << bits) < n) bits++;
  for (int i = 0; i < n; i++) {
    int r = 0;
    for (int b = 0; b < bits; b++)
      if (i & (1 << b)) r |= 1 << (bits - 1 - b);
    a[2 * i] = in[2 * r];
    a[2 * i + 1] = in[2 * r + 1];
  }
  for (int len = 2; len <= n; len <<= 1) {
    const int half = len >> 1, step = n / len;
    for (int i = 0; i < n; i += len)
      for (int j = 0; j < half; j++) {
        const float wr = tw[j * step].x, wi = tw[j * step].y;
        const float br = a[2 * (i + j + half)], bi = a[2 * (i + j + half) + 1];
        const float tr = wr * br - wi * bi, ti = wr * bi + wi * br;
        const float ur = a[2 * (i + j)], ui = a[2 * (i + j) + 1];
        a[2 * (i + j)] = ur + tr;
        a[2 * (i + j) + 1] = ui + ti;
        a[2 * (i + j + half)] = ur - tr;
        a[2 * (i + j + half) + 1] = ui - ti;
      }
  }
  for (int i = 0; i < 2 * n; i++) out[i] = a[i];
}

// FFT of the analysis window / its DC x degrid; only the fbw kept columns
// are transformed (column transforms are independent).
void degrid_into(int bw, int bh, float degrid, const float* win, const float2* twr, const float2* twc,
                 float* gs) {
  const int fbw = bw / 2 + 1;
  float row[2 * kMaxDim], res[2 * kMaxDim], col[2 * kMaxDim];
  for (int r = 0; r < bh; r++) {
    for (int c = 0; c < bw; c++) {
      row[2 * c] = win[r * bw + c];
      row[2 * c + 1] = 0.0f;
    }
    fft_forward(bw, twr, row, res);
    for (int c = 0; c < fbw; c++) {
      gs[2 * (r * fbw + c)] = res[2 * c];
      gs[2 * (r * fbw + c) + 1] = res[2 * c + 1];
    }
  }
  for (int c = 0; c < fbw; c++) {
    for (int r = 0; r < bh; r++) {
      col[2 * r] = gs[2 * (r * fbw + c)];
      col[2 * r + 1] = gs[2 * (r * fbw + c) + 1];
    }
    fft_forward(bh, twc, col, res);
    for (int r = 0; r < bh; r++) {
      gs[2 * (r * fbw + c)] = res[2 * r];
      gs[2 * (r * fbw + c) + 1] = res[2 * r + 1];
    }
  }
  const float dc = gs[0];
  for (int i = 0; i < fbw * bh; i++) {
    gs[2 * i] = gs[2 * i] / dc * degrid;
    gs[2 * i + 1] = gs[2 * i + 1] / dc * degrid;
  }
}

// Device address of the scratch array on the current device, looked up once
// per device with that device current.
int scratch_on_current_device(unsigned char** out) {
  int dev = 0;
  cudaError_t ce = cudaGetDevice(&dev);
  if (ce != cudaSuccess) return fail(F3D_E_CUDA, "FFT3DCL: no current CUDA device for the no-alloc call");
  if (dev < 0 || dev >= kMaxDevices) return fail(F3D_E_UNSUPPORTED, "FFT3DCL: device ordinal above 63");
  if (!g_scratch_ptr[dev]) {
    void* p = nullptr;
    ce = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (ce != cudaSuccess || !p) {
      char msg[200];
      std::snprintf(msg, sizeof msg, "FFT3DCL: cudaGetSymbolAddress of the no-alloc scratch failed: %s",
                    cudaGetErrorString(ce));
      return fail(F3D_E_CUDA, msg);
    }
    g_scratch_ptr[dev] = static_cast<unsigned char*>(p);
  }
  *out = g_scratch_ptr[dev];
  return F3D_OK;
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
  if (!form_supported(F3D_FORM_EXACT, ip.bw, ip.bh))
    return fail(F3D_E_UNSUPPORTED, "FFT3DCL: block size not supported by the GPU path (powers of two 4..64)");
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

  std::lock_guard<std::mutex> lock(g_mtx);
  unsigned char* base = nullptr;
  int rc = scratch_on_current_device(&base);
  if (rc != F3D_OK) return rc;
  cudaStream_t st = static_cast<cudaStream_t>(stream);

  // Tables on the host (stack and static storage only), then one upload into
  // the head of the scratch array: [win_ana | syn_a | syn_b | pattern | sharpen | gs].
  Twiddles tw{};
  twiddles_into(ip.bw, tw.row);
  twiddles_into(ip.bh, tw.col);
  float* h_ana = g_host.win;
  float* h_sa = h_ana + bwbh;
  float* h_sb = h_sa + bwbh;
  float* h_pat = h_sb + bwbh;
  float* h_shp = h_pat + ps;
  float* h_gs = h_shp + ps;
  if (ip.mode == 0) {
    window_mode0_into(ip.bw, ip.bh, h_ana);
  } else {
    windows_mode1_into(ip.bw, ip.bh, ip.ow, ip.oh, ip.wintype, h_ana, h_sa, h_sb);
  }
  if (ip.use_pattern) pattern_into(ip.bw, ip.bh, ip.bt, ip.sigma * 255.0f, ip.sigma2, ip.sigma3, ip.sigma4, h_pat);
  if (ip.sharpen_on) sharpen_into(ip.bw, ip.bh, ip.sharpen, ip.svr, ip.scutoff, h_shp);
  if (ip.degrid_on) degrid_into(ip.bw, ip.bh, ip.degrid, h_ana, tw.row, tw.col, h_gs);
  // The staging lives in g_host, contiguous from h_ana; pageable copies return
  // once the bytes are staged, so the next call may rewrite g_host.
  cudaError_t ce = cudaMemcpyAsync(base, h_ana, tab_floats * sizeof(float), cudaMemcpyHostToDevice, st);
  if (ce != cudaSuccess) {
    cudaGetLastError();
    return fail(F3D_E_CUDA, "FFT3DCL: table upload into the no-alloc scratch failed");
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
