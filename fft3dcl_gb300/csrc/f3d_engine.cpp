// f3d_engine.cpp -- the per-plane engine behind the C ABI (include/fft3d_gb300.h).
//
// Replaces the reference's OpenCL backend host class GpuRef
// (src/cl/gpu.{h,cpp}). An engine owns, on one CUDA device and one stream:
//   - the tables (windows, sigma pattern, sharpen LUT, degrid sample), built on
//     the host exactly like the reference's CPU tables and uploaded once;
//   - the spectra cache: one nb x bh x fbw complex buffer per cached frame,
//     with the reference's reuse pool and 256 MiB retire budget;
//   - the per-frame work buffers (raw plane in, windowed blocks, plane out);
//   - the Kalman state for bt=0, resident across frames.
// All device memory is counted in the process-wide live-bytes total.
#include "f3d_host.hpp"
#include "f3d_batch_plan.hpp"
#include "f3d_kernels.hpp"

#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

namespace f3d {
unsigned long long launch_count();
}

using namespace f3d;

namespace {

thread_local std::string t_last_error;
std::atomic<int> g_live{0};
std::atomic<size_t> g_bytes{0};

int fail_thread(int code, const std::string& msg) {
  t_last_error = msg;
  return code;
}

}  // namespace

namespace f3d {
// Records the message f3d_last_error returns (for entry points in other files).
void set_last_error(const char* msg) { t_last_error = msg; }
}  // namespace f3d

struct f3d_engine {
  std::mutex mtx;
  std::string err;
  f3d_internal_params ip{};
  f3d_plane_geom geom{};
  Grid grid;
  int device = 0, form = F3D_FORM_EXACT;
  // Form of the filter/inverse side: the tensor-core form's forward feeds
  // the fast-form sweep where no tensor-core inverse covers the geometry.
  int inv_form = F3D_FORM_EXACT;
  uint8_t* d_tc = nullptr;   // tensor-core form tables
  size_t tc_bytes = 0;
  int* d_err = nullptr;      // set by a tensor-core kernel whose wait gave up
  TcTune tune;               // tensor-core launch shape
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  int fbw = 0, ps = 0, bps = 1, fmt = FMT_U8;
  float norm = 1.0f, inv_norm = 1.0f, max_pix = 0.0f, cnorm = 0.0f;
  size_t spec_bytes = 0;

  std::vector<float> win_ana, syn_a, syn_b, pattern, sharpen, gs, tw_row, tw_col;
  Mode1Axes axes;  // mode-1 window factors
  float *d_win_ana = nullptr, *d_syn_a = nullptr, *d_syn_b = nullptr;
  float *d_pattern = nullptr, *d_sharpen = nullptr;
  float2* d_gs = nullptr;
  bool degrid_active = false;

  std::map<int, float2*> cache;
  std::vector<float2*> pool;
  int pool_min = 2;  // spectra the retire pool keeps whatever the budget: a batch raises it to its outputs per step
  bool half = false; // spectra stored as fp16 pairs (F3D_FLAG_HALF_SPECTRA applied)
  bool test_skip = false; // F3D_FLAG_TEST_WAIT_TIMEOUT, not applied yet

  uint8_t* d_in = nullptr;   // raw or float plane, width*height*4 bytes
  uint8_t* d_out = nullptr;  // packed or float output plane
  float* d_blocks = nullptr; // nb x bh x bw windowed blocks
  float2* d_twr = nullptr;   // blocks above 64: device twiddles (bw/2, bh/2 entries)
  float2* d_twc = nullptr;
  float2* d_work = nullptr;  // blocks above 64: nb x bh x bw complex inverse work space
  float2* d_klast = nullptr;
  float* d_kcov = nullptr;
  float* d_kproc = nullptr;
  bool kalman_first = true;

  // Fused sweep (mode 1, half overlap): CTA grid and seam scratch.
  bool fused = false;
  int sweep_strips = 0, sweep_segs = 0, sweep_prefetch = 0;
  float* d_seam = nullptr;
  size_t seam_floats = 0;
  uint8_t* d_img = nullptr;  // tensor-core sweep: filtered operand tiles
  size_t img_bytes = 0;

  size_t bytes = 0;
  // Kernel timing on the engine stream: forward [0,1], filter+inverse [2,4],
  // overlap-add [4,3].
  cudaEvent_t ev[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
  bool fwd_timed = false, proc_timed = false;

  int fail(int code, const std::string& msg) {
    err = msg;
    return code;
  }
  int cuda_fail(cudaError_t e, const char* where) {
    return fail(e == cudaErrorMemoryAllocation ? F3D_E_NOMEM : F3D_E_CUDA,
                std::string("FFT3DCL: CUDA error at ") + where + ": " + cudaGetErrorString(e));
  }
  template <class T>
  cudaError_t alloc(T** p, size_t n_bytes) {
    cudaError_t e = cudaMalloc(reinterpret_cast<void**>(p), n_bytes);
    if (e == cudaSuccess) {
      bytes += n_bytes;
      g_bytes += n_bytes;
    } else {
      *p = nullptr;
      cudaGetLastError();
    }
    return e;
  }
  template <class T>
  void release(T*& p, size_t n_bytes) {
    if (p) {
      cudaFree(p);
      bytes -= n_bytes;
      g_bytes -= n_bytes;
      p = nullptr;
    }
  }
};

namespace {

Geo make_geo(const f3d_engine* e) {
  Geo g{};
  g.W = e->geom.width;
  g.H = e->geom.height;
  g.bw = e->ip.bw;
  g.bh = e->ip.bh;
  g.fbw = e->fbw;
  g.nb = e->grid.nb;
  g.mode = e->grid.mode;
  g.ncols = e->grid.ncols;
  g.nrows = e->grid.nrows;
  g.xoff = e->grid.xoff;
  g.xstep = e->grid.xstep;
  g.yoff = e->grid.yoff;
  g.ystep = e->grid.ystep;
  return g;
}

Twiddles make_twiddles(const f3d_engine* e) {
  Twiddles t{};
  if (e->ip.bw <= 64)
    for (int k = 0; k < e->ip.bw / 2; k++) t.row[k] = make_float2(e->tw_row[2 * k], e->tw_row[2 * k + 1]);
  if (e->ip.bh <= 64)
    for (int k = 0; k < e->ip.bh / 2; k++) t.col[k] = make_float2(e->tw_col[2 * k], e->tw_col[2 * k + 1]);
  return t;
}

// GpuRef::spectra (src/cl/gpu.cpp:272-287): cached buffer of frame fn, or a
// recycled / new one.
float2* spectra_slot(f3d_engine* e, int fn, bool create) {
  auto it = e->cache.find(fn);
  if (it != e->cache.end()) return it->second;
  if (!create) return nullptr;
  float2* m = nullptr;
  if (!e->pool.empty()) {
    m = e->pool.back();
    e->pool.pop_back();
  } else if (e->alloc(&m, e->spec_bytes) != cudaSuccess) {
    return nullptr;
  }
  e->cache[fn] = m;
  return m;
}

// GpuRef::retireSpectra (src/cl/gpu.cpp:289-306): keep recycled buffers up
// to 256 MiB, release the rest; at least pool_min are kept (two, or the
// outputs per step of a batch the engine is in), so that steps that enter
// several frames do not allocate every time.
void retire(f3d_engine* e, float2* m) {
  const size_t budget = std::max(size_t(256) << 20, (size_t)e->pool_min * e->spec_bytes);
  if (e->pool.size() * e->spec_bytes + e->spec_bytes <= budget)
    e->pool.push_back(m);
  else
    e->release(m, e->spec_bytes);
}

// Tensor-core forward arguments for frame fn whose spectra go to `spec`.
TcFwdArgs tc_forward_args(const f3d_engine* e, const uint8_t* dsrc, long long pitch, int fmt, float2* spec) {
  TcFwdArgs t{};
  t.g = make_geo(e);
  t.src = dsrc;
  t.pitch = pitch;
  t.fmt = fmt;
  t.split = !(fmt == FMT_U8 || (fmt == FMT_U16 && e->geom.bits <= 11));
  t.norm = e->norm;
  t.out_scale = t.split ? 1.0f : (fmt == FMT_U8 ? 1.0f / 255.0f : e->norm);
  t.chroma_norm = e->cnorm;
  t.tab = e->d_tc;
  t.spec = spec;
  t.half = e->half ? 1 : 0;
  t.err = e->d_err;
  return t;
}

// Forward arguments of the exact and fast forms for a frame whose spectra go
// to `spec`.
FwdArgs forward_args(const f3d_engine* e, const uint8_t* dsrc, long long pitch, int fmt, float2* spec) {
  FwdArgs a{};
  a.g = make_geo(e);
  a.tw = make_twiddles(e);
  a.src = dsrc;
  a.pitch = pitch;
  a.fmt = fmt;
  a.norm = e->norm;
  a.chroma_norm = e->cnorm;
  a.win = e->d_win_ana;
  a.spec = spec;
  a.twr = e->d_twr;
  a.twc = e->d_twc;
  return a;
}

int run_forward(f3d_engine* e, int fn, const uint8_t* dsrc, long long pitch, int fmt) {
  float2* spec = spectra_slot(e, fn, true);
  if (!spec) return e->fail(F3D_E_NOMEM, "FFT3DCL: GPU spectra alloc failed");
  const FwdArgs a = forward_args(e, dsrc, pitch, fmt, spec);
  cudaEventRecord(e->ev[0], e->stream);
  cudaError_t ce;
  if (e->form == F3D_FORM_TC) {
    const TcFwdArgs t = tc_forward_args(e, dsrc, pitch, fmt, spec);
    ce = launch_forward_tc_batch(&t, 1, e->tune, e->stream);
  } else {
    ce = launch_forward(e->form, a, e->stream);
  }
  cudaEventRecord(e->ev[1], e->stream);
  e->fwd_timed = true;
  if (ce != cudaSuccess) {
    e->cache.erase(fn);
    retire(e, spec);
    return e->cuda_fail(ce, "the forward transform launch");
  }
  return F3D_OK;
}

// Filter/inverse arguments of a window; fails on missing spectra.
int inverse_args(f3d_engine* e, const int* window, int n, InvArgs& a) {
  const int need = e->ip.bm >= 2 ? e->ip.bt : 1;
  if (!window || n < need)
    return e->fail(F3D_E_PARAM, "FFT3DCL: the window must hold " + std::to_string(need) + " frame(s)");
  a = InvArgs{};
  for (int i = 0; i < 4; i++) {
    const int fn = window[i < need ? i : 0];
    const float2* s = spectra_slot(e, fn, false);
    if (!s) return e->fail(F3D_E_STATE, "FFT3DCL: missing spectra in window (frame " + std::to_string(fn) + ")");
    a.s[i] = s;
  }
  if (e->ip.degrid_on && !e->degrid_active) e->degrid_active = true;
  a.g = make_geo(e);
  a.tw = make_twiddles(e);
  a.half = e->half ? 1 : 0;
  a.cur = e->ip.bm >= 2 ? e->ip.current : 0;
  a.bm = e->ip.bm;
  a.dg = e->ip.degrid_on && e->degrid_active;
  a.pat = e->ip.use_pattern;
  a.shp = e->ip.sharpen_on;
  a.kalman_init = e->ip.bm == 0 && e->kalman_first;
  a.gs = e->d_gs;
  a.pattern = e->d_pattern;
  a.sharpen = e->d_sharpen;
  a.klast = e->d_klast;
  a.kcov = e->d_kcov;
  a.kproc = e->d_kproc;
  a.win_a = e->grid.mode == 1 ? e->d_syn_a : e->d_win_ana;
  a.win_b = e->grid.mode == 1 ? e->d_syn_b : e->d_win_ana;
  a.blocks = e->d_blocks;
  a.sigma_x = e->ip.beta * e->ip.wiener_s;
  a.sigma_y = e->ip.wiener_s;
  a.beta_x = e->ip.beta_x;
  a.beta = e->ip.beta;
  a.ssmin = e->ip.ssmin;
  a.ssmax = e->ip.ssmax;
  a.kalman_cn = e->ip.kalman_cn;
  a.kr2 = e->ip.kratio * e->ip.kratio;
  a.twr = e->d_twr;
  a.twc = e->d_twc;
  a.work = e->d_work;
  return F3D_OK;
}

// Sweep arguments (fused path) of a window's filter/inverse arguments.
SweepArgs sweep_args(const f3d_engine* e, const InvArgs& a, uint8_t* ddst, long long pitch, int fmt) {
  SweepArgs sa{};
  sa.inv = a;
  sa.dst = ddst;
  sa.pitch = pitch;
  sa.fmt = fmt;
  sa.chroma_norm = e->cnorm;
  sa.inv_norm = e->inv_norm;
  sa.max_pix = e->max_pix;
  sa.cells_x = (a.g.W + a.g.bw / 2 - 1) / (a.g.bw / 2);
  sa.cells_y = (a.g.H + a.g.bh / 2 - 1) / (a.g.bh / 2);
  sa.strips = e->sweep_strips;
  sa.segs = e->sweep_segs;
  sa.seam_w = sa.cells_x * (a.g.bw / 2);
  sa.seam_b = e->d_seam;
  sa.seam_t = e->d_seam ? e->d_seam + (size_t)(sa.segs - 1) * (a.g.bh / 2) * sa.seam_w : nullptr;
  sa.prefetch = e->sweep_prefetch;
  sa.tab = e->d_tc;
  sa.err = e->d_err;
  sa.img = e->d_img;
  sa.test_skip = e->test_skip ? 1 : 0;
  return sa;
}

int run_process(f3d_engine* e, const int* window, int n, uint8_t* ddst, long long pitch, int fmt) {
  InvArgs a;
  int rc = inverse_args(e, window, n, a);
  if (rc != F3D_OK) return rc;
  if (e->fused) {
    // One fused launch (plus the seam merge) writes the packed plane.
    const SweepArgs sa = sweep_args(e, a, ddst, pitch, fmt);
    e->test_skip = false;
    cudaEventRecord(e->ev[2], e->stream);
    cudaError_t ce = e->inv_form == F3D_FORM_TC ? launch_sweep_tc_batch(&sa, 1, e->tune, e->stream, e->ev[4])
                                                : launch_sweep(e->inv_form, sa, e->stream, e->ev[4]);
    cudaEventRecord(e->ev[3], e->stream);
    e->proc_timed = true;
    if (ce != cudaSuccess) return e->cuda_fail(ce, "the fused filter/inverse/overlap-add launch");
    return F3D_OK;
  }
  cudaEventRecord(e->ev[2], e->stream);
  cudaError_t ce = launch_filter_inverse(e->inv_form, a, e->stream);
  cudaEventRecord(e->ev[4], e->stream);
  if (ce != cudaSuccess) return e->cuda_fail(ce, "the filter/inverse launch");
  if (a.kalman_init) e->kalman_first = false;
  OlaArgs o{};
  o.g = a.g;
  o.blocks = e->d_blocks;
  o.dst = ddst;
  o.pitch = pitch;
  o.fmt = fmt;
  o.chroma_norm = e->cnorm;
  o.inv_norm = e->inv_norm;
  o.max_pix = e->max_pix;
  ce = launch_ola(o, e->stream);
  cudaEventRecord(e->ev[3], e->stream);
  e->proc_timed = true;
  if (ce != cudaSuccess) return e->cuda_fail(ce, "the overlap-add launch");
  return F3D_OK;
}

struct Lock {
  std::lock_guard<std::mutex> g;
  explicit Lock(f3d_engine* e) : g(e->mtx) { cudaSetDevice(e->device); }
};

}  // namespace

extern "C" {

void f3d_default_params(f3d_script_params* sp) {
  // ScriptParams defaults, src/params.h:8-27, with the plugin's dependent
  // defaults applied to them (src/fft3dcl.cpp:182-194).
  sp->sigma = 2.0f;
  sp->beta = 1.0f;
  sp->bw = sp->bh = 32;
  sp->bt = 3;
  sp->sharpen = 0.0f;
  sp->plane = 0;
  sp->mode = 1;
  sp->bordersize = 1;
  sp->precision = 0;
  sp->degrid = 1.0f;
  sp->scutoff = 0.3f;
  sp->svr = 1.0f;
  sp->smin = 4.0f;
  sp->smax = 20.0f;
  sp->kratio = 2.0f;
  sp->ow = sp->oh = 16;
  sp->wintype = 0;
  sp->interlaced = 0;
  sp->sigma2 = sp->sigma3 = sp->sigma4 = 2.0f;
  sp->oldfft = -1;
}

int f3d_validate_params(const f3d_script_params* sp, int width, int height, int bits,
                        f3d_internal_params* out) {
  if (!sp || !out) return fail_thread(F3D_E_PARAM, "FFT3DCL: null argument");
  std::string err;
  if (!validate_params(*sp, width, height, bits, *out, &err)) return fail_thread(F3D_E_PARAM, err);
  return F3D_OK;
}

const char* f3d_last_error(void) { return t_last_error.c_str(); }

int f3d_engine_create(const f3d_script_params* sp, const f3d_plane_geom* geom,
                      const f3d_options* opts, f3d_engine** out) {
  if (!sp || !geom || !out) return fail_thread(F3D_E_PARAM, "FFT3DCL: null argument");
  *out = nullptr;
  const f3d_plane_geom& g = *geom;
  if (g.width <= 0 || g.height <= 0)
    return fail_thread(F3D_E_PARAM, "FFT3DCL: plane size must be positive");
  if (g.sample_type == 1 ? g.bits != 32 : (g.bits < 8 || g.bits > 16))
    return fail_thread(F3D_E_PARAM, "FFT3DCL: integer bit depths 8-16 and 32-bit float only");
  f3d_internal_params ip;
  std::string err;
  if (!validate_params(*sp, g.width, g.height, g.bits, ip, &err)) return fail_thread(F3D_E_PARAM, err);
  int form = opts ? opts->form : F3D_FORM_EXACT;
  const int device = opts ? opts->device : 0;
  if (form < F3D_FORM_EXACT || form > F3D_FORM_TC) return fail_thread(F3D_E_PARAM, "FFT3DCL: unknown form");
  // Kalman's reset is a threshold on per-bin frame differences: any rounding
  // difference flips bins near it, so bt=0 runs the exact kernels in every
  // form. Blocks the faster forms do not cover (4-wide) use them too.
  if (ip.bm == 0) form = F3D_FORM_EXACT;
  if (form == F3D_FORM_TC && !tc_supported(ip.mode, ip.bw, ip.bh, ip.bm)) form = F3D_FORM_FAST;
  if (!form_supported(form, ip.bw, ip.bh)) form = F3D_FORM_EXACT;
  if (!form_supported(form, ip.bw, ip.bh))
    return fail_thread(F3D_E_UNSUPPORTED,
                       "FFT3DCL: block size " + std::to_string(ip.bw) + "x" + std::to_string(ip.bh) +
                           " is not supported by this GPU form (powers of two 4..512)");
  int ndev = 0;
  cudaError_t ce = cudaGetDeviceCount(&ndev);
  if (ce != cudaSuccess || ndev <= 0) {
    cudaGetLastError();
    return fail_thread(F3D_E_CUDA, std::string("FFT3DCL: no CUDA device available: ") +
                                       (ce != cudaSuccess ? cudaGetErrorString(ce) : "none found"));
  }
  if (device < 0 || device >= ndev) return fail_thread(F3D_E_PARAM, "FFT3DCL: device ordinal out of range");
  ce = cudaSetDevice(device);
  if (ce != cudaSuccess) return fail_thread(F3D_E_CUDA, std::string("FFT3DCL: cudaSetDevice: ") + cudaGetErrorString(ce));

  auto* e = new f3d_engine();
  ++g_live;
  e->ip = ip;
  e->geom = g;
  e->grid = make_grid(ip);
  e->device = device;
  e->form = form;
  // The tensor-core sweep covers half-overlap mode 1 with 32x32 blocks; other
  // tensor-core geometries pair its forward with the fast-form inverse.
  e->inv_form = form;
  if (form == F3D_FORM_TC && !(ip.ow * 2 == ip.bw && ip.oh * 2 == ip.bh)) e->inv_form = F3D_FORM_FAST;
  if (form == F3D_FORM_TC && opts && (opts->flags & F3D_FLAG_UNFUSED)) e->inv_form = F3D_FORM_FAST;
  e->fbw = ip.bw / 2 + 1;
  e->ps = e->fbw * ip.bh;
  e->spec_bytes = sizeof(float2) * (size_t)e->grid.nb * e->ps;
  if (g.sample_type == 1) {
    e->fmt = FMT_F32;
    e->bps = 4;
  } else if (g.bits <= 8) {
    e->fmt = FMT_U8;
    e->bps = 1;
  } else {
    e->fmt = FMT_U16;
    e->bps = 2;
    // Conversion constants of src/cpu/reference.cpp:97-98 and :126-127.
    e->norm = (float)(1u << (16 - g.bits)) / 65535.0f;
    e->inv_norm = 1.0f / (float)(1u << (16 - g.bits));
    e->max_pix = (float)((1u << g.bits) - 1);
  }
  e->cnorm = chroma_norm(ip, g);
  {
    PlaneTables t = build_tables(ip);
    e->tw_row = std::move(t.tw_row);
    e->tw_col = std::move(t.tw_col);
    e->win_ana = std::move(t.win_ana);
    e->syn_a = std::move(t.syn_a);
    e->syn_b = std::move(t.syn_b);
    e->pattern = std::move(t.pattern);
    e->sharpen = std::move(t.sharpen);
    e->gs = std::move(t.gs);
    if (ip.mode == 1) {
      std::vector<float> a, sa, sb;
      windows_mode1(ip.bw, ip.bh, ip.ow, ip.oh, ip.wintype, a, sa, sb, &e->axes);
    }
  }

  auto finish_fail = [&](int code) {
    std::string m = e->err;
    f3d_engine_destroy(e);
    return fail_thread(code, m);
  };
  if (opts && opts->stream) {
    e->stream = static_cast<cudaStream_t>(opts->stream);
  } else {
    ce = cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking);
    if (ce != cudaSuccess) return finish_fail(e->cuda_fail(ce, "stream creation"));
    e->own_stream = true;
  }
  for (auto& ev : e->ev) {
    ce = cudaEventCreate(&ev);
    if (ce != cudaSuccess) return finish_fail(e->cuda_fail(ce, "event creation"));
  }
  const size_t bwbh = (size_t)ip.bw * ip.bh;
  const size_t plane_bytes = (size_t)g.width * g.height * 4;
  auto up = [&](float** d, const std::vector<float>& h) -> cudaError_t {
    if (h.empty()) return cudaSuccess;
    cudaError_t x = e->alloc(d, h.size() * sizeof(float));
    if (x != cudaSuccess) return x;
    return cudaMemcpy(*d, h.data(), h.size() * sizeof(float), cudaMemcpyHostToDevice);
  };
  if ((ce = up(&e->d_win_ana, e->win_ana)) != cudaSuccess ||
      (ce = up(&e->d_syn_a, e->syn_a)) != cudaSuccess ||
      (ce = up(&e->d_syn_b, e->syn_b)) != cudaSuccess ||
      (ce = up(&e->d_pattern, e->pattern)) != cudaSuccess ||
      (ce = up(&e->d_sharpen, e->sharpen)) != cudaSuccess ||
      (ce = up(reinterpret_cast<float**>(&e->d_gs), e->gs)) != cudaSuccess)
    return finish_fail(e->cuda_fail(ce, "table upload"));
  if (form == F3D_FORM_TC) {
    const std::vector<uint8_t> tab = tc_tables(ip.bw, e->axes.ax, e->axes.ay, e->axes.sxa, e->axes.sxb, e->axes.sy);
    if (tab.empty()) return finish_fail(e->fail(F3D_E_UNSUPPORTED, "FFT3DCL: no tensor-core tables for this block size"));
    e->tc_bytes = tab.size();
    if ((ce = e->alloc(&e->d_tc, e->tc_bytes)) != cudaSuccess ||
        (ce = cudaMemcpy(e->d_tc, tab.data(), tab.size(), cudaMemcpyHostToDevice)) != cudaSuccess ||
        (ce = e->alloc(&e->d_err, sizeof(int))) != cudaSuccess || (ce = cudaMemset(e->d_err, 0, sizeof(int))) != cudaSuccess)
      return finish_fail(e->cuda_fail(ce, "tensor-core table upload"));
  }
  if ((ce = e->alloc(&e->d_in, plane_bytes)) != cudaSuccess ||
      (ce = e->alloc(&e->d_out, plane_bytes)) != cudaSuccess)
    return finish_fail(e->cuda_fail(ce, "buffer allocation"));
  if (ip.bm == 0) {
    const size_t nbin = (size_t)e->grid.nb * e->ps;
    if ((ce = e->alloc(&e->d_klast, sizeof(float2) * nbin)) != cudaSuccess ||
        (ce = e->alloc(&e->d_kcov, sizeof(float) * nbin)) != cudaSuccess ||
        (ce = e->alloc(&e->d_kproc, sizeof(float) * nbin)) != cudaSuccess)
      return finish_fail(e->cuda_fail(ce, "Kalman state allocation"));
  }
  const Geo geo = make_geo(e);
  if (!(opts && (opts->flags & F3D_FLAG_UNFUSED)) && sweep_supported(e->inv_form, geo, ip.bm)) {
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    sweep_plan(e->inv_form, geo, sms > 0 ? sms : 1, &e->sweep_strips, &e->sweep_segs);
    e->seam_floats = sweep_seam_floats(geo, e->sweep_segs);
    if (e->seam_floats && (ce = e->alloc(&e->d_seam, sizeof(float) * e->seam_floats)) != cudaSuccess)
      return finish_fail(e->cuda_fail(ce, "seam buffer allocation"));
    if (e->inv_form == F3D_FORM_TC) {
      e->img_bytes = tc_image_bytes(geo, e->sweep_strips);
      if ((ce = e->alloc(&e->d_img, e->img_bytes)) != cudaSuccess)
        return finish_fail(e->cuda_fail(ce, "tensor-core operand buffer allocation"));
    }
    e->fused = true;
    const int fl = opts ? opts->flags : 0;
    e->sweep_prefetch = (fl & F3D_FLAG_PREFETCH_EARLY) ? 1 : (fl & F3D_FLAG_PREFETCH_LATE) ? 2 : 0;
    // Half storage where the original filter used it (8-bit, precision 0/1)
    // and the tensor-core kernels read and write it.
    e->half = (fl & F3D_FLAG_HALF_SPECTRA) && e->form == F3D_FORM_TC && e->inv_form == F3D_FORM_TC &&
              e->fmt == FMT_U8 && ip.precision < 2;
    e->test_skip = (fl & F3D_FLAG_TEST_WAIT_TIMEOUT) && e->inv_form == F3D_FORM_TC;
    if (e->half) e->spec_bytes = sizeof(__half2) * (size_t)e->grid.nb * e->ps;
  }
  // The windowed-block buffer of the separate inverse and overlap-add kernels.
  if (!e->fused && (ce = e->alloc(&e->d_blocks, sizeof(float) * bwbh * e->grid.nb)) != cudaSuccess)
    return finish_fail(e->cuda_fail(ce, "buffer allocation"));
  // Blocks above 64: twiddles in device memory and the inverse's work space.
  if (big_block(ip.bw, ip.bh)) {
    if ((ce = up(reinterpret_cast<float**>(&e->d_twr), e->tw_row)) != cudaSuccess ||
        (ce = up(reinterpret_cast<float**>(&e->d_twc), e->tw_col)) != cudaSuccess ||
        (ce = e->alloc(&e->d_work, sizeof(float2) * bwbh * e->grid.nb)) != cudaSuccess)
      return finish_fail(e->cuda_fail(ce, "large-block buffer allocation"));
  }
  *out = e;
  return F3D_OK;
}

void f3d_engine_destroy(f3d_engine* e) {
  if (!e) return;
  {
    Lock l(e);
    if (e->stream) cudaStreamSynchronize(e->stream);
    for (auto& kv : e->cache) e->release(kv.second, e->spec_bytes);
    e->cache.clear();
    for (float2*& m : e->pool) e->release(m, e->spec_bytes);
    e->pool.clear();
    e->release(e->d_win_ana, e->win_ana.size() * sizeof(float));
    e->release(e->d_tc, e->tc_bytes);
    e->release(e->d_img, e->img_bytes);
    e->release(e->d_err, sizeof(int));
    e->release(e->d_syn_a, e->syn_a.size() * sizeof(float));
    e->release(e->d_syn_b, e->syn_b.size() * sizeof(float));
    e->release(e->d_pattern, e->pattern.size() * sizeof(float));
    e->release(e->d_sharpen, e->sharpen.size() * sizeof(float));
    e->release(e->d_gs, e->gs.size() * sizeof(float));
    const size_t plane_bytes = (size_t)e->geom.width * e->geom.height * 4;
    e->release(e->d_in, plane_bytes);
    e->release(e->d_out, plane_bytes);
    e->release(e->d_blocks, sizeof(float) * (size_t)e->ip.bw * e->ip.bh * e->grid.nb);
    e->release(e->d_twr, e->tw_row.size() * sizeof(float));
    e->release(e->d_twc, e->tw_col.size() * sizeof(float));
    e->release(e->d_work, sizeof(float2) * (size_t)e->ip.bw * e->ip.bh * e->grid.nb);
    const size_t nbin = (size_t)e->grid.nb * e->ps;
    e->release(e->d_klast, sizeof(float2) * nbin);
    e->release(e->d_kcov, sizeof(float) * nbin);
    e->release(e->d_kproc, sizeof(float) * nbin);
    e->release(e->d_seam, sizeof(float) * e->seam_floats);
    for (auto& ev : e->ev)
      if (ev) cudaEventDestroy(ev);
    if (e->own_stream && e->stream) cudaStreamDestroy(e->stream);
  }
  --g_live;
  delete e;
}

const char* f3d_engine_error(const f3d_engine* e) { return e ? e->err.c_str() : ""; }

int f3d_engine_get_info(f3d_engine* e, f3d_engine_info* info) {
  if (!e || !info) return fail_thread(F3D_E_PARAM, "FFT3DCL: null argument");
  Lock l(e);
  info->nblocks = e->grid.nb;
  info->fbw = e->fbw;
  info->ncols = e->grid.ncols;
  info->nrows = e->grid.nrows;
  info->bytes_per_sample = e->bps;
  info->raw_path = e->geom.sample_type != 1;
  info->spectrum_bytes = e->spec_bytes;
  info->device_bytes = e->bytes;
  info->cached_frames = (int)e->cache.size();
  info->chroma_norm = e->cnorm;
  info->form = e->form;
  info->fused = e->fused ? 1 : 0;
  info->half_spectra = e->half ? 1 : 0;
  return F3D_OK;
}

int f3d_engine_get_table(f3d_engine* e, int which, float* dst) {
  if (!e) return fail_thread(F3D_E_PARAM, "FFT3DCL: null engine");
  if (which < F3D_TAB_WIN_ANA || which > F3D_TAB_TWIDDLE_COL)
    return e->fail(F3D_E_PARAM, "FFT3DCL: unknown table");
  Lock l(e);
  PlaneTables t{e->win_ana, e->syn_a, e->syn_b, e->pattern, e->sharpen, e->gs, e->tw_row, e->tw_col};
  const std::vector<float> v = table_of(t, which);
  if (dst && !v.empty()) std::memcpy(dst, v.data(), v.size() * sizeof(float));
  return (int)v.size();
}

int f3d_compute_table(const f3d_script_params* sp, const f3d_plane_geom* geom, int which, float* dst) {
  if (!sp || !geom) return fail_thread(F3D_E_PARAM, "FFT3DCL: null argument");
  if (which < F3D_TAB_WIN_ANA || which > F3D_TAB_TWIDDLE_COL)
    return fail_thread(F3D_E_PARAM, "FFT3DCL: unknown table");
  f3d_internal_params ip;
  std::string err;
  if (!validate_params(*sp, geom->width, geom->height, geom->bits, ip, &err)) return fail_thread(F3D_E_PARAM, err);
  const std::vector<float> v = table_of(build_tables(ip), which);
  if (dst && !v.empty()) std::memcpy(dst, v.data(), v.size() * sizeof(float));
  return (int)v.size();
}

int f3d_forward(f3d_engine* e, int fn, const float* plane) {
  if (!e || !plane) return fail_thread(F3D_E_PARAM, "FFT3DCL: null argument");
  Lock l(e);
  const size_t n = (size_t)e->geom.width * e->geom.height * sizeof(float);
  cudaError_t ce = cudaMemcpyAsync(e->d_in, plane, n, cudaMemcpyHostToDevice, e->stream);
  if (ce != cudaSuccess) return e->cuda_fail(ce, "the plane upload");
  return run_forward(e, fn, e->d_in, (long long)e->geom.width * 4, FMT_F32);
}

int f3d_forward_raw(f3d_engine* e, int fn, const void* raw, size_t bytes) {
  if (!e || !raw) return fail_thread(F3D_E_PARAM, "FFT3DCL: null argument");
  Lock l(e);
  const size_t row = (size_t)e->geom.width * e->bps;
  if (bytes != row * e->geom.height) return e->fail(F3D_E_PARAM, "FFT3DCL: raw plane size mismatch");
  cudaError_t ce = cudaMemcpyAsync(e->d_in, raw, bytes, cudaMemcpyHostToDevice, e->stream);
  if (ce != cudaSuccess) return e->cuda_fail(ce, "the raw plane upload");
  return run_forward(e, fn, e->d_in, (long long)row, e->fmt);
}

int f3d_forward_device(f3d_engine* e, int fn, const void* dev_plane, size_t pitch) {
  if (!e || !dev_plane) return fail_thread(F3D_E_PARAM, "FFT3DCL: null argument");
  Lock l(e);
  if (pitch < (size_t)e->geom.width * e->bps) return e->fail(F3D_E_PARAM, "FFT3DCL: pitch too small");
  return run_forward(e, fn, static_cast<const uint8_t*>(dev_plane), (long long)pitch, e->fmt);
}

int f3d_get_spectra(f3d_engine* e, int fn, float* dst) {
  if (!e || !dst) return fail_thread(F3D_E_PARAM, "FFT3DCL: null argument");
  Lock l(e);
  const float2* s = spectra_slot(e, fn, false);
  if (!s) return e->fail(F3D_E_STATE, "FFT3DCL: frame " + std::to_string(fn) + " is not cached");
  if (e->half) {
    // fp16 pairs, widened to float on the host.
    std::vector<__half2> h(e->spec_bytes / sizeof(__half2));
    cudaError_t ce = cudaMemcpyAsync(h.data(), s, e->spec_bytes, cudaMemcpyDeviceToHost, e->stream);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(e->stream);
    if (ce != cudaSuccess) return e->cuda_fail(ce, "spectra readback");
    for (size_t i = 0; i < h.size(); i++) {
      dst[2 * i] = __low2float(h[i]);
      dst[2 * i + 1] = __high2float(h[i]);
    }
    return F3D_OK;
  }
  cudaError_t ce = cudaMemcpyAsync(dst, s, e->spec_bytes, cudaMemcpyDeviceToHost, e->stream);
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(e->stream);
  if (ce != cudaSuccess) return e->cuda_fail(ce, "spectra readback");
  return F3D_OK;
}

int f3d_has(f3d_engine* e, int fn) {
  if (!e) return 0;
  Lock l(e);
  return e->cache.count(fn) ? 1 : 0;
}

int f3d_raw_path(f3d_engine* e) { return e && e->geom.sample_type != 1 ? 1 : 0; }
int f3d_bytes_per_sample(f3d_engine* e) { return e ? e->bps : 0; }

int f3d_upload_degrid_sample(f3d_engine* e) {
  if (!e) return fail_thread(F3D_E_PARAM, "FFT3DCL: null engine");
  Lock l(e);
  if (e->ip.degrid_on) e->degrid_active = true;
  return F3D_OK;
}

int f3d_process(f3d_engine* e, const int* window, int n, float* out) {
  if (!e || !out) return fail_thread(F3D_E_PARAM, "FFT3DCL: null argument");
  Lock l(e);
  const size_t row = (size_t)e->geom.width * 4;
  int rc = run_process(e, window, n, e->d_out, (long long)row, FMT_F32);
  if (rc != F3D_OK) return rc;
  cudaError_t ce = cudaMemcpyAsync(out, e->d_out, row * e->geom.height, cudaMemcpyDeviceToHost, e->stream);
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(e->stream);
  if (ce != cudaSuccess) return e->cuda_fail(ce, "readback");
  return F3D_OK;
}

int f3d_process_raw(f3d_engine* e, const int* window, int n, void* dst, size_t bytes) {
  if (!e || !dst) return fail_thread(F3D_E_PARAM, "FFT3DCL: null argument");
  Lock l(e);
  const size_t row = (size_t)e->geom.width * e->bps;
  if (bytes != row * e->geom.height) return e->fail(F3D_E_PARAM, "FFT3DCL: raw plane size mismatch");
  int rc = run_process(e, window, n, e->d_out, (long long)row, e->fmt);
  if (rc != F3D_OK) return rc;
  cudaError_t ce = cudaMemcpyAsync(dst, e->d_out, bytes, cudaMemcpyDeviceToHost, e->stream);
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(e->stream);
  if (ce != cudaSuccess) return e->cuda_fail(ce, "readback");
  return F3D_OK;
}

int f3d_process_device(f3d_engine* e, const int* window, int n, void* dev_dst, size_t pitch) {
  if (!e || !dev_dst) return fail_thread(F3D_E_PARAM, "FFT3DCL: null argument");
  Lock l(e);
  if (pitch < (size_t)e->geom.width * e->bps) return e->fail(F3D_E_PARAM, "FFT3DCL: pitch too small");
  return run_process(e, window, n, static_cast<uint8_t*>(dev_dst), (long long)pitch, e->fmt);
}

int f3d_prune(f3d_engine* e, int lo, int hi) {
  if (!e) return fail_thread(F3D_E_PARAM, "FFT3DCL: null engine");
  Lock l(e);
  for (auto it = e->cache.begin(); it != e->cache.end();) {
    const bool keep = (lo < 0 || it->first >= lo) && (hi < 0 || it->first <= hi);
    if (keep) {
      ++it;
    } else {
      retire(e, it->second);
      it = e->cache.erase(it);
    }
  }
  return F3D_OK;
}

int f3d_synchronize(f3d_engine* e) {
  if (!e) return fail_thread(F3D_E_PARAM, "FFT3DCL: null engine");
  Lock l(e);
  cudaError_t ce = cudaStreamSynchronize(e->stream);
  if (ce != cudaSuccess) return e->cuda_fail(ce, "synchronize");
  if (e->d_err) {
    int flag = 0;
    ce = cudaMemcpy(&flag, e->d_err, sizeof(int), cudaMemcpyDeviceToHost);
    if (ce != cudaSuccess) return e->cuda_fail(ce, "synchronize");
    if (flag) {
      std::string which;
      if (flag & kErrWaitForward) which += ", forward transform (tensor-core steps)";
      if (flag & kErrWaitTile) which += ", inverse kernel (operand tile copy)";
      if (flag & kErrWaitColumn) which += ", inverse kernel (column-inverse products)";
      if (flag & kErrWaitRow) which += ", inverse kernel (row-inverse products)";
      cudaMemset(e->d_err, 0, sizeof(int));
      return e->fail(F3D_E_CUDA, "FFT3DCL: a tensor-core wait timed out: " + which.substr(2) +
                                     "; the outputs since the last check are invalid");
    }
  }
  return F3D_OK;
}

int f3d_last_kernel_ms(f3d_engine* e, float* ms) {
  if (!e || !ms) return fail_thread(F3D_E_PARAM, "FFT3DCL: null argument");
  Lock l(e);
  ms[0] = ms[1] = ms[2] = -1.0f;
  if (e->fwd_timed) cudaEventElapsedTime(&ms[0], e->ev[0], e->ev[1]);
  if (e->proc_timed) {
    cudaEventElapsedTime(&ms[1], e->ev[2], e->ev[4]);
    cudaEventElapsedTime(&ms[2], e->ev[4], e->ev[3]);
  }
  cudaGetLastError();
  return F3D_OK;
}

int f3d_live_instances(void) { return g_live.load(); }
size_t f3d_live_bytes(void) { return g_bytes.load(); }
uint64_t f3d_kernel_launches(void) { return launch_count(); }

}  // extern "C"

// ---- batches of planes ------------------------------------------------------

struct f3d_batch {
  std::vector<f3d_engine*> eng;
  int flags = 0;
  cudaStream_t stream = nullptr;
  TcTune tune;
  bool tuned = false;
  struct Graph {
    cudaGraph_t g = nullptr;
    cudaGraphExec_t x = nullptr;
    int kernels = 0;
  };
  std::map<uint64_t, Graph> graphs;  // by the planes with a forward (bits 0-15), an output (16-31), overlap (32)
  std::string err;
  // Side stream of the forward when it does not feed this step's outputs.
  cudaStream_t side = nullptr;
  cudaEvent_t fork = nullptr, join = nullptr;
  // Kernel timing of the last step run outside a graph: before the filter,
  // after it, after the inverse kernels.
  cudaEvent_t kev[3] = {nullptr, nullptr, nullptr};
  bool ktimed = false;
  // Entries whose engine appeared earlier in the batch (one more output of
  // that plane per step) have operand tiles and seam rows of their own.
  std::vector<uint8_t*> img;   // per entry, null: the engine's own
  std::vector<float*> seam;
  std::vector<size_t> img_bytes, seam_bytes;
  std::vector<bool> repeat;    // per entry: its engine appeared earlier
  // Fast-form engines: the forwards launch per entry, the fused sweeps of
  // all entries as one launch; no graph, no launch shapes to tune.
  bool fast = false;
};

namespace {

// Autotuner results by batch shape, shared by all batches of the process.
std::mutex g_tune_mtx;
std::map<std::string, TcTune> g_tune_cache;

std::string tune_key(const f3d_batch* b) {
  std::string k;
  for (const f3d_engine* e : b->eng)
    k += std::to_string(e->geom.width) + "x" + std::to_string(e->geom.height) + "b" + std::to_string(e->fmt) + "m" +
         std::to_string(e->ip.bm) + ";";
  return k;
}

int batch_fail(f3d_batch* b, int code, const std::string& m) {
  b->err = m;
  return fail_thread(code, m);
}

}  // namespace

extern "C" {

int f3d_batch_create(f3d_engine* const* engines, int n, int flags, f3d_batch** out) {
  if (!engines || !out || n < 1 || n > kMaxBatch)
    return fail_thread(F3D_E_PARAM, "FFT3DCL: a batch holds 1 to " + std::to_string(kMaxBatch) + " engines");
  *out = nullptr;
  const f3d_engine* e0 = engines[0];
  for (int i = 0; i < n; i++) {
    const f3d_engine* e = engines[i];
    if (!e) return fail_thread(F3D_E_PARAM, "FFT3DCL: null engine in batch");
    const bool tc = e->form == F3D_FORM_TC && e->inv_form == F3D_FORM_TC && e->fused;
    const bool fast = e->form == F3D_FORM_FAST && e->inv_form == F3D_FORM_FAST && e->fused;
    if (!tc && !fast)
      return fail_thread(F3D_E_UNSUPPORTED, "FFT3DCL: batches run the fused tensor-core or fast form");
    if (e->form != e0->form)
      return fail_thread(F3D_E_UNSUPPORTED, "FFT3DCL: the engines of a batch run one form");
    if (e->device != e0->device || e->stream != e0->stream)
      return fail_thread(F3D_E_PARAM, "FFT3DCL: the engines of a batch share one device and stream");
    if (e->ip.bw != e0->ip.bw || e->ip.bh != e0->ip.bh || e->ip.ow != e0->ip.ow || e->ip.oh != e0->ip.oh ||
        e->ip.wintype != e0->ip.wintype || e->ip.bm != e0->ip.bm || e->fmt != e0->fmt || e->half != e0->half)
      return fail_thread(F3D_E_UNSUPPORTED, "FFT3DCL: the planes of a batch share block size, overlap, window, "
                                            "temporal mode, format and spectrum storage");
  }
  auto* b = new f3d_batch();
  b->eng.assign(engines, engines + n);
  b->flags = flags;
  b->stream = e0->stream;
  cudaSetDevice(e0->device);
  b->img.assign(n, nullptr);
  b->seam.assign(n, nullptr);
  b->img_bytes.assign(n, 0);
  b->seam_bytes.assign(n, 0);
  b->repeat.assign(n, false);
  b->fast = e0->form == F3D_FORM_FAST;
  for (int i = 0; i < n; i++) {
    // An engine that appears k times enters k frames per step.
    int k = 0;
    for (int j = 0; j < n; j++) k += engines[j] == engines[i];
    {
      std::lock_guard<std::mutex> lk(engines[i]->mtx);
      engines[i]->pool_min = std::max(engines[i]->pool_min, k);
    }
    bool repeat = false;
    for (int j = 0; j < i; j++) repeat |= engines[j] == engines[i];
    if (!repeat) continue;
    b->repeat[i] = true;
    const f3d_engine* e = engines[i];
    b->img_bytes[i] = b->fast ? 0 : e->img_bytes;  // the fast sweep has no operand tiles
    b->seam_bytes[i] = sizeof(float) * e->seam_floats;
    if ((b->img_bytes[i] && cudaMalloc(&b->img[i], b->img_bytes[i]) != cudaSuccess) ||
        (b->seam_bytes[i] && cudaMalloc(&b->seam[i], b->seam_bytes[i]) != cudaSuccess)) {
      cudaGetLastError();
      f3d_batch_destroy(b);
      return fail_thread(F3D_E_NOMEM, "FFT3DCL: batch output buffers could not be allocated");
    }
  }
  if (cudaStreamCreateWithFlags(&b->side, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&b->join, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreate(&b->kev[0]) != cudaSuccess || cudaEventCreate(&b->kev[1]) != cudaSuccess ||
      cudaEventCreate(&b->kev[2]) != cudaSuccess) {
    cudaGetLastError();
    f3d_batch_destroy(b);
    return fail_thread(F3D_E_CUDA, "FFT3DCL: batch stream creation failed");
  }
  if (!b->fast) {  // the fast form has no launch shapes to tune
    std::lock_guard<std::mutex> lk(g_tune_mtx);
    auto it = g_tune_cache.find(tune_key(b));
    if (it != g_tune_cache.end()) {
      b->tune = it->second;
      b->tuned = true;
    }
  }
  *out = b;
  return F3D_OK;
}

void f3d_batch_destroy(f3d_batch* b) {
  if (!b) return;
  cudaSetDevice(b->eng[0]->device);
  if (b->stream) cudaStreamSynchronize(b->stream);
  if (b->side) cudaStreamSynchronize(b->side);
  for (auto& kv : b->graphs) {
    if (kv.second.x) cudaGraphExecDestroy(kv.second.x);
    if (kv.second.g) cudaGraphDestroy(kv.second.g);
  }
  if (b->fork) cudaEventDestroy(b->fork);
  if (b->join) cudaEventDestroy(b->join);
  for (cudaEvent_t ev : b->kev)
    if (ev) cudaEventDestroy(ev);
  if (b->side) cudaStreamDestroy(b->side);
  for (uint8_t* p : b->img)
    if (p) cudaFree(p);
  for (float* p : b->seam)
    if (p) cudaFree(p);
  delete b;
}

const char* f3d_batch_error(f3d_batch* b) { return b ? b->err.c_str() : ""; }

int f3d_batch_step(f3d_batch* b, const int* fns, const void* const* dev_src, const size_t* src_pitch,
                   const int* const* windows, const int* nwin, void* const* dev_dst, const size_t* dst_pitch) {
  if (!b || !fns || !dev_src || !src_pitch || !windows || !nwin || !dev_dst || !dst_pitch)
    return fail_thread(F3D_E_PARAM, "FFT3DCL: null argument");
  const int n = (int)b->eng.size();
  std::vector<std::unique_lock<std::mutex>> locks;
  for (int i = 0; i < n; i++) {
    bool seen = false;
    for (int j = 0; j < i; j++) seen |= b->eng[j] == b->eng[i];
    if (!seen) locks.emplace_back(b->eng[i]->mtx);
  }
  cudaSetDevice(b->eng[0]->device);
  TcFwdArgs fa[kMaxBatch];
  FwdArgs ff[kMaxBatch];  // fast form
  SweepArgs sa[kMaxBatch];
  int nf = 0;
  uint64_t mask = 0;
  for (int i = 0; i < n; i++) {
    f3d_engine* e = b->eng[i];
    if (fns[i] >= 0 && !e->cache.count(fns[i])) {
      if (!dev_src[i] || src_pitch[i] < (size_t)e->geom.width * e->bps)
        return batch_fail(b, F3D_E_PARAM, "FFT3DCL: bad source plane in batch");
      float2* spec = spectra_slot(e, fns[i], true);
      if (!spec) return batch_fail(b, F3D_E_NOMEM, "FFT3DCL: GPU spectra alloc failed");
      const uint8_t* src = static_cast<const uint8_t*>(dev_src[i]);
      if (b->fast) ff[nf] = forward_args(e, src, (long long)src_pitch[i], e->fmt, spec);
      else fa[nf] = tc_forward_args(e, src, (long long)src_pitch[i], e->fmt, spec);
      nf++;
      mask |= 1ull << i;
    }
  }
  int ns = 0;
  for (int i = 0; i < n; i++) {
    if (nwin[i] <= 0) continue;  // forward only
    f3d_engine* e = b->eng[i];
    InvArgs a;
    int rc = inverse_args(e, windows[i], nwin[i], a);
    if (rc != F3D_OK) return batch_fail(b, rc, e->err);
    if (!dev_dst[i] || dst_pitch[i] < (size_t)e->geom.width * e->bps)
      return batch_fail(b, F3D_E_PARAM, "FFT3DCL: bad output plane in batch");
    sa[ns] = sweep_args(e, a, static_cast<uint8_t*>(dev_dst[i]), (long long)dst_pitch[i], e->fmt);
    e->test_skip = false;
    if (b->repeat[i]) {  // a repeated engine: this output's own tiles and seam rows
      sa[ns].img = b->img[i];
      sa[ns].seam_b = b->seam[i];
      sa[ns].seam_t = b->seam[i] ? b->seam[i] + (size_t)(sa[ns].segs - 1) * (a.g.bh / 2) * sa[ns].seam_w : nullptr;
    }
    ns++;
    mask |= 1ull << (16 + i);
  }
  if (nf == 0 && ns == 0) return F3D_OK;
  // When no plane's entering frame is in its own window (the caller runs one
  // frame ahead), the forward does not feed this step's outputs: it runs on a
  // side stream once the filter is done, concurrently with the inverse, and
  // joins the main stream at the end of the step (the next step's outputs
  // need it).
  bool overlap = nf > 0 && ns > 0;
  for (int i = 0; i < n && overlap; i++)
    if (fns[i] >= 0 && (mask & (1ull << i)))
      for (int j = 0; j < n; j++)
        if (b->eng[j] == b->eng[i])
          for (int k = 0; k < nwin[j]; k++)
            if (windows[j][k] == fns[i]) overlap = false;
  if (overlap) mask |= 1ull << 32;
  // Filter, inverse and seam merge; timed by events unless being captured.
  auto sweep = [&](const TcTune& t, cudaEvent_t after_filter) -> cudaError_t {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    cudaStreamIsCapturing(b->stream, &cs);
    const bool timed = cs == cudaStreamCaptureStatusNone;
    if (timed) cudaEventRecord(b->kev[0], b->stream);
    cudaError_t ce = b->fast ? launch_sweep_fast_batch(sa, ns, b->stream, timed ? b->kev[1] : nullptr)
                             : launch_sweep_tc_batch(sa, ns, t, b->stream, timed ? b->kev[1] : nullptr, after_filter);
    if (timed && ce == cudaSuccess) {
      cudaEventRecord(b->kev[2], b->stream);
      b->ktimed = true;
    }
    return ce;
  };
  auto forwards = [&](const TcTune& t, cudaStream_t st) -> cudaError_t {
    if (!b->fast) return launch_forward_tc_batch(fa, nf, t, st);
    for (int k = 0; k < nf; k++) {
      const cudaError_t ce = launch_forward(F3D_FORM_FAST, ff[k], st);
      if (ce != cudaSuccess) return ce;
    }
    return cudaSuccess;
  };
  auto launch = [&](const TcTune& t) -> cudaError_t {
    cudaError_t ce = cudaSuccess;
    if (overlap && b->fast) {  // the fused fast sweep has no filter-only part: fork at the start
      ce = cudaEventRecord(b->fork, b->stream);
      if (ce == cudaSuccess) ce = cudaStreamWaitEvent(b->side, b->fork, 0);
      if (ce == cudaSuccess) ce = forwards(t, b->side);
      if (ce == cudaSuccess) ce = cudaEventRecord(b->join, b->side);
      if (ce == cudaSuccess) ce = sweep(t, nullptr);
      if (ce == cudaSuccess) ce = cudaStreamWaitEvent(b->stream, b->join, 0);
      return ce;
    }
    if (overlap) {
      ce = sweep(t, b->fork);
      if (ce == cudaSuccess) ce = cudaStreamWaitEvent(b->side, b->fork, 0);
      if (ce == cudaSuccess) ce = forwards(t, b->side);
      if (ce == cudaSuccess) ce = cudaEventRecord(b->join, b->side);
      if (ce == cudaSuccess) ce = cudaStreamWaitEvent(b->stream, b->join, 0);
      return ce;
    }
    ce = nf ? forwards(t, b->stream) : cudaSuccess;
    if (ce == cudaSuccess && ns) ce = sweep(t, nullptr);
    return ce;
  };
  // Autotuner: on the first step in which every plane enters a new frame,
  // time each candidate launch shape four times, interleaved (the step's
  // result is the same for all of them; the last run leaves it in place),
  // and keep the one with the fastest run, the default unless that is more
  // than 1 % slower: step-to-step noise of about 1 % picked a filter variant
  // 1-3 % slower in steady state at eight and ten outputs.
  const uint64_t all = (1ull << n) - 1;
  if (!b->fast && (b->flags & F3D_BATCH_AUTOTUNE) && !b->tuned && (mask & 0xFFFFFFFFull) == (all | (all << 16))) {
    const TcTune cands[] = {{3, 5}, {2, 5}, {1, 5}, {3, 4}, {2, 4}, {1, 4}, {3, 3}, {2, 3}, {1, 3}};
    constexpr int kCands = sizeof(cands) / sizeof(cands[0]);
    cudaEvent_t t0, t1;
    cudaEventCreate(&t0);
    cudaEventCreate(&t1);
    float fastest[kCands];
    for (float& f : fastest) f = 1e30f;
    for (int rep = 0; rep < 4; rep++)
      for (int c = 0; c < kCands; c++) {
        cudaEventRecord(t0, b->stream);
        cudaError_t ce = launch(cands[c]);
        cudaEventRecord(t1, b->stream);
        if (ce == cudaSuccess) ce = cudaEventSynchronize(t1);
        if (ce != cudaSuccess) {
          cudaEventDestroy(t0);
          cudaEventDestroy(t1);
          return batch_fail(b, F3D_E_CUDA, std::string("FFT3DCL: autotune launch: ") + cudaGetErrorString(ce));
        }
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, t0, t1);
        fastest[c] = std::min(fastest[c], ms);
      }
    cudaEventDestroy(t0);
    cudaEventDestroy(t1);
    // The default shape (the first candidate) stays unless another is more
    // than 1 % faster: single-step timings vary by about that much.
    b->tune = cands[autotune_pick(fastest, kCands)];
    b->tuned = true;
    std::lock_guard<std::mutex> lk(g_tune_mtx);
    g_tune_cache[tune_key(b)] = b->tune;
    return launch(b->tune) == cudaSuccess ? F3D_OK : batch_fail(b, F3D_E_CUDA, "FFT3DCL: batch launch failed");
  }
  cudaError_t ce = cudaSuccess;
  if ((b->flags & F3D_BATCH_GRAPH) && !b->fast) {  // fast batches launch directly
    // One CUDA graph per batch shape, captured at its first step; later steps
    // re-point its kernel nodes at the step's buffers and replay it.
    auto it = b->graphs.find(mask);
    if (it == b->graphs.end()) {
      f3d_batch::Graph gr;
      ce = cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeRelaxed);
      const long long l0 = f3d_kernel_launches();
      if (ce == cudaSuccess) {
        cudaError_t le = launch(b->tune);
        ce = cudaStreamEndCapture(b->stream, &gr.g);
        if (le != cudaSuccess) ce = le;
      }
      if (ce == cudaSuccess) ce = cudaGraphInstantiate(&gr.x, gr.g, 0);
      gr.kernels = (int)(f3d_kernel_launches() - l0);
      if (ce == cudaSuccess) ce = cudaGraphLaunch(gr.x, b->stream);
      if (ce != cudaSuccess) {
        if (gr.x) cudaGraphExecDestroy(gr.x);
        if (gr.g) cudaGraphDestroy(gr.g);
        cudaGetLastError();
        return batch_fail(b, F3D_E_CUDA, std::string("FFT3DCL: batch graph: ") + cudaGetErrorString(ce));
      }
      b->graphs[mask] = gr;
      return F3D_OK;
    }
    ce = tc_graph_update(it->second.x, it->second.g, fa, nf, sa, ns);
    if (ce == cudaSuccess) ce = cudaGraphLaunch(it->second.x, b->stream);
    if (ce == cudaSuccess)
      for (int k = 0; k < it->second.kernels; k++) count_launch();
  } else {
    ce = launch(b->tune);
  }
  if (ce != cudaSuccess) return batch_fail(b, F3D_E_CUDA, std::string("FFT3DCL: batch launch: ") + cudaGetErrorString(ce));
  return F3D_OK;
}

int f3d_batch_tune(f3d_batch* b, int* fwd_ctas_per_sm, int* filter_minb) {
  if (!b) return fail_thread(F3D_E_PARAM, "FFT3DCL: null batch");
  if (fwd_ctas_per_sm) *fwd_ctas_per_sm = b->tune.fwd_ctas_per_sm;
  if (filter_minb) *filter_minb = b->tune.filter_minb;
  return b->tuned ? 1 : 0;
}

int f3d_batch_last_kernel_ms(f3d_batch* b, float* ms) {
  if (!b || !ms) return fail_thread(F3D_E_PARAM, "FFT3DCL: null argument");
  if (!b->ktimed) return batch_fail(b, F3D_E_STATE, "FFT3DCL: no batch step with outputs ran outside a CUDA graph");
  cudaSetDevice(b->eng[0]->device);
  cudaError_t ce = cudaEventSynchronize(b->kev[2]);
  if (ce == cudaSuccess) ce = cudaEventElapsedTime(&ms[0], b->kev[0], b->kev[1]);
  if (ce == cudaSuccess) ce = cudaEventElapsedTime(&ms[1], b->kev[1], b->kev[2]);
  if (ce != cudaSuccess)
    return batch_fail(b, F3D_E_CUDA, std::string("FFT3DCL: batch kernel timing: ") + cudaGetErrorString(ce));
  return F3D_OK;
}

int f3d_batch_set_tune(f3d_batch* b, int fwd_ctas_per_sm, int filter_minb) {
  if (!b) return fail_thread(F3D_E_PARAM, "FFT3DCL: null batch");
  if (fwd_ctas_per_sm < 1 || fwd_ctas_per_sm > 3 || filter_minb < 3 || filter_minb > 5)
    return batch_fail(b, F3D_E_PARAM, "FFT3DCL: unsupported launch shape");
  cudaSetDevice(b->eng[0]->device);
  if (b->stream) cudaStreamSynchronize(b->stream);
  // Graphs captured with the previous shape are rebuilt at their next step.
  for (auto& kv : b->graphs) {
    if (kv.second.x) cudaGraphExecDestroy(kv.second.x);
    if (kv.second.g) cudaGraphDestroy(kv.second.g);
  }
  b->graphs.clear();
  b->tune = TcTune{fwd_ctas_per_sm, filter_minb};
  b->tuned = true;
  return F3D_OK;
}

}  // extern "C"


// ---- engine steps shared across engines (the serving loop) -----------------

#include "f3d_engine_internal.hpp"

namespace f3d {

bool engine_batchable(const f3d_engine* e) {
  return e && e->form == F3D_FORM_TC && e->inv_form == F3D_FORM_TC && e->fused;
}

namespace {
uint64_t batch_key(const f3d_internal_params& p, int fmt, bool half) {
  return (uint64_t)p.bw | ((uint64_t)p.bh << 10) | ((uint64_t)p.ow << 20) | ((uint64_t)p.oh << 30) |
         ((uint64_t)p.wintype << 40) | ((uint64_t)(p.bm + 1) << 42) | ((uint64_t)fmt << 46) |
         ((uint64_t)half << 52);
}
}  // namespace

uint64_t engine_batch_key(const f3d_engine* e) { return batch_key(e->ip, e->fmt, e->half); }

uint64_t plane_batch_key(const f3d_internal_params& p, const f3d_plane_geom& g) {
  return batch_key(p, g.sample_type == 1 ? FMT_F32 : (g.bits <= 8 ? FMT_U8 : FMT_U16), false);
}

int engines_step(f3d_engine* const* eng, int n, const int* fns, const void* const* src, const size_t* src_pitch,
                 const int* const* win, const int* nwin, void* const* dst, const size_t* dst_pitch, cudaStream_t st,
                 std::string* err) {
  auto bad = [&](int code, const std::string& m) {
    if (err) *err = m;
    return code;
  };
  if (n < 1 || n > kMaxBatch) return bad(F3D_E_PARAM, "FFT3DCL: a shared step holds 1 to 16 engines");
  for (int i = 0; i < n; i++) {
    if (!engine_batchable(eng[i]) || eng[i]->stream != st ||
        engine_batch_key(eng[i]) != engine_batch_key(eng[0]))
      return bad(F3D_E_UNSUPPORTED, "FFT3DCL: engines of a shared step run the fused tensor-core form alike");
    for (int j = 0; j < i; j++)
      if (eng[j] == eng[i]) return bad(F3D_E_PARAM, "FFT3DCL: an engine appears twice in a shared step");
  }
  std::vector<std::unique_lock<std::mutex>> locks;
  for (int i = 0; i < n; i++) locks.emplace_back(eng[i]->mtx);
  TcFwdArgs fa[kMaxBatch];
  SweepArgs sa[kMaxBatch];
  int nf = 0, ns = 0;
  for (int i = 0; i < n; i++) {
    f3d_engine* e = eng[i];
    if (fns[i] < 0 || e->cache.count(fns[i])) continue;
    if (!src[i] || src_pitch[i] < (size_t)e->geom.width * e->bps)
      return bad(F3D_E_PARAM, "FFT3DCL: bad source plane in a shared step");
    float2* spec = spectra_slot(e, fns[i], true);
    if (!spec) return bad(F3D_E_NOMEM, "FFT3DCL: GPU spectra alloc failed");
    fa[nf++] = tc_forward_args(e, static_cast<const uint8_t*>(src[i]), (long long)src_pitch[i], e->fmt, spec);
  }
  for (int i = 0; i < n; i++) {
    if (nwin[i] <= 0) continue;
    f3d_engine* e = eng[i];
    InvArgs a;
    const int rc = inverse_args(e, win[i], nwin[i], a);
    if (rc != F3D_OK) return bad(rc, e->err);
    if (!dst[i] || dst_pitch[i] < (size_t)e->geom.width * e->bps)
      return bad(F3D_E_PARAM, "FFT3DCL: bad output plane in a shared step");
    sa[ns++] = sweep_args(e, a, static_cast<uint8_t*>(dst[i]), (long long)dst_pitch[i], e->fmt);
    e->test_skip = false;
  }
  cudaSetDevice(eng[0]->device);
  cudaError_t ce = nf ? launch_forward_tc_batch(fa, nf, TcTune{}, st) : cudaSuccess;
  if (ce == cudaSuccess && ns) ce = launch_sweep_tc_batch(sa, ns, TcTune{}, st, nullptr);
  if (ce != cudaSuccess) return bad(F3D_E_CUDA, std::string("FFT3DCL: shared step launch: ") + cudaGetErrorString(ce));
  return F3D_OK;
}

}  // namespace f3d
