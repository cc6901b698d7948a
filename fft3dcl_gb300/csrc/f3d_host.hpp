// f3d_host.hpp -- parameter contract, block grid and tables of the engine.
//
// The values here must be the reference's own: the temporal filter compares
// against thresholds derived from them and the engine's exact form reproduces
// the reference output bit for bit. So every formula keeps the reference's
// expression and evaluation order (double where it uses double, float where
// it uses float), each one citing the reference file:line it restates.
#pragma once

#include "fft3d_gb300.h"

#include <cmath>
#include <cstdint>
#include <string>
#include <vector>

namespace f3d {

// roundPow2Clamp, src/params.h:62-72. The doubling runs in unsigned
// arithmetic; for v <= 0 the reference's loop wraps to 0 and the clamp gives 4.
inline int round_pow2_clamp(int v) {
  unsigned int logn = 0;
  for (unsigned int i = static_cast<unsigned int>(v - 1); i > 0; i /= 2, logn++)
    ;
  unsigned int r = 1;
  for (unsigned int i = 1; i <= logn; i++) r *= 2u;
  if (static_cast<int>(r) < 4) r = 4;
  if (r > 512u) r = 512u;
  return static_cast<int>(r);
}

// validateParams, src/params.h:76-148. Returns false with *err set on the
// reference's hard errors.
inline bool validate_params(const f3d_script_params& sp, int width, int height, int bits,
                            f3d_internal_params& out, std::string* err) {
  out = f3d_internal_params{};
  out.sigma = sp.sigma / 255.0f;
  out.beta = sp.beta;
  out.bm = sp.bt;
  if (out.bm < -1 || out.bm > 4) {
    *err = "FFT3DCL: valid modes for bt are -1,0,1,2,3,4";
    return false;
  }
  out.bt = sp.bt > 0 ? sp.bt : 1;
  out.sharpen = sp.sharpen;
  out.sharpen_on = sp.sharpen != 0.0f;
  out.mode = (sp.mode < 0 || sp.mode > 2) ? 0 : sp.mode;
  out.bordersize = sp.bordersize;
  out.degrid = sp.degrid;
  out.degrid_on = sp.degrid != 0.0f;
  out.scutoff = sp.scutoff;
  out.svr = sp.svr;
  out.smin = sp.smin / 255.0f;
  out.smax = sp.smax / 255.0f;
  out.kratio = sp.kratio;
  out.wintype = (sp.wintype < 0 || sp.wintype > 2) ? 0 : sp.wintype;
  out.interlaced = sp.interlaced;
  out.sigma2 = sp.sigma2;
  out.sigma3 = sp.sigma3;
  out.sigma4 = sp.sigma4;
  out.use_pattern = (sp.sigma != sp.sigma2 || sp.sigma3 != sp.sigma4 || sp.sigma != sp.sigma3);
  out.oldfft = sp.oldfft;
  out.current = (out.bm == 1) ? 0 : (out.bm == 4) ? 2 : 1;

  if (sp.bw <= 0 || sp.bh <= 0) {
    // The reference divides by the script bw/bh when scaling ow/oh below.
    *err = "FFT3DCL: bw and bh must be positive";
    return false;
  }
  out.bw = round_pow2_clamp(sp.bw);
  out.bh = round_pow2_clamp(sp.bh);
  out.ow = static_cast<int>(sp.ow * (float)out.bw / (float)sp.bw);
  out.ow &= static_cast<int>(0xFFFFFFFE);
  out.oh = static_cast<int>(sp.oh * (float)out.bh / (float)sp.bh);
  if (out.oh * 2 > out.bh) out.oh = out.bh / 2;
  if (out.ow * 2 > out.bw) out.ow = out.bw / 2;

  int precision = sp.precision;
  if (bits > 8) precision = 2;
  if (precision < 0 || precision > 2) precision = 1;
  out.precision = precision;

  if (out.mode == 2) {
    *err = "FFT3DCL: mode 2 is not implemented yet in this port (use mode 0 or 1)";
    return false;
  }
  if (out.interlaced) {
    *err = "FFT3DCL: interlaced is not implemented yet in this port";
    return false;
  }
  if (out.mode == 0 || (out.bw == out.ow * 2 && out.bh == out.oh * 2)) {
    out.ny = static_cast<int>((height + out.bh * 1.5 - 1) / out.bh);
    out.nx = static_cast<int>((width + out.bw * 1.5 - 1) / out.bw);
  } else {
    if (out.bw - out.ow <= 0 || out.bh - out.oh <= 0) {
      *err = "FFT3DCL: overlap must be smaller than the block";
      return false;
    }
    out.nx = ((width + out.ow - 1) / (out.bw - out.ow) + 1 + 1) / 2;
    out.ny = ((height + out.oh - 1) / (out.bh - out.oh) + 1 + 1) / 2;
  }
  out.totw = out.nx * out.bw;
  out.toth = out.ny * out.bh;

  out.wiener_s = out.sigma * out.sigma * out.bt * out.bw * out.bh;
  out.beta_x = (out.beta - 1.0f) / out.beta;
  out.kalman_cn = out.sigma * out.sigma * out.bw * out.bh;
  out.ssmin = out.smin * out.smin * out.bw * out.bh * out.bt;
  out.ssmax = out.smax * out.smax * out.bw * out.bh * out.bt;
  return true;
}

// Block grid of one plane (src/cpu/reference.cpp:19-58): mode 1 is a
// 2nx x 2ny grid at (-ow + n(bw-ow), -oh + m(bh-oh)); mode 0 is two nx x ny
// grids, the second shifted by (-bw/2, -bh/2). Blocks are numbered row-major,
// grid 0 first; the per-pixel overlap-add follows this order.
struct Grid {
  int mode = 1;
  int nb = 0, ncols = 0, nrows = 0, nx = 0, ny = 0;
  int xoff = 0, xstep = 0, yoff = 0, ystep = 0;
};

inline Grid make_grid(const f3d_internal_params& p) {
  Grid g;
  g.mode = p.mode;
  g.nx = p.nx;
  g.ny = p.ny;
  if (p.mode == 0) {
    g.ncols = p.nx;
    g.nrows = p.ny;
    g.nb = 2 * p.nx * p.ny;
    g.xoff = 0;
    g.xstep = p.bw;
    g.yoff = 0;
    g.ystep = p.bh;
  } else {
    g.ncols = 2 * p.nx;
    g.nrows = 2 * p.ny;
    g.nb = g.ncols * g.nrows;
    g.xoff = -p.ow;
    g.xstep = p.bw - p.ow;
    g.yoff = -p.oh;
    g.ystep = p.bh - p.oh;
  }
  return g;
}

constexpr double kPi = 3.14159265358979323846;

// The table builders below write into caller storage and allocate nothing,
// so that the no-alloc entry point (f3d_noalloc.cu) can use them with stack
// storage; the vector-returning versions further down wrap them.

// FftPlan twiddles, src/cpu/fft.cpp:8-14: exp(-2*pi*i*k/n) in double, stored
// as float, k < n/2; interleaved re, im (n floats).
inline void twiddles_into(int n, float* tw) {
  for (int k = 0; k < n / 2; k++) {
    double a = -2.0 * 3.14159265358979323846 * k / n;
    tw[2 * k] = (float)std::cos(a);
    tw[2 * k + 1] = (float)std::sin(a);
  }
}

// buildWindowMode0, src/cpu/tables.cpp:8-19 (bw*bh floats).
inline void window_mode0_into(int bw, int bh, float* w) {
  int off = 0;
  for (double n1 = -bh / 2.0 + 0.5; n1 < bh / 2.0; n1++) {
    double cosy = std::cos(n1 * kPi / bh);
    for (double n2 = -bw / 2.0 + 0.5; n2 < bw / 2.0; n2++) {
      double cosx = std::cos(n2 * kPi / bw);
      w[off++] = (float)std::sqrt(0.5 * (cosx * cosx + cosy * cosy));
    }
  }
}

// Ramp i (0 <= i < o) of the mode-1 analysis and synthesis windows of one
// axis, src/cpu/tables.cpp:29-60.
inline void mode1_ramp(int i, int o, int wintype, double& an, double& syn) {
  const double hc = std::cos(kPi * (i - o + 0.5) / (o * 2.0));
  if (wintype == 1) {
    an = std::sqrt(hc);
    syn = an * an * an;
  } else if (wintype == 2) {
    an = 1.0;
    syn = hc;
    syn *= syn;
  } else {
    an = hc;
    syn = an;
  }
}

// Axis factors of the separable mode-1 windows, src/cpu/tables.cpp:62-105,
// with the odd grid's synthesis shift of src/cpu/reference.cpp:51-57:
// A[y][x] = float(ax[x] * ay[y]), synA[y][x] = float(sxa[x] * sy[y]),
// synB[y][x] = float(sxb[x] * sy[y]). ax, sxa, sxb hold bw doubles, ay, sy bh.
// Rising ramp, flat middle, falling ramp; the odd grid's synthesis ramp runs
// the other way round, sampled (bw - ow) further along x.
inline void mode1_axes_into(int bw, int bh, int ow, int oh, int wintype, double* ax, double* ay, double* sxa,
                            double* sxb, double* sy) {
  double an, syn;
  for (int lx = 0; lx < bw; lx++) {
    if (lx < ow) {
      mode1_ramp(lx, ow, wintype, an, syn);
      ax[lx] = an;
      sxa[lx] = syn;
    } else if (lx < bw - ow) {
      ax[lx] = sxa[lx] = 1.0;
    } else {
      mode1_ramp((ow - 1) - (lx - (bw - ow)), ow, wintype, an, syn);
      ax[lx] = an;
      sxa[lx] = syn;
    }
    // Odd-grid synthesis factor at lx' = (lx + bw - ow) % bw: wsynx[(ow-1)-lx']
    // on the rising part, 1 in the middle, wsynx[lx' - (bw-ow)] on the falling part.
    const int s = (lx + bw - ow) % bw;
    if (s < ow) {
      mode1_ramp((ow - 1) - s, ow, wintype, an, syn);
      sxb[lx] = syn;
    } else if (s < bw - ow) {
      sxb[lx] = 1.0;
    } else {
      mode1_ramp(s - (bw - ow), ow, wintype, an, syn);
      sxb[lx] = syn;
    }
  }
  for (int ly = 0; ly < bh; ly++) {
    if (ly < oh) {
      mode1_ramp(ly, oh, wintype, an, syn);
      ay[ly] = an;
      sy[ly] = syn;
    } else if (ly < bh - oh) {
      ay[ly] = sy[ly] = 1.0;
    } else {
      mode1_ramp(bh - 1 - ly, oh, wintype, an, syn);
      ay[ly] = an;
      sy[ly] = syn;
    }
  }
}

// buildWindowsMode1, src/cpu/tables.cpp:21-105, from the axis factors
// (bw*bh floats each).
inline void windows_mode1_into(int bw, int bh, const double* ax, const double* ay, const double* sxa,
                               const double* sxb, const double* sy, float* A, float* synA, float* synB) {
  for (int ly = 0; ly < bh; ly++)
    for (int lx = 0; lx < bw; lx++) {
      A[ly * bw + lx] = (float)(ax[lx] * ay[ly]);
      synA[ly * bw + lx] = (float)(sxa[lx] * sy[ly]);
      synB[ly * bw + lx] = (float)(sxb[lx] * sy[ly]);
    }
}

// buildPattern, src/cpu/tables.cpp:107-137 (float arithmetic as there;
// (bw/2+1)*bh floats).
inline void sigma_pattern_into(int bw, int bh, int bt, float sigma, float sigma2, float sigma3, float sigma4,
                               float* pat) {
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

// buildSharpenLUT, src/cpu/tables.cpp:139-156 ((bw/2+1)*bh floats).
inline void sharpen_lut_into(int bw, int bh, float strength, float svr, float scutoff, float* lut) {
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

// Largest transform length the host transform below takes (the reference
// rounds block sizes to at most 512, src/params.h:62-72).
constexpr int kMaxHostFft = 512;

// Reference radix-2 DIT transform (src/cpu/fft.cpp:28-58) on the host, used
// once per engine to build the degrid sample the same way the reference does.
// tw: interleaved twiddles of length n; in, out: n interleaved complex values.
inline void host_fft(int n, const float* tw, const float* in, float* out, bool inv) {
  float a[2 * kMaxHostFft];
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
        float wr = tw[2 * (j * step)], wi = tw[2 * (j * step) + 1];
        if (inv) wi = -wi;
        float br = a[2 * (i + j + half)], bi = a[2 * (i + j + half) + 1];
        float tr = wr * br - wi * bi, ti = wr * bi + wi * br;
        float ur = a[2 * (i + j)], ui = a[2 * (i + j) + 1];
        a[2 * (i + j)] = ur + tr;
        a[2 * (i + j) + 1] = ui + ti;
        a[2 * (i + j + half)] = ur - tr;
        a[2 * (i + j + half) + 1] = ui - ti;
      }
  }
  const float invn = 1.0f / n;
  for (int i = 0; i < 2 * n; i++) out[i] = inv ? a[i] * invn : a[i];
}

// buildDegridSample, src/cpu/reference.cpp:172-198: FFT of the analysis
// window (the reference transforms a white frame, whose blocks all equal the
// window) divided by its DC and scaled by degrid. One fbw x bh table serves
// every block; gs receives 2*fbw*bh floats, interleaved re, im. The row
// transforms keep their fbw columns and only those columns are transformed
// (column transforms are independent of each other).
inline void degrid_sample_into(int bw, int bh, float degrid, const float* win, const float* tw_row,
                               const float* tw_col, float* gs) {
  const int fbw = bw / 2 + 1;
  float buf[2 * kMaxHostFft], res[2 * kMaxHostFft];
  for (int r = 0; r < bh; r++) {
    for (int c = 0; c < bw; c++) {
      buf[2 * c] = win[r * bw + c];
      buf[2 * c + 1] = 0.0f;
    }
    host_fft(bw, tw_row, buf, res, false);
    for (int c = 0; c < fbw; c++) {
      gs[2 * (r * fbw + c)] = res[2 * c];
      gs[2 * (r * fbw + c) + 1] = res[2 * c + 1];
    }
  }
  for (int c = 0; c < fbw; c++) {
    for (int r = 0; r < bh; r++) {
      buf[2 * r] = gs[2 * (r * fbw + c)];
      buf[2 * r + 1] = gs[2 * (r * fbw + c) + 1];
    }
    host_fft(bh, tw_col, buf, res, false);
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

// ---- vector-returning wrappers (the engine) ---------------------------------

inline std::vector<float> twiddles(int n) {
  std::vector<float> tw(n);
  twiddles_into(n, tw.data());
  return tw;
}

inline std::vector<float> window_mode0(int bw, int bh) {
  std::vector<float> w(bw * bh);
  window_mode0_into(bw, bh, w.data());
  return w;
}

struct Mode1Axes {
  std::vector<double> ax, ay, sxa, sxb, sy;
};
inline Mode1Axes mode1_axes(int bw, int bh, int ow, int oh, int wintype) {
  Mode1Axes a{std::vector<double>(bw), std::vector<double>(bh), std::vector<double>(bw),
              std::vector<double>(bw), std::vector<double>(bh)};
  mode1_axes_into(bw, bh, ow, oh, wintype, a.ax.data(), a.ay.data(), a.sxa.data(), a.sxb.data(), a.sy.data());
  return a;
}
inline void windows_mode1(int bw, int bh, int ow, int oh, int wintype, std::vector<float>& A,
                          std::vector<float>& synA, std::vector<float>& synB, Mode1Axes* axes = nullptr) {
  const Mode1Axes a = mode1_axes(bw, bh, ow, oh, wintype);
  A.assign(bw * bh, 0.0f);
  synA.assign(bw * bh, 0.0f);
  synB.assign(bw * bh, 0.0f);
  windows_mode1_into(bw, bh, a.ax.data(), a.ay.data(), a.sxa.data(), a.sxb.data(), a.sy.data(), A.data(),
                     synA.data(), synB.data());
  if (axes) *axes = a;
}

inline std::vector<float> sigma_pattern(int bw, int bh, int bt, float sigma, float sigma2, float sigma3,
                                        float sigma4) {
  std::vector<float> pat((bw / 2 + 1) * bh);
  sigma_pattern_into(bw, bh, bt, sigma, sigma2, sigma3, sigma4, pat.data());
  return pat;
}

inline std::vector<float> sharpen_lut(int bw, int bh, float strength, float svr, float scutoff) {
  std::vector<float> lut((bw / 2 + 1) * bh);
  sharpen_lut_into(bw, bh, strength, svr, scutoff, lut.data());
  return lut;
}

inline std::vector<float> degrid_sample(int bw, int bh, float degrid, const std::vector<float>& win) {
  std::vector<float> gs(2 * (bw / 2 + 1) * bh), twr = twiddles(bw), twc = twiddles(bh);
  degrid_sample_into(bw, bh, degrid, win.data(), twr.data(), twc.data(), gs.data());
  return gs;
}

// All host tables of one plane (the PlaneRef constructor,
// src/cpu/reference.cpp:19-61, and buildDegridSample :172-198). Tables that
// are off stay empty; twiddles and the degrid sample are interleaved re, im.
struct PlaneTables {
  std::vector<float> win_ana, syn_a, syn_b, pattern, sharpen, gs, tw_row, tw_col;
};

inline PlaneTables build_tables(const f3d_internal_params& ip) {
  PlaneTables t;
  t.tw_row = twiddles(ip.bw);
  t.tw_col = twiddles(ip.bh);
  if (ip.mode == 0)
    t.win_ana = window_mode0(ip.bw, ip.bh);
  else
    windows_mode1(ip.bw, ip.bh, ip.ow, ip.oh, ip.wintype, t.win_ana, t.syn_a, t.syn_b);
  if (ip.use_pattern)
    t.pattern = sigma_pattern(ip.bw, ip.bh, ip.bt, ip.sigma * 255.0f, ip.sigma2, ip.sigma3, ip.sigma4);
  if (ip.sharpen_on) t.sharpen = sharpen_lut(ip.bw, ip.bh, ip.sharpen, ip.svr, ip.scutoff);
  if (ip.degrid_on) t.gs = degrid_sample(ip.bw, ip.bh, ip.degrid, t.win_ana);
  return t;
}

// Table `which` (F3D_TAB_*) as a flat float vector; the degrid sample is
// split into its real and imaginary parts.
inline std::vector<float> table_of(const PlaneTables& t, int which) {
  switch (which) {
  case F3D_TAB_WIN_ANA: return t.win_ana;
  case F3D_TAB_WIN_SYN_A: return t.syn_a;
  case F3D_TAB_WIN_SYN_B: return t.syn_b;
  case F3D_TAB_PATTERN: return t.pattern;
  case F3D_TAB_SHARPEN: return t.sharpen;
  case F3D_TAB_GS_RE:
  case F3D_TAB_GS_IM: {
    std::vector<float> v;
    for (size_t i = (which == F3D_TAB_GS_IM); i < t.gs.size(); i += 2) v.push_back(t.gs[i]);
    return v;
  }
  case F3D_TAB_TWIDDLE_ROW: return t.tw_row;
  case F3D_TAB_TWIDDLE_COL: return t.tw_col;
  default: return {};
  }
}

// CHROMANORM, src/cpu/reference.cpp:70-79: mode-1 YUV chroma only.
inline float chroma_norm(const f3d_internal_params& p, const f3d_plane_geom& g) {
  if (p.mode != 1 || !g.chroma || g.sample_type == 1) return 0.0f;
  return g.bits <= 8 ? 128.0f / 255.0f : 32768.0f / 65535.0f;
}

} // namespace f3d
