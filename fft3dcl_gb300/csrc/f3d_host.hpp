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

// FftPlan twiddles, src/cpu/fft.cpp:8-14: exp(-2*pi*i*k/n) in double, stored
// as float, k < n/2; interleaved re, im.
inline std::vector<float> twiddles(int n) {
  std::vector<float> tw(n);
  for (int k = 0; k < n / 2; k++) {
    double a = -2.0 * 3.14159265358979323846 * k / n;
    tw[2 * k] = (float)std::cos(a);
    tw[2 * k + 1] = (float)std::sin(a);
  }
  return tw;
}

// buildWindowMode0, src/cpu/tables.cpp:8-19.
inline std::vector<float> window_mode0(int bw, int bh) {
  std::vector<float> w(bw * bh);
  int off = 0;
  for (double n1 = -bh / 2.0 + 0.5; n1 < bh / 2.0; n1++) {
    double cosy = std::cos(n1 * kPi / bh);
    for (double n2 = -bw / 2.0 + 0.5; n2 < bw / 2.0; n2++) {
      double cosx = std::cos(n2 * kPi / bw);
      w[off++] = (float)std::sqrt(0.5 * (cosx * cosx + cosy * cosy));
    }
  }
  return w;
}

// buildWindowsMode1, src/cpu/tables.cpp:21-105, plus the odd-parity synthesis
// window shifted by (bw-ow), src/cpu/reference.cpp:51-57.
// The windows are separable: A[y][x] = float(ax[x] * ay[y]), synA[y][x] =
// float(sxa[x] * sy[y]), synB[y][x] = float(sxb[x] * sy[y]) (sxb includes
// the odd grid's shift).
struct Mode1Axes {
  std::vector<double> ax, ay, sxa, sxb, sy;
};
inline void windows_mode1(int bw, int bh, int ow, int oh, int wintype, std::vector<float>& A,
                          std::vector<float>& synA, std::vector<float>& synB, Mode1Axes* axes = nullptr) {
  std::vector<double> wanx(ow), wany(oh), wsynx(ow), wsyny(oh);
  auto half_cos = [](int i, int o) { return std::cos(kPi * (i - o + 0.5) / (o * 2.0)); };
  for (int i = 0; i < ow; i++) {
    if (wintype == 1) {
      wanx[i] = std::sqrt(half_cos(i, ow));
      wsynx[i] = wanx[i] * wanx[i] * wanx[i];
    } else if (wintype == 2) {
      wanx[i] = 1.0;
      wsynx[i] = half_cos(i, ow);
      wsynx[i] *= wsynx[i];
    } else {
      wanx[i] = half_cos(i, ow);
      wsynx[i] = wanx[i];
    }
  }
  for (int i = 0; i < oh; i++) {
    if (wintype == 1) {
      wany[i] = std::sqrt(half_cos(i, oh));
      wsyny[i] = wany[i] * wany[i] * wany[i];
    } else if (wintype == 2) {
      wany[i] = 1.0;
      wsyny[i] = half_cos(i, oh);
      wsyny[i] *= wsyny[i];
    } else {
      wany[i] = half_cos(i, oh);
      wsyny[i] = wany[i];
    }
  }
  // Rising ramp, flat middle, falling ramp; the odd grid's synthesis ramp
  // runs the other way round.
  std::vector<double> wxA(bw), wxSA(bw), wxSB(bw), wyA(bh), wySA(bh);
  for (int lx = 0; lx < bw; lx++) {
    if (lx < ow) {
      wxA[lx] = wanx[lx];
      wxSA[lx] = wsynx[lx];
      wxSB[lx] = wsynx[(ow - 1) - lx];
    } else if (lx < bw - ow) {
      wxA[lx] = wxSA[lx] = wxSB[lx] = 1.0;
    } else {
      int x = lx - (bw - ow);
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
  if (axes) {
    // synB below is sb shifted cyclically by bw - ow along x.
    std::vector<double> sxb(bw);
    for (int lx = 0; lx < bw; lx++) sxb[lx] = wxSB[(lx + bw - ow) % bw];
    *axes = Mode1Axes{wxA, wyA, wxSA, sxb, wySA};
  }
  A.assign(bw * bh, 0.0f);
  synA.assign(bw * bh, 0.0f);
  std::vector<float> sb(bw * bh);
  for (int ly = 0; ly < bh; ly++)
    for (int lx = 0; lx < bw; lx++) {
      A[ly * bw + lx] = (float)(wxA[lx] * wyA[ly]);
      synA[ly * bw + lx] = (float)(wxSA[lx] * wySA[ly]);
      sb[ly * bw + lx] = (float)(wxSB[lx] * wySA[ly]);
    }
  synB.assign(bw * bh, 0.0f);
  for (int ly = 0; ly < bh; ly++)
    for (int lx = 0; lx < bw; lx++) synB[ly * bw + lx] = sb[ly * bw + ((lx + bw - ow) % bw)];
}

// buildPattern, src/cpu/tables.cpp:107-137 (float arithmetic as there).
inline std::vector<float> sigma_pattern(int bw, int bh, int bt, float sigma, float sigma2,
                                        float sigma3, float sigma4) {
  const int fbw = bw / 2 + 1;
  auto scale = [&](float s) {
    double v = s / 255.0;
    return (float)(v * v * bt * bw * bh);
  };
  float s = scale(sigma), s2 = scale(sigma2), s3 = scale(sigma3), s4 = scale(sigma4);
  float ft2 = (float)(std::sqrt(0.5) / 2.0);
  float ft3 = (float)(std::sqrt(0.5) / 4.0);
  std::vector<float> pat(fbw * bh);
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
  return pat;
}

// buildSharpenLUT, src/cpu/tables.cpp:139-156.
inline std::vector<float> sharpen_lut(int bw, int bh, float strength, float svr, float scutoff) {
  const int fbw = bw / 2 + 1;
  std::vector<float> lut(fbw * bh);
  for (int j = 0; j < bh; j++) {
    int dj = j >= bh / 2 ? bh - j : j;
    float d2v = (float)(dj * dj) * (svr * svr) / ((bh / 2.0f) * (bh / 2.0f));
    for (int i = 0; i < fbw; i++) {
      float d2 = d2v + (float)(i * i) / ((bw / 2.0f) * (bw / 2.0f));
      lut[j * fbw + i] = strength * (1.0f - std::exp(-d2 / (2.0f * scutoff * scutoff)));
    }
  }
  return lut;
}

// Reference radix-2 DIT transform (src/cpu/fft.cpp:28-58) on the host, used
// once per engine to build the degrid sample the same way the reference does.
inline void host_fft(int n, const std::vector<float>& tw, const float* in, float* out, bool inv) {
  std::vector<float> a(2 * n);
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
// every block. Interleaved re, im.
inline std::vector<float> degrid_sample(int bw, int bh, float degrid, const std::vector<float>& win) {
  const int fbw = bw / 2 + 1;
  std::vector<float> twr = twiddles(bw), twc = twiddles(bh);
  std::vector<float> full(2 * bw * bh), row(2 * bw), col(2 * bh), colout(2 * bh);
  for (int r = 0; r < bh; r++) {
    for (int c = 0; c < bw; c++) {
      row[2 * c] = win[r * bw + c];
      row[2 * c + 1] = 0.0f;
    }
    host_fft(bw, twr, row.data(), &full[2 * r * bw], false);
  }
  for (int c = 0; c < fbw; c++) {
    for (int r = 0; r < bh; r++) {
      col[2 * r] = full[2 * (r * bw + c)];
      col[2 * r + 1] = full[2 * (r * bw + c) + 1];
    }
    host_fft(bh, twc, col.data(), colout.data(), false);
    for (int r = 0; r < bh; r++) {
      full[2 * (r * bw + c)] = colout[2 * r];
      full[2 * (r * bw + c) + 1] = colout[2 * r + 1];
    }
  }
  std::vector<float> gs(2 * fbw * bh);
  const float dc = full[0];
  for (int r = 0; r < bh; r++)
    for (int c = 0; c < fbw; c++) {
      gs[2 * (r * fbw + c)] = full[2 * (r * bw + c)] / dc * degrid;
      gs[2 * (r * fbw + c) + 1] = full[2 * (r * bw + c) + 1] / dc * degrid;
    }
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
