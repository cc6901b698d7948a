// f3d_device.cuh -- device helpers shared by all kernel forms: block grid,
// pixel formats, the per-bin temporal filter and the radix-2 transforms.
//
// The arithmetic is written with plain operators. The exact-form translation
// units are compiled with --fmad=false and IEEE division and square root, so
// every expression rounds exactly like the reference's fp32 CPU code
// (src/cpu/reference.cpp) when it is written in the same order, which it is.
#pragma once

#include "f3d_kernels.hpp"
#include "fft3d_gb300.h"

#include <cuda_runtime.h>
#include <cstdint>

namespace f3d {

template <int N>
struct Log2 {
  static constexpr int v = 1 + Log2<N / 2>::v;
};
template <>
struct Log2<1> {
  static constexpr int v = 0;
};

__host__ __device__ constexpr int bit_reverse(int i, int bits) {
  int r = 0;
  for (int b = 0; b < bits; b++)
    if (i & (1 << b)) r |= 1 << (bits - 1 - b);
  return r;
}

// D3D9 MIRROR addressing, src/cpu/reference.cpp:10-17.
__device__ __forceinline__ int mirror_i(int x, int w) {
  int p = x % (2 * w);
  if (p < 0) p += 2 * w;
  if (p >= w) p = 2 * w - 1 - p;
  return p;
}

// Top-left corner and synthesis parity of block b (src/cpu/reference.cpp:23-46).
__device__ __forceinline__ void block_origin(const Geo& g, int b, int& bx, int& by, int& par) {
  if (g.mode == 1) {
    const int m = b / g.ncols, n = b - m * g.ncols;
    bx = g.xoff + n * g.xstep;
    by = g.yoff + m * g.ystep;
    par = n & 1;
  } else {
    const int per = g.ncols * g.nrows;
    const int grid = b >= per ? 1 : 0;
    const int r = b - grid * per;
    const int j = r / g.ncols, i = r - j * g.ncols;
    bx = i * g.bw - (grid ? g.bw / 2 : 0);
    by = j * g.bh - (grid ? g.bh / 2 : 0);
    par = 0;
  }
}

// Source sample to float, src/cpu/reference.cpp:82-105.
__device__ __forceinline__ float load_sample(const uint8_t* row, int x, int fmt, float norm) {
  if (fmt == FMT_U8) return (float)row[x] * (1.0f / 255.0f);
  if (fmt == FMT_U16) return (float)reinterpret_cast<const uint16_t*>(row)[x] * norm;
  return reinterpret_cast<const float*>(row)[x];
}

// Float to destination sample, src/cpu/reference.cpp:107-138. The product
// and the +0.5 are rounded separately (no fused multiply-add), and the cast
// truncates a non-negative value, i.e. floors it.
__device__ __forceinline__ uint32_t pack_u8(float v) {
  v = v < 0.0f ? 0.0f : (v > 1.0f ? 1.0f : v);
  return __float2uint_rz(__fadd_rn(__fmul_rn(v, 255.0f), 0.5f));
}
__device__ __forceinline__ uint32_t pack_u16(float v, float inv_norm, float max_pix) {
  v = __fmul_rn(v, inv_norm);
  v = v < max_pix ? v : max_pix;
  v = v < 0.0f ? 0.0f : (v > 1.0f ? 1.0f : v);
  return __float2uint_rz(__fadd_rn(__fmul_rn(v, 65535.0f), 0.5f));
}
__device__ __forceinline__ void store_sample(uint8_t* row, int x, float v, int fmt, float inv_norm,
                                             float max_pix) {
  if (fmt == FMT_U8) {
    row[x] = (uint8_t)pack_u8(v);
  } else if (fmt == FMT_U16) {
    reinterpret_cast<uint16_t*>(row)[x] = (uint16_t)pack_u16(v, inv_norm, max_pix);
  } else {
    reinterpret_cast<float*>(row)[x] = v;
  }
}

// Wiener shrink of one complex value, src/cpu/reference.cpp:201-209.
__device__ __forceinline__ void wienner(float& re, float& im, float sx, float sy, float beta_x) {
  float psd = re * re + im * im + 0.0000000000000000000000000000000000001f;
  float psd_inv = 1.0f / psd;
  float mul = beta_x;
  if (1.0f / sx > psd_inv) mul = 1.0f - sy * psd_inv;
  re *= mul;
  im *= mul;
}

// The same shrink for the fast forms. With sx = beta * sy (both the plain
// and the pattern sigmas are built that way) the factor 1 - sy/psd passes
// beta_x = 1 - 1/beta exactly at psd = sx and grows with psd, so the
// reference's branch is max(1 - sy/psd, beta_x); psd = 0 gives -inf -> beta_x.
template <bool FAST>
__device__ __forceinline__ void wienner_t(float& re, float& im, float sx, float sy, float beta_x) {
  if (!FAST) {
    wienner(re, im, sx, sy, beta_x);
    return;
  }
  const float psd = fmaf(re, re, im * im);
  const float mul = fmaxf(fmaf(-sy, 1.0f / psd, 1.0f), beta_x);
  re *= mul;
  im *= mul;
}

// Fast forms, temporal modes 2-4: the Wiener gain of one temporal
// frequency with the average's 1/bm folded in, s * max(1 - sy/psd, beta_x)
// evaluated as max(s - (s sy)/psd, s beta_x) (exact for s = 1/2, 1/4), so that
// the filtered value is a fused sum of gain x frequency.
__device__ __forceinline__ float wiener_gain_scaled(float re, float im, float ssy, float s, float sbx) {
  const float psd = fmaf(re, re, im * im);
  return fmaxf(fmaf(-ssy, 1.0f / psd, s), sbx);
}

// Temporal mode as a template argument: -1..4 fixed at compile time (no
// branch, and no Kalman state stores in the other modes' code, so the
// compiler may move spectra loads freely), kRuntimeBm to read a.bm.
constexpr int kRuntimeBm = -2;

// DC of block b in the current frame's spectrum (the degrid correction's scale).
__device__ __forceinline__ float block_dc(const InvArgs& a, int b) {
  return a.dg ? a.s[a.cur][(size_t)b * a.g.bh * a.g.fbw].x : 0.0f;
}

// The per-bin table values of bin i (0 <= i < bh*fbw): degrid sample, sigma
// pattern and sharpen factor, read only where they are on. Kernels that
// filter the same bin of several blocks read them once.
struct BinTables {
  float2 gs;
  float pat, shp;
};
__device__ __forceinline__ BinTables bin_tables(const InvArgs& a, int i) {
  BinTables t{make_float2(0.0f, 0.0f), 0.0f, 0.0f};
  if (a.dg) t.gs = a.gs[i];
  if (a.pat) t.pat = a.pattern[i];
  if (a.shp) t.shp = a.sharpen[i];
  return t;
}

// Kalman state of one bin as read before its update (a.kalman_init: unused).
struct KState {
  float2 last;
  float cov, proc;
};
__device__ __forceinline__ KState load_kstate(const InvArgs& a, size_t gi) {
  KState k{make_float2(0.0f, 0.0f), 0.0f, 0.0f};
  if (!a.kalman_init) {
    k.last = a.klast[gi];
    k.cov = a.kcov[gi];
    k.proc = a.kproc[gi];
  }
  return k;
}

// Temporal filter + sharpen of bin i (0 <= i < bh*fbw) of a block whose
// current-frame DC is dc, with tb the bin's tables (bin_tables(a, i)),
// gi = b*bh*fbw + i and sv the bin's window spectra (load_window). Follows
// src/cpu/reference.cpp:229-409 per bin: degrid correction, bm 2/3/4
// temporal DFT + Wiener, bm 1 Wiener, bm 0 Kalman (state updated in place),
// bm -1 pass-through, then sharpen. FAST evaluates the 3- and 4-point
// temporal transforms with fewer additions (a different rounding; the exact
// form keeps the reference's expressions).
// ks: the bin's Kalman state (bm 0) as load_kstate read it, so that a
// caller can issue the loads of several bins before their updates.
template <int BM, bool FAST = false>
__device__ __forceinline__ float2 filter_vals_ks(const InvArgs& a, float dc, const BinTables& tb, size_t gi,
                                                 const float2 (&sv)[4], const KState& ks) {
  float d_re = 0.0f, d_im = 0.0f;
  if (a.dg) {
    const float2 g = tb.gs;
    d_re = dc * g.x;
    d_im = dc * g.y;
  }
  float sx = a.sigma_x, sy = a.sigma_y;
  if (a.pat) {
    const float pv = tb.pat;
    sx = pv * a.beta;
    sy = pv;
  }
  float fr, fi;
  const int bm = BM == kRuntimeBm ? a.bm : BM;
  if (bm == 2) {
    const float2 p = sv[0], c = sv[1];
    float ar = c.x - p.x, ai = c.y - p.y;
    float br = c.x + p.x, bi = c.y + p.y;
    if (a.dg) {
      br -= 2.0f * d_re;
      bi -= 2.0f * d_im;
    }
    if (FAST) {
      const float s = 0.5f, ssy = s * sy, sbx = s * a.beta_x;
      const float ga = wiener_gain_scaled(ar, ai, ssy, s, sbx), gb = wiener_gain_scaled(br, bi, ssy, s, sbx);
      fr = fmaf(gb, br, ga * ar);
      fi = fmaf(gb, bi, ga * ai);
    } else {
      wienner(ar, ai, sx, sy, a.beta_x);
      wienner(br, bi, sx, sy, a.beta_x);
      fr = (ar + br) * 0.5f;
      fi = (ai + bi) * 0.5f;
    }
    if (a.dg) {
      fr += d_re;
      fi += d_im;
    }
  } else if (bm == 3) {
    const float2 p = sv[0], c = sv[1], n = sv[2];
    const float K = 0.8660254f;  // truncated literal, src/cpu/reference.cpp:247
    float t1r = p.x + n.x, t1i = p.y + n.y;
    float y1r = c.x - 0.5f * t1r, y1i = c.y - 0.5f * t1i;
    float dnr = n.x - p.x, dni = n.y - p.y;
    float y2r = K * dni, y2i = -K * dnr;
    float d0r = y1r + y2r, d0i = y1i + y2i;
    float d1r = c.x + t1r, d1i = c.y + t1i;
    float d2r = y1r - y2r, d2i = y1i - y2i;
    if (a.dg) {
      d1r -= 3.0f * d_re;
      d1i -= 3.0f * d_im;
    }
    if (FAST) {
      const float s = 1.0f / 3.0f, ssy = s * sy, sbx = s * a.beta_x;
      const float g0 = wiener_gain_scaled(d0r, d0i, ssy, s, sbx), g1 = wiener_gain_scaled(d1r, d1i, ssy, s, sbx);
      const float g2 = wiener_gain_scaled(d2r, d2i, ssy, s, sbx);
      fr = fmaf(g2, d2r, fmaf(g1, d1r, g0 * d0r));
      fi = fmaf(g2, d2i, fmaf(g1, d1i, g0 * d0i));
    } else {
      wienner(d0r, d0i, sx, sy, a.beta_x);
      wienner(d1r, d1i, sx, sy, a.beta_x);
      wienner(d2r, d2i, sx, sy, a.beta_x);
      fr = (d0r + d1r + d2r) * (1.0f / 3.0f);
      fi = (d0i + d1i + d2i) * (1.0f / 3.0f);
    }
    if (a.dg) {
      fr += d_re;
      fi += d_im;
    }
  } else if (bm == 4) {
    const float2 p2 = sv[0], p1 = sv[1], c = sv[2], n = sv[3];
    float fp1r, fp1i, fcr, fci, fnr, fni, fp2r, fp2i;
    if (FAST) {  // radix 2 x 2: (c +- p2), (p1 +- n), on (re, im) pairs
#if __CUDA_ARCH__ >= 1000
      // Packed fp32x2 adds; a - b as b * -1 + a, one rounding like the
      // scalar subtraction, so the values equal the scalar form's.
      const float2 m1 = make_float2(-1.0f, -1.0f);
      const float2 s2 = __fadd2_rn(c, p2), d2 = __ffma2_rn(p2, m1, c);
      const float2 t2 = __fadd2_rn(p1, n), e2 = __ffma2_rn(n, m1, p1);
      const float2 fc2 = __fadd2_rn(s2, t2), fp22 = __ffma2_rn(t2, m1, s2);
      const float2 es = make_float2(e2.y, e2.x);
      const float2 fp12 = __ffma2_rn(es, make_float2(1.0f, -1.0f), d2);
      const float2 fn2 = __ffma2_rn(es, make_float2(-1.0f, 1.0f), d2);
      fcr = fc2.x, fci = fc2.y, fp2r = fp22.x, fp2i = fp22.y;
      fp1r = fp12.x, fp1i = fp12.y, fnr = fn2.x, fni = fn2.y;
#else
      const float sr = c.x + p2.x, si = c.y + p2.y, dr = c.x - p2.x, di = c.y - p2.y;
      const float tr = p1.x + n.x, ti = p1.y + n.y, er = p1.x - n.x, ei = p1.y - n.y;
      fcr = sr + tr, fci = si + ti, fp2r = sr - tr, fp2i = si - ti;
      fp1r = dr + ei, fp1i = di - er, fnr = dr - ei, fni = di + er;
#endif
    } else {
      fp1r = -p2.x + p1.y + c.x - n.y;
      fp1i = -p2.y - p1.x + c.y + n.x;
      fcr = p2.x + p1.x + c.x + n.x;
      fci = p2.y + p1.y + c.y + n.y;
      fnr = -p2.x - p1.y + c.x + n.y;
      fni = -p2.y + p1.x + c.y - n.x;
      fp2r = p2.x - p1.x + c.x - n.x;
      fp2i = p2.y - p1.y + c.y - n.y;
    }
    if (a.dg) {
      fp1r -= 4.0f * d_re;
      fp1i -= 4.0f * d_im;
    }
    if (FAST) {
      const float s = 0.25f, ssy = s * sy, sbx = s * a.beta_x;
      const float g2 = wiener_gain_scaled(fp2r, fp2i, ssy, s, sbx), g1 = wiener_gain_scaled(fp1r, fp1i, ssy, s, sbx);
      const float gc = wiener_gain_scaled(fcr, fci, ssy, s, sbx), gn = wiener_gain_scaled(fnr, fni, ssy, s, sbx);
      fr = fmaf(gn, fnr, fmaf(gc, fcr, fmaf(g1, fp1r, g2 * fp2r)));
      fi = fmaf(gn, fni, fmaf(gc, fci, fmaf(g1, fp1i, g2 * fp2i)));
    } else {
      wienner(fp2r, fp2i, sx, sy, a.beta_x);
      wienner(fp1r, fp1i, sx, sy, a.beta_x);
      wienner(fcr, fci, sx, sy, a.beta_x);
      wienner(fnr, fni, sx, sy, a.beta_x);
      fr = (fp2r + fp1r + fcr + fnr) * 0.25f;
      fi = (fp2i + fp1i + fci + fni) * 0.25f;
    }
    if (a.dg) {
      fr += d_re;
      fi += d_im;
    }
  } else if (bm == 1) {
    const float2 c = sv[0];
    float re = c.x, im = c.y;
    if (a.dg) {
      re -= d_re;
      im -= d_im;
    }
    wienner_t<FAST>(re, im, sx, sy, a.beta_x);
    if (a.dg) {
      re += d_re;
      im += d_im;
    }
    fr = re;
    fi = im;
  } else if (bm == 0) {
    const float2 c = sv[0];
    const float cn = a.pat ? tb.pat : a.kalman_cn;
    float2 l;
    float s;
    if (a.kalman_init) {  // src/cpu/reference.cpp:336-355: last = current, covar = proc = cn
      l = c;
      s = cn + cn;
    } else {
      l = ks.last;
      s = ks.cov + ks.proc;
    }
    float dr = c.x - l.x, di = c.y - l.y;
    float a2 = dr * dr, b2 = di * di;
    float mask = a2 < b2 ? b2 : a2;  // std::max
    float gain = s / (s + cn);
    float new_proc = gain * gain * cn;
    float new_covar = (1.0f - gain) * s;
    float dst_r = gain * c.x + (1.0f - gain) * l.x;
    float dst_i = gain * c.y + (1.0f - gain) * l.y;
    if (mask > a.kr2 * cn) {
      dst_r = c.x;
      dst_i = c.y;
      new_covar = cn;
      new_proc = cn;
    }
    a.kcov[gi] = new_covar;
    a.kproc[gi] = new_proc;
    a.klast[gi] = make_float2(dst_r, dst_i);
    fr = dst_r;
    fi = dst_i;
  } else {
    const float2 c = sv[0];
    fr = c.x;
    fi = c.y;
  }
  if (a.shp) {  // src/cpu/reference.cpp:393-409
    float re = fr, im = fi;
    if (a.dg) {
      re -= d_re;
      im -= d_im;
    }
    float psd = re * re + im * im + 0.0000000000000000000000000000000000001f;
    float factor = tb.shp;
    float g = 1.0f + factor * sqrtf(psd * a.ssmax / ((psd + a.ssmin) * (psd + a.ssmax)));
    re *= g;
    im *= g;
    if (a.dg) {
      re += d_re;
      im += d_im;
    }
    fr = re;
    fi = im;
  }
  return make_float2(fr, fi);
}

// filter_vals_ks with the Kalman state read here.
template <int BM, bool FAST = false>
__device__ __forceinline__ float2 filter_vals_t(const InvArgs& a, float dc, const BinTables& tb, size_t gi,
                                                const float2 (&sv)[4]) {
  const int bm = BM == kRuntimeBm ? a.bm : BM;
  KState ks{make_float2(0.0f, 0.0f), 0.0f, 0.0f};
  if (bm == 0) ks = load_kstate(a, gi);
  return filter_vals_ks<BM, FAST>(a, dc, tb, gi, sv, ks);
}

template <int BM, bool FAST = false>
__device__ __forceinline__ float2 filter_vals(const InvArgs& a, float dc, int i, size_t gi, const float2 (&sv)[4]) {
  return filter_vals_t<BM, FAST>(a, dc, bin_tables(a, i), gi, sv);
}

// The window's spectra of bin gi, in temporal order (frames the mode reads).
template <int BM>
__device__ __forceinline__ void load_window(const InvArgs& a, size_t gi, float2 (&sv)[4]) {
  const int bm = BM == kRuntimeBm ? a.bm : BM;
  const int nf = bm >= 2 ? bm : 1;
#pragma unroll
  for (int k = 0; k < 4; k++)
    if (k < nf) sv[k] = a.s[k][gi];
}

template <int BM, bool FAST = false>
__device__ __forceinline__ float2 filter_bin_t(const InvArgs& a, float dc, int i, size_t gi) {
  float2 sv[4];
  load_window<BM>(a, gi, sv);
  return filter_vals<BM, FAST>(a, dc, i, gi, sv);
}

__device__ __forceinline__ float2 filter_bin(const InvArgs& a, int b, int i, size_t gi) {
  return filter_bin_t<kRuntimeBm>(a, block_dc(a, b), i, gi);
}

// One radix-2 DIT stage of length LEN over N register values: butterflies
// (u + w*b, u - w*b) with twiddle tw[j * N/LEN], conjugated for the inverse.
// The j = 0 twiddle is (1, -0) and its product equals b, so it is skipped.
// Stages recurse at compile time so that every loop bound is a constant and
// the array stays in registers.
template <int N, int LEN, bool INV>
__device__ __forceinline__ void fft_r2_stage(float2 (&a)[N], const float2* tw) {
  constexpr int half = LEN / 2, step = N / LEN;
#pragma unroll
  for (int i = 0; i < N; i += LEN) {
#pragma unroll
    for (int j = 0; j < half; j++) {
      const float2 b = a[i + j + half];
      float2 t;
      if (j == 0) {
        t = b;
      } else {
        const float2 w = tw[j * step];
        const float wy = INV ? -w.y : w.y;
        t.x = w.x * b.x - wy * b.y;
        t.y = w.x * b.y + wy * b.x;
      }
      const float2 u = a[i + j];
      a[i + j] = make_float2(u.x + t.x, u.y + t.y);
      a[i + j + half] = make_float2(u.x - t.x, u.y - t.y);
    }
  }
  if constexpr (LEN < N) fft_r2_stage<N, LEN * 2, INV>(a, tw);
}

// Radix-2 decimation-in-time transform of N values held in registers, in the
// operation order of the reference's FftPlan (src/cpu/fft.cpp:28-58): bit
// reversal, stages len = 2..N, and for the inverse a final scale by 1/N.
template <int N, bool INV>
__device__ __forceinline__ void fft_r2(float2 (&a)[N], const float2* tw) {
  constexpr int L = Log2<N>::v;
#pragma unroll
  for (int i = 0; i < N; i++) {
    const int r = bit_reverse(i, L);
    if (i < r) {
      const float2 t = a[i];
      a[i] = a[r];
      a[r] = t;
    }
  }
  fft_r2_stage<N, 2, INV>(a, tw);
  if (INV) {
    const float invn = 1.0f / N;
#pragma unroll
    for (int i = 0; i < N; i++) a[i] = make_float2(a[i].x * invn, a[i].y * invn);
  }
}

}  // namespace f3d
