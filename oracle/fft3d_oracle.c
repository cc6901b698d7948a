/*
 * fft3d_oracle.c -- CPU oracle for the FFT3D block-FFT denoise path.
 *
 * TEST INFRASTRUCTURE ONLY: the oracle the CUDA engine is compared with, never
 * part of the product. A C99 restatement of the fp32 CPU backend of HumbleUser33/FFT3dCL;
 * every function names the reference file:line it follows. Build with
 * -ffp-contract=off (oracle/Makefile) so that no multiply-add is fused: the
 * reference is specified with MSVC /fp:precise (CMakeLists.txt:19-25).
 */
#include "fft3d_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

typedef struct {
  float re, im;
} cpx;

/* std::complex<float> multiply as libstdc++ evaluates it: (a+bi)(c+di) =
 * (ac - bd) + (ad + bc)i. */
static inline cpx cmul(cpx w, cpx t) {
  cpx r;
  r.re = w.re * t.re - w.im * t.im;
  r.im = w.re * t.im + w.im * t.re;
  return r;
}

/* ---------------------------------------------------------------- params -- */

/* src/params.h:62-72: round down to a power of two, clamp to [4, 512]. The
 * doubling is done in unsigned arithmetic; for v <= 0 the reference's loop
 * overflows to 0 and the clamp gives 4, which is what this returns too. */
int orc_round_pow2_clamp(int v) {
  unsigned int logn = 0;
  for (unsigned int i = (unsigned int)(v - 1); i > 0; i /= 2, logn++)
    ;
  unsigned int r = 1;
  for (unsigned int i = 1; i <= logn; i++)
    r *= 2u;
  if ((int)r < 4) r = 4; /* r wraps to 0 when logn == 32 */
  if (r > 512u) r = 512u;
  return (int)r;
}

/* src/params.h:76-148. */
int orc_validate_params(const orc_script_params* sp, int width, int height, int bits,
                        orc_internal_params* out, const char** err) {
  memset(out, 0, sizeof(*out));
  out->sigma = sp->sigma / 255.0f;
  out->beta = sp->beta;
  out->bm = sp->bt;
  if (out->bm < -1 || out->bm > 4) {
    *err = "FFT3DCL: valid modes for bt are -1,0,1,2,3,4";
    return 0;
  }
  out->bt = sp->bt > 0 ? sp->bt : 1;
  out->sharpen = sp->sharpen;
  out->sharpen_on = sp->sharpen != 0.0f;
  out->mode = (sp->mode < 0 || sp->mode > 2) ? 0 : sp->mode;
  out->bordersize = sp->bordersize;
  out->degrid = sp->degrid;
  out->degrid_on = sp->degrid != 0.0f;
  out->scutoff = sp->scutoff;
  out->svr = sp->svr;
  out->smin = sp->smin / 255.0f;
  out->smax = sp->smax / 255.0f;
  out->kratio = sp->kratio;
  out->wintype = (sp->wintype < 0 || sp->wintype > 2) ? 0 : sp->wintype;
  out->interlaced = sp->interlaced;
  out->sigma2 = sp->sigma2;
  out->sigma3 = sp->sigma3;
  out->sigma4 = sp->sigma4;
  out->use_pattern = (sp->sigma != sp->sigma2 || sp->sigma3 != sp->sigma4 || sp->sigma != sp->sigma3);
  out->oldfft = sp->oldfft;
  out->current = (out->bm == 1) ? 0 : (out->bm == 4) ? 2 : 1;

  out->bw = orc_round_pow2_clamp(sp->bw);
  out->bh = orc_round_pow2_clamp(sp->bh);
  out->ow = (int)(sp->ow * (float)out->bw / (float)sp->bw);
  out->ow &= (int)0xFFFFFFFE;
  out->oh = (int)(sp->oh * (float)out->bh / (float)sp->bh);
  if (out->oh * 2 > out->bh) out->oh = out->bh / 2;
  if (out->ow * 2 > out->bw) out->ow = out->bw / 2;

  int precision = sp->precision;
  if (bits > 8) precision = 2;
  if (precision < 0 || precision > 2) precision = 1;
  out->precision = precision;

  if (out->mode == 2) {
    *err = "FFT3DCL: mode 2 is not implemented yet in this port (use mode 0 or 1)";
    return 0;
  }
  if (out->interlaced) {
    *err = "FFT3DCL: interlaced is not implemented yet in this port";
    return 0;
  }
  if (out->mode == 0 || (out->bw == out->ow * 2 && out->bh == out->oh * 2)) {
    out->ny = (int)((height + out->bh * 1.5 - 1) / out->bh);
    out->nx = (int)((width + out->bw * 1.5 - 1) / out->bw);
  } else {
    out->nx = ((width + out->ow - 1) / (out->bw - out->ow) + 1 + 1) / 2;
    out->ny = ((height + out->oh - 1) / (out->bh - out->oh) + 1 + 1) / 2;
  }
  out->totw = out->nx * out->bw;
  out->toth = out->ny * out->bh;

  out->wiener_s = out->sigma * out->sigma * out->bt * out->bw * out->bh;
  out->beta_x = (out->beta - 1.0f) / out->beta;
  out->kalman_cn = out->sigma * out->sigma * out->bw * out->bh;
  out->ssmin = out->smin * out->smin * out->bw * out->bh * out->bt;
  out->ssmax = out->smax * out->smax * out->bw * out->bh * out->bt;
  return 1;
}

/* ------------------------------------------------------------------- fft -- */

typedef struct {
  int n;
  cpx* tw;  /* exp(-2*pi*i*k/n), k < n/2, double -> float */
  int* rev; /* bit reversal */
} fft_plan;

/* src/cpu/fft.cpp:8-25. */
static void plan_init(fft_plan* p, int n) {
  p->n = n;
  p->tw = (cpx*)malloc(sizeof(cpx) * (size_t)(n / 2 > 0 ? n / 2 : 1));
  for (int k = 0; k < n / 2; k++) {
    double a = -2.0 * 3.14159265358979323846 * k / n;
    p->tw[k].re = (float)cos(a);
    p->tw[k].im = (float)sin(a);
  }
  p->rev = (int*)malloc(sizeof(int) * (size_t)n);
  int bits = 0;
  while ((1 << bits) < n) bits++;
  for (int i = 0; i < n; i++) {
    int r = 0;
    for (int b = 0; b < bits; b++)
      if (i & (1 << b)) r |= 1 << (bits - 1 - b);
    p->rev[i] = r;
  }
}

static void plan_free(fft_plan* p) {
  free(p->tw);
  free(p->rev);
}

/* Radix-2 DIT with bit reversal, inverse scaled by 1/n (src/cpu/fft.cpp:28-58).
 * a is scratch of n elements. */
static void transform(const fft_plan* p, const cpx* in, cpx* out, int inverse, cpx* a) {
  const int n = p->n;
  for (int i = 0; i < n; i++) a[i] = in[p->rev[i]];
  for (int len = 2; len <= n; len <<= 1) {
    const int half = len >> 1;
    const int step = n / len;
    for (int i = 0; i < n; i += len)
      for (int j = 0; j < half; j++) {
        cpx w = p->tw[j * step];
        if (inverse) w.im = -w.im;
        cpx t = cmul(w, a[i + j + half]);
        cpx u = a[i + j];
        a[i + j].re = u.re + t.re;
        a[i + j].im = u.im + t.im;
        a[i + j + half].re = u.re - t.re;
        a[i + j + half].im = u.im - t.im;
      }
  }
  if (inverse) {
    const float invn = 1.0f / n;
    for (int i = 0; i < n; i++) {
      out[i].re = a[i].re * invn;
      out[i].im = a[i].im * invn;
    }
  } else {
    for (int i = 0; i < n; i++) out[i] = a[i];
  }
}

typedef struct {
  cpx *row, *col, *colout, *a, *full;
} fft_scratch;

static void scratch_init(fft_scratch* s, int bw, int bh) {
  int m = bw > bh ? bw : bh;
  s->row = (cpx*)malloc(sizeof(cpx) * (size_t)m);
  s->col = (cpx*)malloc(sizeof(cpx) * (size_t)m);
  s->colout = (cpx*)malloc(sizeof(cpx) * (size_t)m);
  s->a = (cpx*)malloc(sizeof(cpx) * (size_t)m);
  s->full = (cpx*)malloc(sizeof(cpx) * (size_t)bw * bh);
}

static void scratch_free(fft_scratch* s) {
  free(s->row);
  free(s->col);
  free(s->colout);
  free(s->a);
  free(s->full);
}

/* src/cpu/fft.cpp:68-86. Only columns 0..ncols-1 are transformed: the column
 * transforms are independent, so the kept columns are bit-identical to those
 * of a full transform. */
static void fft2d_forward(const float* block, int bw, int bh, const fft_plan* rp,
                          const fft_plan* cp, cpx* full, int ncols, fft_scratch* s) {
  for (int r = 0; r < bh; r++) {
    for (int c = 0; c < bw; c++) {
      s->row[c].re = block[r * bw + c];
      s->row[c].im = 0.0f;
    }
    transform(rp, s->row, full + r * bw, 0, s->a);
  }
  for (int c = 0; c < ncols; c++) {
    for (int r = 0; r < bh; r++) s->col[r] = full[r * bw + c];
    transform(cp, s->col, s->colout, 0, s->a);
    for (int r = 0; r < bh; r++) full[r * bw + c] = s->colout[r];
  }
}

/* src/cpu/fft.cpp:88-119: Hermitian completion, column then row inverse,
 * real part. */
static void fft2d_inverse_half(const cpx* half, int bw, int bh, int fbw, const fft_plan* rp,
                               const fft_plan* cp, float* block, fft_scratch* s) {
  cpx* full = s->full;
  for (int r = 0; r < bh; r++)
    for (int c = 0; c < fbw; c++) full[r * bw + c] = half[r * fbw + c];
  for (int r = 0; r < bh; r++) {
    int rm = (bh - r) % bh;
    for (int c = fbw; c < bw; c++) {
      int cm = bw - c;
      full[r * bw + c].re = full[rm * bw + cm].re;
      full[r * bw + c].im = -full[rm * bw + cm].im;
    }
  }
  for (int c = 0; c < bw; c++) {
    for (int r = 0; r < bh; r++) s->col[r] = full[r * bw + c];
    transform(cp, s->col, s->colout, 1, s->a);
    for (int r = 0; r < bh; r++) full[r * bw + c] = s->colout[r];
  }
  for (int r = 0; r < bh; r++) {
    transform(rp, full + r * bw, s->row, 1, s->a);
    for (int c = 0; c < bw; c++) block[r * bw + c] = s->row[c].re;
  }
}

void orc_fft1d(int n, const float* in, float* out, int inverse) {
  fft_plan p;
  plan_init(&p, n);
  cpx* a = (cpx*)malloc(sizeof(cpx) * (size_t)n);
  transform(&p, (const cpx*)in, (cpx*)out, inverse, a);
  free(a);
  plan_free(&p);
}

void orc_fft2d_forward(const float* block, int bw, int bh, float* full) {
  fft_plan rp, cp;
  fft_scratch s;
  plan_init(&rp, bw);
  plan_init(&cp, bh);
  scratch_init(&s, bw, bh);
  fft2d_forward(block, bw, bh, &rp, &cp, (cpx*)full, bw, &s);
  scratch_free(&s);
  plan_free(&rp);
  plan_free(&cp);
}

void orc_fft2d_inverse_half(const float* half, int bw, int bh, float* block) {
  fft_plan rp, cp;
  fft_scratch s;
  plan_init(&rp, bw);
  plan_init(&cp, bh);
  scratch_init(&s, bw, bh);
  fft2d_inverse_half((const cpx*)half, bw, bh, bw / 2 + 1, &rp, &cp, block, &s);
  scratch_free(&s);
  plan_free(&rp);
  plan_free(&cp);
}

/* ---------------------------------------------------------------- tables -- */

static const double kPi = 3.14159265358979323846;

/* src/cpu/tables.cpp:8-19. */
static void build_window_mode0(int bw, int bh, float* w) {
  int off = 0;
  for (double n1 = -bh / 2.0 + 0.5; n1 < bh / 2.0; n1++) {
    double cosy = cos(n1 * kPi / bh);
    for (double n2 = -bw / 2.0 + 0.5; n2 < bw / 2.0; n2++) {
      double cosx = cos(n2 * kPi / bw);
      w[off++] = (float)sqrt(0.5 * (cosx * cosx + cosy * cosy));
    }
  }
}

/* src/cpu/tables.cpp:21-105. */
static void build_windows_mode1(int bw, int bh, int ow, int oh, int wintype, float* A,
                                float* SynA, float* SynB) {
  double* wanx = (double*)calloc((size_t)(ow > 0 ? ow : 1), sizeof(double));
  double* wsynx = (double*)calloc((size_t)(ow > 0 ? ow : 1), sizeof(double));
  double* wany = (double*)calloc((size_t)(oh > 0 ? oh : 1), sizeof(double));
  double* wsyny = (double*)calloc((size_t)(oh > 0 ? oh : 1), sizeof(double));
  switch (wintype) {
  case 1:
    for (int i = 0; i < ow; i++) {
      wanx[i] = sqrt(cos(kPi * (i - ow + 0.5) / (ow * 2.0)));
      wsynx[i] = wanx[i] * wanx[i] * wanx[i];
    }
    for (int i = 0; i < oh; i++) {
      wany[i] = sqrt(cos(kPi * (i - oh + 0.5) / (oh * 2.0)));
      wsyny[i] = wany[i] * wany[i] * wany[i];
    }
    break;
  case 2:
    for (int i = 0; i < ow; i++) {
      wanx[i] = 1.0;
      wsynx[i] = cos(kPi * (i - ow + 0.5) / (ow * 2.0));
      wsynx[i] *= wsynx[i];
    }
    for (int i = 0; i < oh; i++) {
      wany[i] = 1.0;
      wsyny[i] = cos(kPi * (i - oh + 0.5) / (oh * 2.0));
      wsyny[i] *= wsyny[i];
    }
    break;
  default:
    for (int i = 0; i < ow; i++) {
      wanx[i] = cos(kPi * (i - ow + 0.5) / (ow * 2.0));
      wsynx[i] = wanx[i];
    }
    for (int i = 0; i < oh; i++) {
      wany[i] = cos(kPi * (i - oh + 0.5) / (oh * 2.0));
      wsyny[i] = wany[i];
    }
    break;
  }
  double* wxA = (double*)calloc((size_t)bw, sizeof(double));
  double* wxSA = (double*)calloc((size_t)bw, sizeof(double));
  double* wxSB = (double*)calloc((size_t)bw, sizeof(double));
  double* wyA = (double*)calloc((size_t)bh, sizeof(double));
  double* wySA = (double*)calloc((size_t)bh, sizeof(double));
  for (int lx = 0; lx < ow; lx++) {
    wxA[lx] = wanx[lx];
    wxSA[lx] = wsynx[lx];
    wxSB[lx] = wsynx[(ow - 1) - lx];
  }
  for (int lx = ow; lx < bw - ow; lx++) {
    wxA[lx] = 1.0;
    wxSA[lx] = 1.0;
    wxSB[lx] = 1.0;
  }
  for (int lx = bw - ow; lx < bw; lx++) {
    int x = lx - (bw - ow);
    wxA[lx] = wanx[(ow - 1) - x];
    wxSA[lx] = wsynx[(ow - 1) - x];
    wxSB[lx] = wsynx[x];
  }
  for (int ly = 0; ly < oh; ly++) {
    wyA[ly] = wany[ly];
    wySA[ly] = wsyny[ly];
  }
  for (int ly = oh; ly < bh - oh; ly++) {
    wyA[ly] = 1.0;
    wySA[ly] = 1.0;
  }
  for (int ly = bh - oh; ly < bh; ly++) {
    wyA[ly] = wany[bh - 1 - ly];
    wySA[ly] = wsyny[bh - 1 - ly];
  }
  for (int ly = 0; ly < bh; ly++)
    for (int lx = 0; lx < bw; lx++) {
      A[ly * bw + lx] = (float)(wxA[lx] * wyA[ly]);
      SynA[ly * bw + lx] = (float)(wxSA[lx] * wySA[ly]);
      SynB[ly * bw + lx] = (float)(wxSB[lx] * wySA[ly]);
    }
  free(wanx);
  free(wsynx);
  free(wany);
  free(wsyny);
  free(wxA);
  free(wxSA);
  free(wxSB);
  free(wyA);
  free(wySA);
}

static float pattern_scale(float s, int bt, int bw, int bh) {
  double v = s / 255.0;
  return (float)(v * v * bt * bw * bh);
}

/* src/cpu/tables.cpp:107-137. */
static void build_pattern(int bw, int bh, int bt, float sigma, float sigma2, float sigma3,
                          float sigma4, float* pat) {
  const int fbw = bw / 2 + 1;
  float s = pattern_scale(sigma, bt, bw, bh), s2 = pattern_scale(sigma2, bt, bw, bh);
  float s3 = pattern_scale(sigma3, bt, bw, bh), s4 = pattern_scale(sigma4, bt, bw, bh);
  float ft2 = (float)(sqrt(0.5) / 2.0);
  float ft3 = (float)(sqrt(0.5) / 4.0);
  for (int h = 0; h < bh; h++) {
    float fy = (bh - 2.0f * fabsf(h - bh / 2.0f)) / bh;
    for (int w = 0; w < fbw; w++) {
      float fx = w * 1.0f / fbw;
      float f = sqrtf((fx * fx + fy * fy) * 0.5f);
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

/* src/cpu/tables.cpp:139-156. */
static void build_sharpen_lut(int bw, int bh, float strength, float svr, float scutoff,
                              float* lut) {
  const int fbw = bw / 2 + 1;
  for (int j = 0; j < bh; j++) {
    int dj = j;
    if (j >= bh / 2) dj = bh - j;
    float d2v = (float)(dj * dj) * (svr * svr) / ((bh / 2.0f) * (bh / 2.0f));
    for (int i = 0; i < fbw; i++) {
      float d2 = d2v + (float)(i * i) / ((bw / 2.0f) * (bw / 2.0f));
      lut[j * fbw + i] = strength * (1.0f - expf(-d2 / (2.0f * scutoff * scutoff)));
    }
  }
}

/* ----------------------------------------------------------------- plane -- */

struct orc_plane {
  orc_internal_params p;
  int width, height, bits, sample_type, chroma;
  int fbw, nb, ncols;
  int *bx, *by;
  uint8_t* par;
  float *win_ana, *win_syn_a, *win_syn_b; /* syn tables NULL in mode 0 */
  float *pattern, *sharpen;               /* NULL when off */
  float *gs_re, *gs_im;                   /* fbw*bh, NULL until built */
  float chroma_norm;
  fft_plan row_plan, col_plan;
  /* filter state */
  float *filt_re, *filt_im, *corr_re, *corr_im, *blk; /* sized on first use */
  float *k_last_re, *k_last_im, *k_covar, *k_proc;     /* Kalman */
  int kalman_first;
  /* overlap-add: per output row, the covering blocks in ascending order */
  int *row_start, *row_list;
};

/* src/cpu/reference.cpp:10-17: D3D9 MIRROR addressing. */
static inline int mirror_i(int x, int w) {
  int p = x % (2 * w);
  if (p < 0) p += 2 * w;
  if (p >= w) p = 2 * w - 1 - p;
  return p;
}

/* src/cpu/reference.cpp:19-80. */
orc_plane* orc_plane_new(const orc_internal_params* p, int width, int height, int bits,
                         int sample_type, int chroma) {
  orc_plane* pl = (orc_plane*)calloc(1, sizeof(orc_plane));
  pl->p = *p;
  pl->width = width;
  pl->height = height;
  pl->bits = bits;
  pl->sample_type = sample_type;
  pl->chroma = chroma;
  const int bw = p->bw, bh = p->bh;
  pl->fbw = bw / 2 + 1;
  plan_init(&pl->row_plan, bw);
  plan_init(&pl->col_plan, bh);

  pl->win_ana = (float*)malloc(sizeof(float) * (size_t)bw * bh);
  if (p->mode == 0) {
    pl->nb = 2 * p->nx * p->ny;
    pl->bx = (int*)malloc(sizeof(int) * (size_t)pl->nb);
    pl->by = (int*)malloc(sizeof(int) * (size_t)pl->nb);
    pl->par = (uint8_t*)malloc((size_t)pl->nb);
    int k = 0;
    for (int grid = 0; grid < 2; grid++)
      for (int j = 0; j < p->ny; j++)
        for (int i = 0; i < p->nx; i++) {
          int off = grid ? -bw / 2 : 0, offy = grid ? -bh / 2 : 0;
          pl->bx[k] = i * bw + off;
          pl->by[k] = j * bh + offy;
          pl->par[k] = 0;
          k++;
        }
    build_window_mode0(bw, bh, pl->win_ana);
    pl->ncols = 0;
  } else {
    int ncols = 2 * p->nx, nrows = 2 * p->ny;
    pl->ncols = ncols;
    pl->nb = ncols * nrows;
    pl->bx = (int*)malloc(sizeof(int) * (size_t)pl->nb);
    pl->by = (int*)malloc(sizeof(int) * (size_t)pl->nb);
    pl->par = (uint8_t*)malloc((size_t)pl->nb);
    int ystep = bh - p->oh, k = 0;
    for (int m = 0; m < nrows; m++)
      for (int n = 0; n < ncols; n++) {
        pl->bx[k] = -p->ow + n * (bw - p->ow);
        pl->by[k] = -p->oh + m * ystep;
        pl->par[k] = (uint8_t)(n & 1);
        k++;
      }
    float* synB = (float*)malloc(sizeof(float) * (size_t)bw * bh);
    pl->win_syn_a = (float*)malloc(sizeof(float) * (size_t)bw * bh);
    pl->win_syn_b = (float*)malloc(sizeof(float) * (size_t)bw * bh);
    build_windows_mode1(bw, bh, p->ow, p->oh, p->wintype, pl->win_ana, pl->win_syn_a, synB);
    /* reference.cpp:51-57: odd-parity synthesis window sampled (bw-ow) right */
    for (int ly = 0; ly < bh; ly++)
      for (int lx = 0; lx < bw; lx++)
        pl->win_syn_b[ly * bw + lx] = synB[ly * bw + ((lx + bw - p->ow) % bw)];
    free(synB);
  }
  const int ps = pl->fbw * bh;
  if (p->use_pattern) {
    pl->pattern = (float*)malloc(sizeof(float) * (size_t)ps);
    build_pattern(bw, bh, p->bt, p->sigma * 255.0f, p->sigma2, p->sigma3, p->sigma4, pl->pattern);
  }
  if (p->sharpen != 0.0f) {
    pl->sharpen = (float*)malloc(sizeof(float) * (size_t)ps);
    build_sharpen_lut(bw, bh, p->sharpen, p->svr, p->scutoff, pl->sharpen);
  }
  if (p->mode == 1 && chroma) {
    if (sample_type == 1)
      pl->chroma_norm = 0.0f;
    else if (bits <= 8)
      pl->chroma_norm = 128.0f / 255.0f;
    else
      pl->chroma_norm = 32768.0f / 65535.0f;
  }
  pl->kalman_first = 1;

  /* Overlap-add lists: rows [by, by+bh) of each block, ascending block index,
   * so a gather per output row adds the blocks in the reference's order
   * (reference.cpp:392-430 adds block b before block b+1 into every pixel). */
  pl->row_start = (int*)calloc((size_t)height + 1, sizeof(int));
  for (int b = 0; b < pl->nb; b++)
    for (int ly = 0; ly < bh; ly++) {
      int y = pl->by[b] + ly;
      if (y >= 0 && y < height) pl->row_start[y + 1]++;
    }
  for (int y = 0; y < height; y++) pl->row_start[y + 1] += pl->row_start[y];
  pl->row_list = (int*)malloc(sizeof(int) * (size_t)(pl->row_start[height] + 1));
  int* fill = (int*)malloc(sizeof(int) * (size_t)(height + 1));
  memcpy(fill, pl->row_start, sizeof(int) * (size_t)(height + 1));
  for (int b = 0; b < pl->nb; b++)
    for (int ly = 0; ly < bh; ly++) {
      int y = pl->by[b] + ly;
      if (y >= 0 && y < height) pl->row_list[fill[y]++] = b;
    }
  free(fill);
  return pl;
}

void orc_plane_free(orc_plane* pl) {
  if (!pl) return;
  plan_free(&pl->row_plan);
  plan_free(&pl->col_plan);
  free(pl->bx);
  free(pl->by);
  free(pl->par);
  free(pl->win_ana);
  free(pl->win_syn_a);
  free(pl->win_syn_b);
  free(pl->pattern);
  free(pl->sharpen);
  free(pl->gs_re);
  free(pl->gs_im);
  free(pl->filt_re);
  free(pl->filt_im);
  free(pl->corr_re);
  free(pl->corr_im);
  free(pl->blk);
  free(pl->k_last_re);
  free(pl->k_last_im);
  free(pl->k_covar);
  free(pl->k_proc);
  free(pl->row_start);
  free(pl->row_list);
  free(pl);
}

int orc_nblocks(const orc_plane* pl) { return pl->nb; }
int orc_fbw(const orc_plane* pl) { return pl->fbw; }
int orc_ncols(const orc_plane* pl) { return pl->ncols; }
float orc_chroma_norm(const orc_plane* pl) { return pl->chroma_norm; }

void orc_get_grid(const orc_plane* pl, int* bx, int* by, uint8_t* par) {
  if (bx) memcpy(bx, pl->bx, sizeof(int) * (size_t)pl->nb);
  if (by) memcpy(by, pl->by, sizeof(int) * (size_t)pl->nb);
  if (par) memcpy(par, pl->par, (size_t)pl->nb);
}

static int copy_tab(const float* src, int n, float* dst) {
  if (!src) return 0;
  if (dst) memcpy(dst, src, sizeof(float) * (size_t)n);
  return n;
}

int orc_get_table(orc_plane* pl, int which, float* dst) {
  const int bw = pl->p.bw, bh = pl->p.bh, ps = pl->fbw * bh;
  switch (which) {
  case ORC_TAB_WIN_ANA: return copy_tab(pl->win_ana, bw * bh, dst);
  case ORC_TAB_WIN_SYN_A: return copy_tab(pl->win_syn_a, bw * bh, dst);
  case ORC_TAB_WIN_SYN_B: return copy_tab(pl->win_syn_b, bw * bh, dst);
  case ORC_TAB_PATTERN: return copy_tab(pl->pattern, ps, dst);
  case ORC_TAB_SHARPEN: return copy_tab(pl->sharpen, ps, dst);
  case ORC_TAB_GS_RE: return copy_tab(pl->gs_re, ps, dst);
  case ORC_TAB_GS_IM: return copy_tab(pl->gs_im, ps, dst);
  case ORC_TAB_TWIDDLE_ROW: return copy_tab((const float*)pl->row_plan.tw, bw, dst);
  case ORC_TAB_TWIDDLE_COL: return copy_tab((const float*)pl->col_plan.tw, bh, dst);
  default: return -1;
  }
}

/* src/cpu/reference.cpp:82-105. */
void orc_upload(const orc_plane* pl, const uint8_t* src, ptrdiff_t pitch, float* dst) {
  const int W = pl->width, H = pl->height;
  if (pl->sample_type == 1) {
    for (int y = 0; y < H; y++) {
      const float* row = (const float*)(src + y * pitch);
      for (int x = 0; x < W; x++) dst[y * W + x] = row[x];
    }
  } else if (pl->bits <= 8) {
    for (int y = 0; y < H; y++) {
      const uint8_t* row = src + y * pitch;
      for (int x = 0; x < W; x++) dst[y * W + x] = row[x] * (1.0f / 255.0f);
    }
  } else {
    const float norm = (float)(1u << (16 - pl->bits)) / 65535.0f;
    for (int y = 0; y < H; y++) {
      const uint16_t* row = (const uint16_t*)(src + y * pitch);
      for (int x = 0; x < W; x++) dst[y * W + x] = row[x] * norm;
    }
  }
}

/* src/cpu/reference.cpp:107-138. The 16-bit path divides by 2^(16-bits)
 * before comparing with the maximum pixel value, so that comparison never
 * bites and the result is clamped to [0, 65535] only. */
void orc_download(const orc_plane* pl, const float* src, uint8_t* dst, ptrdiff_t pitch) {
  const int W = pl->width, H = pl->height;
  if (pl->sample_type == 1) {
    for (int y = 0; y < H; y++) {
      float* row = (float*)(dst + y * pitch);
      for (int x = 0; x < W; x++) row[x] = src[y * W + x];
    }
  } else if (pl->bits <= 8) {
    for (int y = 0; y < H; y++) {
      uint8_t* row = dst + y * pitch;
      for (int x = 0; x < W; x++) {
        float v = src[y * W + x];
        v = v < 0.0f ? 0.0f : (v > 1.0f ? 1.0f : v);
        row[x] = (uint8_t)(v * 255.0f + 0.5f);
      }
    }
  } else {
    const float inv_norm = 1.0f / (float)(1u << (16 - pl->bits));
    const float max_pix = (float)((1u << pl->bits) - 1);
    for (int y = 0; y < H; y++) {
      uint16_t* row = (uint16_t*)(dst + y * pitch);
      for (int x = 0; x < W; x++) {
        float v = src[y * W + x] * inv_norm;
        v = v < max_pix ? v : max_pix;
        v = v < 0.0f ? 0.0f : (v > 1.0f ? 1.0f : v);
        row[x] = (uint16_t)(v * 65535.0f + 0.5f);
      }
    }
  }
}

/* ------------------------------------------------------------- threading -- */

typedef void (*range_fn)(void* ctx, int lo, int hi, int tid);

typedef struct {
  range_fn fn;
  void* ctx;
  int lo, hi, tid;
} range_job;

static void* range_thread(void* arg) {
  range_job* j = (range_job*)arg;
  j->fn(j->ctx, j->lo, j->hi, j->tid);
  return NULL;
}

/* Static contiguous split of [0, n) over `threads` host threads. */
static void parallel_for(int n, int threads, range_fn fn, void* ctx) {
  if (threads <= 1 || n < 2) {
    fn(ctx, 0, n, 0);
    return;
  }
  if (threads > n) threads = n;
  pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * (size_t)threads);
  range_job* jobs = (range_job*)malloc(sizeof(range_job) * (size_t)threads);
  for (int t = 0; t < threads; t++) {
    jobs[t].fn = fn;
    jobs[t].ctx = ctx;
    jobs[t].lo = (int)((long long)n * t / threads);
    jobs[t].hi = (int)((long long)n * (t + 1) / threads);
    jobs[t].tid = t;
  }
  for (int t = 1; t < threads; t++) pthread_create(&th[t], NULL, range_thread, &jobs[t]);
  range_thread(&jobs[0]);
  for (int t = 1; t < threads; t++) pthread_join(th[t], NULL);
  free(th);
  free(jobs);
}

/* ------------------------------------------------------------ spectra ---- */

typedef struct {
  orc_plane* pl;
  const float* plane;
  float *re, *im;
} spectra_ctx;

/* src/cpu/reference.cpp:140-170, for blocks [lo, hi). */
static void spectra_range(void* vctx, int lo, int hi, int tid) {
  (void)tid;
  spectra_ctx* c = (spectra_ctx*)vctx;
  orc_plane* pl = c->pl;
  const int fbw = pl->fbw, bw = pl->p.bw, bh = pl->p.bh, W = pl->width, H = pl->height;
  const int center = pl->chroma_norm != 0.0f;
  float* block = (float*)malloc(sizeof(float) * (size_t)bw * bh);
  fft_scratch s;
  scratch_init(&s, bw, bh);
  for (int b = lo; b < hi; b++) {
    const int x0 = pl->bx[b], y0 = pl->by[b];
    for (int ly = 0; ly < bh; ly++) {
      const float* prow = &c->plane[mirror_i(y0 + ly, H) * W];
      const float* wrow = &pl->win_ana[ly * bw];
      float* brow = &block[ly * bw];
      for (int lx = 0; lx < bw; lx++) {
        float v = prow[mirror_i(x0 + lx, W)];
        if (center) v -= pl->chroma_norm;
        brow[lx] = v * wrow[lx];
      }
    }
    fft2d_forward(block, bw, bh, &pl->row_plan, &pl->col_plan, s.full, fbw, &s);
    float* dRe = &c->re[(size_t)b * fbw * bh];
    float* dIm = &c->im[(size_t)b * fbw * bh];
    for (int r = 0; r < bh; r++)
      for (int cc = 0; cc < fbw; cc++) {
        dRe[r * fbw + cc] = s.full[r * bw + cc].re;
        dIm[r * fbw + cc] = s.full[r * bw + cc].im;
      }
  }
  scratch_free(&s);
  free(block);
}

void orc_compute_spectra(orc_plane* pl, const float* plane, float* re, float* im, int threads) {
  spectra_ctx c = {pl, plane, re, im};
  parallel_for(pl->nb, threads, spectra_range, &c);
}

/* src/cpu/reference.cpp:172-198: FFT of the analysis window divided by its DC,
 * times degrid. Every block gets the same sample, so one fbw*bh table is kept. */
void orc_build_degrid(orc_plane* pl) {
  const int fbw = pl->fbw, bw = pl->p.bw, bh = pl->p.bh, ps = fbw * bh;
  fft_scratch s;
  scratch_init(&s, bw, bh);
  float* blk = (float*)malloc(sizeof(float) * (size_t)bw * bh);
  memcpy(blk, pl->win_ana, sizeof(float) * (size_t)bw * bh);
  fft2d_forward(blk, bw, bh, &pl->row_plan, &pl->col_plan, s.full, bw, &s);
  free(pl->gs_re);
  free(pl->gs_im);
  pl->gs_re = (float*)malloc(sizeof(float) * (size_t)ps);
  pl->gs_im = (float*)malloc(sizeof(float) * (size_t)ps);
  const float dc = s.full[0].re;
  for (int r = 0; r < bh; r++)
    for (int c = 0; c < fbw; c++) {
      cpx z = s.full[r * bw + c];
      pl->gs_re[r * fbw + c] = z.re / dc * pl->p.degrid;
      pl->gs_im[r * fbw + c] = z.im / dc * pl->p.degrid;
    }
  free(blk);
  scratch_free(&s);
}

/* ------------------------------------------------------- filter + synth -- */

/* src/cpu/reference.cpp:201-209 (fft3dgpu.hlsl Wienner). */
static inline void wienner(float* re, float* im, float sigmaX, float sigmaY, float betaX) {
  float psd = *re * *re + *im * *im + 0.0000000000000000000000000000000000001f;
  float psdInv = 1.0f / psd;
  float mulFac = betaX;
  if (1.0f / sigmaX > psdInv) mulFac = 1.0f - sigmaY * psdInv;
  *re *= mulFac;
  *im *= mulFac;
}

typedef struct {
  orc_plane* pl;
  const float* const* wr;
  const float* const* wi;
  float* out;
  int dg;
} filt_ctx;

/* Degrid correction = current DC x degrid sample (reference.cpp:229-239). */
static void corr_range(void* vctx, int lo, int hi, int tid) {
  (void)tid;
  filt_ctx* c = (filt_ctx*)vctx;
  orc_plane* pl = c->pl;
  const int ps = pl->fbw * pl->p.bh;
  const float* cur_re = c->wr[pl->p.bm >= 2 ? pl->p.current : 0];
  for (int b = lo; b < hi; b++) {
    const float dc = cur_re[(size_t)b * ps];
    for (int i = 0; i < ps; i++) {
      pl->corr_re[(size_t)b * ps + i] = dc * pl->gs_re[i];
      pl->corr_im[(size_t)b * ps + i] = dc * pl->gs_im[i];
    }
  }
}

/* Phase 1, temporal filter, for blocks [lo, hi) (reference.cpp:246-389). The
 * reference loops bins outside and blocks inside; every bin is independent,
 * so the loop order does not change any value. */
static void temporal_range(void* vctx, int lo, int hi, int tid) {
  (void)tid;
  filt_ctx* c = (filt_ctx*)vctx;
  orc_plane* pl = c->pl;
  const orc_internal_params* p = &pl->p;
  const int fbw = pl->fbw, bh = p->bh, ps = fbw * bh;
  const int dg = c->dg, pat = pl->pattern != NULL;
  const float sigmaX = p->beta * p->wiener_s;
  const float sigmaY = p->wiener_s;
  const float K = 0.8660254f; /* truncated literal, reference.cpp:247 */
  const float* const* wr = c->wr;
  const float* const* wi = c->wi;
  const int cur = p->bm >= 2 ? p->current : 0;
  const float kr2 = p->kratio * p->kratio;
  for (int b = lo; b < hi; b++) {
    for (int i0 = 0; i0 < ps; i0++) {
      const size_t idx = (size_t)b * ps + i0;
      float dRe = 0, dIm = 0;
      if (dg) {
        dRe = pl->corr_re[idx];
        dIm = pl->corr_im[idx];
      }
      float sX = sigmaX, sY = sigmaY;
      if (pat) {
        float pv = pl->pattern[i0];
        sX = pv * p->beta;
        sY = pv;
      }
      if (p->bm == 2) {
        float pRe = wr[0][idx], pIm = wi[0][idx];
        float cRe = wr[1][idx], cIm = wi[1][idx];
        float aRe = cRe - pRe, aIm = cIm - pIm;
        float bRe = cRe + pRe, bIm = cIm + pIm;
        if (dg) {
          bRe -= 2.0f * dRe;
          bIm -= 2.0f * dIm;
        }
        wienner(&aRe, &aIm, sX, sY, p->beta_x);
        wienner(&bRe, &bIm, sX, sY, p->beta_x);
        pl->filt_re[idx] = (aRe + bRe) * 0.5f + (dg ? dRe : 0.0f);
        pl->filt_im[idx] = (aIm + bIm) * 0.5f + (dg ? dIm : 0.0f);
      } else if (p->bm == 3) {
        float pRe = wr[0][idx], pIm = wi[0][idx];
        float cRe = wr[1][idx], cIm = wi[1][idx];
        float nRe = wr[2][idx], nIm = wi[2][idx];
        float t1Re = pRe + nRe, t1Im = pIm + nIm;
        float y1Re = cRe - 0.5f * t1Re, y1Im = cIm - 0.5f * t1Im;
        float dnRe = nRe - pRe, dnIm = nIm - pIm;
        float y2Re = K * dnIm, y2Im = -K * dnRe;
        float d0Re = y1Re + y2Re, d0Im = y1Im + y2Im;
        float d1Re = cRe + t1Re, d1Im = cIm + t1Im;
        float d2Re = y1Re - y2Re, d2Im = y1Im - y2Im;
        if (dg) {
          d1Re -= 3.0f * dRe;
          d1Im -= 3.0f * dIm;
        }
        wienner(&d0Re, &d0Im, sX, sY, p->beta_x);
        wienner(&d1Re, &d1Im, sX, sY, p->beta_x);
        wienner(&d2Re, &d2Im, sX, sY, p->beta_x);
        pl->filt_re[idx] = (d0Re + d1Re + d2Re) * (1.0f / 3.0f);
        pl->filt_im[idx] = (d0Im + d1Im + d2Im) * (1.0f / 3.0f);
        if (dg) {
          pl->filt_re[idx] += dRe;
          pl->filt_im[idx] += dIm;
        }
      } else if (p->bm == 4) {
        float p2Re = wr[0][idx], p2Im = wi[0][idx];
        float p1Re = wr[1][idx], p1Im = wi[1][idx];
        float cRe = wr[2][idx], cIm = wi[2][idx];
        float nRe = wr[3][idx], nIm = wi[3][idx];
        float fp1r = -p2Re + p1Im + cRe - nIm;
        float fp1i = -p2Im - p1Re + cIm + nRe;
        float fcr = p2Re + p1Re + cRe + nRe;
        float fci = p2Im + p1Im + cIm + nIm;
        float fnr = -p2Re - p1Im + cRe + nIm;
        float fni = -p2Im + p1Re + cIm - nRe;
        float fp2r = p2Re - p1Re + cRe - nRe;
        float fp2i = p2Im - p1Im + cIm - nIm;
        if (dg) {
          fp1r -= 4.0f * dRe;
          fp1i -= 4.0f * dIm;
        }
        wienner(&fp2r, &fp2i, sX, sY, p->beta_x);
        wienner(&fp1r, &fp1i, sX, sY, p->beta_x);
        wienner(&fcr, &fci, sX, sY, p->beta_x);
        wienner(&fnr, &fni, sX, sY, p->beta_x);
        pl->filt_re[idx] = (fp2r + fp1r + fcr + fnr) * 0.25f;
        pl->filt_im[idx] = (fp2i + fp1i + fci + fni) * 0.25f;
        if (dg) {
          pl->filt_re[idx] += dRe;
          pl->filt_im[idx] += dIm;
        }
      } else if (p->bm == 1) {
        float re = wr[cur][idx], im = wi[cur][idx];
        if (dg) {
          re -= dRe;
          im -= dIm;
        }
        wienner(&re, &im, sX, sY, p->beta_x);
        if (dg) {
          re += dRe;
          im += dIm;
        }
        pl->filt_re[idx] = re;
        pl->filt_im[idx] = im;
      } else if (p->bm == 0) {
        /* Kalman, reference.cpp:334-383; state updated in place. */
        float re = wr[0][idx], im = wi[0][idx];
        float lRe = pl->k_last_re[idx], lIm = pl->k_last_im[idx];
        float ddRe = re - lRe, ddIm = im - lIm;
        float a2 = ddRe * ddRe, b2 = ddIm * ddIm;
        float mask = a2 < b2 ? b2 : a2; /* std::max(a, b) = (a < b) ? b : a */
        float cn = pat ? pl->pattern[i0] : p->kalman_cn;
        float s = pl->k_covar[idx] + pl->k_proc[idx];
        float gain = s / (s + cn);
        float newProc = gain * gain * cn;
        float newCovar = (1.0f - gain) * s;
        float dstRe = gain * re + (1.0f - gain) * lRe;
        float dstIm = gain * im + (1.0f - gain) * lIm;
        if (mask > kr2 * cn) {
          dstRe = re;
          dstIm = im;
          newCovar = cn;
          newProc = cn;
        }
        pl->filt_re[idx] = dstRe;
        pl->filt_im[idx] = dstIm;
        pl->k_covar[idx] = newCovar;
        pl->k_proc[idx] = newProc;
        pl->k_last_re[idx] = dstRe;
        pl->k_last_im[idx] = dstIm;
      } else {
        pl->filt_re[idx] = wr[0][idx];
        pl->filt_im[idx] = wi[0][idx];
      }
    }
  }
}

/* Phase 2a, per block (reference.cpp:392-413 and the window product of
 * :415-430): sharpen, inverse transform, times the synthesis window. The
 * windowed block goes to pl->blk; phase 2b adds it into the output. */
static void inverse_range(void* vctx, int lo, int hi, int tid) {
  (void)tid;
  filt_ctx* c = (filt_ctx*)vctx;
  orc_plane* pl = c->pl;
  const orc_internal_params* p = &pl->p;
  const int fbw = pl->fbw, bw = p->bw, bh = p->bh, ps = fbw * bh;
  const int dg = c->dg;
  fft_scratch s;
  scratch_init(&s, bw, bh);
  cpx* half = (cpx*)malloc(sizeof(cpx) * (size_t)ps);
  float* block = (float*)malloc(sizeof(float) * (size_t)bw * bh);
  for (int b = lo; b < hi; b++) {
    if (p->sharpen_on) {
      for (int r = 0; r < bh; r++)
        for (int cc = 0; cc < fbw; cc++) {
          size_t idx = (size_t)b * ps + r * fbw + cc;
          float re = pl->filt_re[idx], im = pl->filt_im[idx];
          float dRe = 0, dIm = 0;
          if (dg) {
            dRe = pl->corr_re[idx];
            dIm = pl->corr_im[idx];
            re -= dRe;
            im -= dIm;
          }
          float psd = re * re + im * im + 0.0000000000000000000000000000000000001f;
          float factor = pl->sharpen[r * fbw + cc];
          float g = 1.0f + factor * sqrtf(psd * p->ssmax / ((psd + p->ssmin) * (psd + p->ssmax)));
          re *= g;
          im *= g;
          if (dg) {
            re += dRe;
            im += dIm;
          }
          pl->filt_re[idx] = re;
          pl->filt_im[idx] = im;
        }
    }
    for (int i = 0; i < ps; i++) {
      half[i].re = pl->filt_re[(size_t)b * ps + i];
      half[i].im = pl->filt_im[(size_t)b * ps + i];
    }
    fft2d_inverse_half(half, bw, bh, fbw, &pl->row_plan, &pl->col_plan, block, &s);
    const float* win =
        (p->mode == 1) ? (pl->par[b] ? pl->win_syn_b : pl->win_syn_a) : pl->win_ana;
    float* dst = &pl->blk[(size_t)b * bw * bh];
    for (int i = 0; i < bw * bh; i++) dst[i] = block[i] * win[i];
  }
  free(half);
  free(block);
  scratch_free(&s);
}

/* Phase 2b, overlap-add for output rows [lo, hi): per pixel the blocks are
 * added in ascending block index, starting from 0, then chroma centering is
 * added back once (reference.cpp:415-436). */
static void ola_range(void* vctx, int lo, int hi, int tid) {
  (void)tid;
  filt_ctx* c = (filt_ctx*)vctx;
  orc_plane* pl = c->pl;
  const int bw = pl->p.bw, bh = pl->p.bh, W = pl->width;
  for (int y = lo; y < hi; y++) {
    float* orow = &c->out[(size_t)y * W];
    for (int x = 0; x < W; x++) orow[x] = 0.0f;
    for (int k = pl->row_start[y]; k < pl->row_start[y + 1]; k++) {
      int b = pl->row_list[k];
      int ly = y - pl->by[b];
      const float* brow = &pl->blk[(size_t)b * bw * bh + (size_t)ly * bw];
      for (int lx = 0; lx < bw; lx++) {
        int dx = pl->bx[b] + lx;
        if (dx < 0 || dx >= W) continue;
        orow[dx] += brow[lx];
      }
    }
    if (pl->chroma_norm != 0.0f)
      for (int x = 0; x < W; x++) orow[x] += pl->chroma_norm;
  }
}

/* src/cpu/reference.cpp:211-437. */
void orc_filter_and_synthesize(orc_plane* pl, const float* const* win_re,
                               const float* const* win_im, int nwin, float* out, int threads) {
  (void)nwin;
  const orc_internal_params* p = &pl->p;
  const int ps = pl->fbw * p->bh;
  const size_t total = (size_t)pl->nb * ps;
  if (!pl->filt_re) {
    pl->filt_re = (float*)malloc(sizeof(float) * total);
    pl->filt_im = (float*)malloc(sizeof(float) * total);
    pl->corr_re = (float*)malloc(sizeof(float) * total);
    pl->corr_im = (float*)malloc(sizeof(float) * total);
    pl->blk = (float*)malloc(sizeof(float) * (size_t)pl->nb * p->bw * p->bh);
  }
  filt_ctx c = {pl, win_re, win_im, out, p->degrid_on && pl->gs_re != NULL};
  if (c.dg) parallel_for(pl->nb, threads, corr_range, &c);

  if (p->bm == 0 && pl->kalman_first) {
    const int cur = 0;
    pl->k_last_re = (float*)malloc(sizeof(float) * total);
    pl->k_last_im = (float*)malloc(sizeof(float) * total);
    pl->k_covar = (float*)malloc(sizeof(float) * total);
    pl->k_proc = (float*)malloc(sizeof(float) * total);
    memcpy(pl->k_last_re, win_re[cur], sizeof(float) * total);
    memcpy(pl->k_last_im, win_im[cur], sizeof(float) * total);
    for (size_t i = 0; i < total; i++) {
      float v = pl->pattern ? pl->pattern[i % ps] : p->kalman_cn;
      pl->k_covar[i] = v;
      pl->k_proc[i] = v;
    }
    pl->kalman_first = 0;
  }
  parallel_for(pl->nb, threads, temporal_range, &c);
  parallel_for(pl->nb, threads, inverse_range, &c);
  parallel_for(pl->height, threads, ola_range, &c);
}

/* --------------------------------------------------------- clip runner -- */

static inline int clamp_frame(int n, int num) {
  if (n < 0) return 0;
  if (n > num - 1) return num - 1;
  return n;
}

typedef struct {
  int fn;
  float *re, *im;
} cache_slot;

/* src/fft3dcl.cpp:471-521 (CPU path of the frame callback) for one plane. */
int orc_run_clip(const orc_script_params* sp, int width, int height, int bits,
                 int sample_type, int chroma, int nframes, const uint8_t* const* frames,
                 ptrdiff_t pitch, int first, int count, uint8_t* const* out,
                 ptrdiff_t opitch, int threads, const char** err) {
  orc_internal_params ip;
  if (!orc_validate_params(sp, width, height, bits, &ip, err)) return -1;
  orc_plane* pl = orc_plane_new(&ip, width, height, bits, sample_type, chroma);
  if (ip.degrid_on) orc_build_degrid(pl);
  const size_t total = (size_t)pl->nb * pl->fbw * ip.bh;
  const int nslots = ip.bt + 2;
  cache_slot* cache = (cache_slot*)calloc((size_t)nslots, sizeof(cache_slot));
  for (int k = 0; k < nslots; k++) {
    cache[k].fn = -1;
    cache[k].re = (float*)malloc(sizeof(float) * total);
    cache[k].im = (float*)malloc(sizeof(float) * total);
  }
  float* plane = (float*)malloc(sizeof(float) * (size_t)width * height);
  float* res = (float*)malloc(sizeof(float) * (size_t)width * height);
  const float* wr[4];
  const float* wi[4];
  /* Kalman carries state from frame 0 on: run the frames before `first`. */
  int start = ip.bm == 0 ? 0 : first;
  for (int n = start; n < first + count; n++) {
    int win[4], nw = 0;
    if (ip.bm >= 2)
      for (int i = 0; i < ip.bt; i++) win[nw++] = clamp_frame(n - ip.current + i, nframes);
    else
      win[nw++] = clamp_frame(n, nframes);
    /* Cache kept to [n-current-1, n-current+bt] like the reference's prune. */
    int lo = n - ip.current - 1, hi = n - ip.current + ip.bt;
    for (int k = 0; k < nslots; k++)
      if (cache[k].fn >= 0 && ip.bm >= 2 && (cache[k].fn < lo || cache[k].fn > hi))
        cache[k].fn = -1;
      else if (ip.bm < 2)
        cache[k].fn = -1;
    for (int i = 0; i < nw; i++) {
      int slot = -1;
      for (int k = 0; k < nslots; k++)
        if (cache[k].fn == win[i]) slot = k;
      if (slot < 0) {
        for (int k = 0; k < nslots; k++)
          if (cache[k].fn < 0) {
            slot = k;
            break;
          }
        orc_upload(pl, frames[win[i]], pitch, plane);
        orc_compute_spectra(pl, plane, cache[slot].re, cache[slot].im, threads);
        cache[slot].fn = win[i];
      }
      wr[i] = cache[slot].re;
      wi[i] = cache[slot].im;
    }
    orc_filter_and_synthesize(pl, wr, wi, nw, res, threads);
    if (n >= first) orc_download(pl, res, out[n - first], opitch);
  }
  for (int k = 0; k < nslots; k++) {
    free(cache[k].re);
    free(cache[k].im);
  }
  free(cache);
  free(plane);
  free(res);
  orc_plane_free(pl);
  return 0;
}
