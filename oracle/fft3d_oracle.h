/*
 * fft3d_oracle.h -- CPU oracle for the FFT3D block-FFT denoise path.
 *
 * TEST INFRASTRUCTURE ONLY. This library is the oracle the CUDA engine is
 * compared with (tests, the smoke check and the CPU baseline leg of the
 * benchmark). The product never links, loads or calls it.
 *
 * It restates, in plain C99, the fp32 CPU backend of HumbleUser33/FFT3dCL
 * (src/cpu/reference.cpp, src/cpu/fft.cpp, src/cpu/tables.cpp, src/params.h)
 * with the same operation order, so that compiled with -ffp-contract=off it
 * produces the same bits as that backend. Each function cites the reference
 * file:line it follows. Parity is pinned two ways: against the reference's own
 * sources compiled in place (oracle/Makefile -> oracle/_ref/) and against the
 * golden vectors in tests/golden/ that were generated from that build.
 *
 * The only structural change is scheduling: the clip runner may spread the
 * blocks of one frame over host threads. Every per-pixel sum keeps the
 * reference's block order, so the output does not depend on the thread count.
 */
#ifndef FFT3D_ORACLE_H
#define FFT3D_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Script-level parameters (src/params.h:8-27). */
typedef struct {
  float sigma, beta;
  int bw, bh, bt;
  float sharpen;
  int plane, mode, bordersize, precision;
  float degrid, scutoff, svr, smin, smax, kratio;
  int ow, oh, wintype, interlaced;
  float sigma2, sigma3, sigma4;
  int oldfft;
} orc_script_params;

/* Validated parameters (src/params.h:30-59). */
typedef struct {
  float sigma, beta;
  int bw, bh, bm, bt;
  float sharpen;
  int sharpen_on, mode, bordersize, precision;
  float degrid;
  int degrid_on;
  float scutoff, svr, smin, smax, kratio;
  int ow, oh, wintype, interlaced;
  float sigma2, sigma3, sigma4;
  int use_pattern, current, nx, ny, totw, toth, oldfft;
  float wiener_s, beta_x, kalman_cn, ssmin, ssmax;
} orc_internal_params;

typedef struct orc_plane orc_plane;

/* Table selectors for orc_get_table. */
enum {
  ORC_TAB_WIN_ANA = 0,  /* bw*bh analysis window                     */
  ORC_TAB_WIN_SYN_A,    /* bw*bh synthesis window, even-parity blocks */
  ORC_TAB_WIN_SYN_B,    /* bw*bh synthesis window, odd-parity blocks  */
  ORC_TAB_PATTERN,      /* fbw*bh sigma pattern (0 entries if off)    */
  ORC_TAB_SHARPEN,      /* fbw*bh sharpen LUT (0 entries if off)      */
  ORC_TAB_GS_RE,        /* fbw*bh degrid sample, real part            */
  ORC_TAB_GS_IM,        /* fbw*bh degrid sample, imaginary part       */
  ORC_TAB_TWIDDLE_ROW,  /* bw/2 complex twiddles, interleaved re,im   */
  ORC_TAB_TWIDDLE_COL   /* bh/2 complex twiddles, interleaved re,im   */
};

int orc_round_pow2_clamp(int v);
int orc_validate_params(const orc_script_params* sp, int width, int height, int bits,
                        orc_internal_params* out, const char** err);

orc_plane* orc_plane_new(const orc_internal_params* p, int width, int height, int bits,
                         int sample_type, int chroma);
void orc_plane_free(orc_plane* pl);
int orc_nblocks(const orc_plane* pl);
int orc_fbw(const orc_plane* pl);
int orc_ncols(const orc_plane* pl);
float orc_chroma_norm(const orc_plane* pl);
void orc_get_grid(const orc_plane* pl, int* bx, int* by, uint8_t* par);
/* Copies a table into dst and returns its element count (floats). dst may be
 * NULL to query the size. */
int orc_get_table(orc_plane* pl, int which, float* dst);

void orc_upload(const orc_plane* pl, const uint8_t* src, ptrdiff_t pitch, float* dst);
void orc_download(const orc_plane* pl, const float* src, uint8_t* dst, ptrdiff_t pitch);
/* re/im hold nblocks*fbw*bh floats each, block-major, row-major in a block. */
void orc_compute_spectra(orc_plane* pl, const float* plane, float* re, float* im, int threads);
void orc_build_degrid(orc_plane* pl);
/* win_re/win_im: nwin spectra (bt for bm>=2, else 1), temporal order. */
void orc_filter_and_synthesize(orc_plane* pl, const float* const* win_re,
                               const float* const* win_im, int nwin, float* out, int threads);

/* 1D transforms of the reference FftPlan (src/cpu/fft.cpp:8-58); data is
 * interleaved complex, n a power of two. */
void orc_fft1d(int n, const float* in, float* out, int inverse);
/* 2D block transforms (src/cpu/fft.cpp:68-119). full: bw*bh interleaved
 * complex; half: fbw*bh interleaved complex. */
void orc_fft2d_forward(const float* block, int bw, int bh, float* full);
void orc_fft2d_inverse_half(const float* half, int bw, int bh, float* block);

/*
 * Whole-clip driver for one plane, the CPU path of the reference plugin
 * (src/fft3dcl.cpp:471-521): window frames clamped to the clip, spectra cached
 * per frame, filter + synthesis, download. frames[k] is source frame k
 * (nframes of them, rows `pitch` bytes apart); output frames first..first+count-1
 * are written to out[0..count-1] (rows `opitch` apart). Returns 0 or -1 with *err.
 */
int orc_run_clip(const orc_script_params* sp, int width, int height, int bits,
                 int sample_type, int chroma, int nframes, const uint8_t* const* frames,
                 ptrdiff_t pitch, int first, int count, uint8_t* const* out,
                 ptrdiff_t opitch, int threads, const char** err);

#ifdef __cplusplus
}
#endif
#endif
