/*
 * fft3d_gb300.h -- C ABI of the GB300 FFT3D block-FFT denoise engine.
 *
 * One engine handles one plane of one filter instance, the unit the reference
 * backend works in (class GpuRef, src/cl/gpu.h:16-88 of HumbleUser33/FFT3dCL).
 * Each entry point below names the reference member it replaces. Plain C types
 * only; a cudaStream_t is passed as void*.
 *
 * Per frame a host does what the reference plugin does (src/fft3dcl.cpp:388-468):
 *   for each frame of the temporal window: if (!f3d_has(e, fn)) f3d_forward_raw(e, fn, ...);
 *   f3d_process_raw(e, window, n, dst, bytes);
 *   f3d_prune(e, lo, hi);
 *
 * Errors: every call returns F3D_OK (0) or a negative F3D_E_* code. The
 * message is kept per engine (f3d_engine_error) and, for calls without an
 * engine, per thread (f3d_last_error). There is no CPU fallback: when the
 * CUDA path cannot run, the call fails.
 *
 * Threading: all calls on one engine are serialised by the engine's own
 * mutex (the reference serialises one instance with a mutex,
 * src/fft3dcl.cpp:365-368). Different engines may be driven from different
 * threads.
 */
#ifndef FFT3D_GB300_H
#define FFT3D_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define F3D_ABI_VERSION 1

enum {
  F3D_OK = 0,
  F3D_E_PARAM = -1,     /* invalid parameters or arguments                */
  F3D_E_CUDA = -2,      /* a CUDA call failed (message has the reason)    */
  F3D_E_NOMEM = -3,     /* device allocation failed                       */
  F3D_E_STATE = -4,     /* call out of order (missing spectra, ...)       */
  F3D_E_UNSUPPORTED = -5, /* feature not available on this path          */
  F3D_E_BUSY = -6         /* no capacity now (server slot, budget, queue); retry later */
};

/* Script-level parameters: names, types and defaults of ScriptParams,
 * src/params.h:8-27. f3d_default_params fills the defaults. */
typedef struct {
  float sigma, beta;
  int bw, bh, bt;
  float sharpen;
  int plane, mode, bordersize, precision;
  float degrid, scutoff, svr, smin, smax, kratio;
  int ow, oh, wintype, interlaced;
  float sigma2, sigma3, sigma4;
  int oldfft;
} f3d_script_params;

/* Validated parameters: InternalParams, src/params.h:30-59. */
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
} f3d_internal_params;

/* Plane geometry: PlaneGeom, src/cpu/reference.h:17-22. */
typedef struct {
  int width, height;
  int bits;        /* 8..16 for integer samples, 32 for float */
  int sample_type; /* 0 integer, 1 float                       */
  int chroma;      /* YUV chroma plane (mode-1 centering)      */
} f3d_plane_geom;

/* Arithmetic form of the block transforms. */
enum {
  F3D_FORM_EXACT = 0, /* radix-2 DIT in the reference's operation order, no
                         fused multiply-add: same bits as the CPU backend   */
  F3D_FORM_FAST = 1,  /* packed real FFTs with FMA, fp32                     */
  F3D_FORM_TC = 2     /* DFT-matrix contraction on the tensor cores          */
};

typedef struct {
  int device;   /* CUDA device ordinal                                   */
  int form;     /* F3D_FORM_*                                            */
  void* stream; /* cudaStream_t to run on, NULL: the engine makes one    */
  int flags;    /* F3D_FLAG_*                                            */
} f3d_options;

/* Run filter/inverse and overlap-add as separate kernels even where the
 * fused sweep kernel applies (for comparisons). */
#define F3D_FLAG_UNFUSED 1
/* Sweep tuning: bulk-prefetch the next block row's spectra into L2 when a
 * row starts, or once the row's spectra are read. Off by default (measured
 * at 4K 10-bit bt=4: off 0.288 ms, late 0.292 ms, early 0.322 ms). */
#define F3D_FLAG_PREFETCH_EARLY 2
#define F3D_FLAG_PREFETCH_LATE 4
/* Cache the spectra as fp16 pairs (half the bytes: the forward writes half
 * as much, the filter reads half as much), the storage of the original
 * filter's precision 0 and 1: its FFT returns spectra in HALF4 textures
 * unless precision is FLOAT32_ALL (upstream/FFT3dGPU/FFT.cpp:152), which is
 * forced above 8 bits (upstream/FFT3dGPU/FFT3dGPU.cpp:244-246; the port's
 * src/params.h:116-120). Honoured where that storage applied and the kernels take it: 8-bit
 * integer planes, precision 0 or 1, the fused tensor-core form; ignored
 * elsewhere (f3d_engine_info.half_spectra says which). Arithmetic stays
 * fp32; results are within the 8-bit tolerance of the fp32 path, not
 * bit-equal to it. The reference port ignores precision, so this is opt-in. */
#define F3D_FLAG_HALF_SPECTRA 8
/* Tests of the error path only: the next output of a fused tensor-core
 * engine leaves out one operand-tile copy of its inverse kernel, so that the
 * bounded wait for it gives up after its one-second limit with nothing in
 * flight; the output is then invalid and f3d_synchronize reports the wait.
 * Applies once. */
#define F3D_FLAG_TEST_WAIT_TIMEOUT (1 << 20)

typedef struct {
  int nblocks, fbw, ncols, nrows;
  int bytes_per_sample;
  int raw_path;
  size_t spectrum_bytes; /* one frame's half spectra in HBM */
  size_t device_bytes;   /* all device memory held by the engine */
  int cached_frames;
  float chroma_norm;
  int form; /* form the engine runs: Kalman (bt=0) and 4-wide blocks run
               F3D_FORM_EXACT whatever was asked */
  int fused; /* filter, inverse, overlap-add and packing run as one kernel */
  int half_spectra; /* spectra cached as fp16 pairs (F3D_FLAG_HALF_SPECTRA applied) */
} f3d_engine_info;

typedef struct f3d_engine f3d_engine;

/* Plugin argument defaults (src/fft3dcl.cpp:171-195) for bw/bh/mode/sigma
 * as given: degrid = mode==1 ? 1 : 0, ow/oh = bw/2, bh/2, sigma2..4 = sigma. */
void f3d_default_params(f3d_script_params* sp);

/* validateParams, src/params.h:76-148 (roundPow2Clamp :62-72). */
int f3d_validate_params(const f3d_script_params* sp, int width, int height, int bits,
                        f3d_internal_params* out);

/* Thread-local message of the last failing call made without an engine. */
const char* f3d_last_error(void);

/* GpuRef::GpuRef (src/cl/gpu.cpp:59-245): validates, builds the block grid
 * and all tables (windows, sigma pattern, sharpen LUT, degrid sample) and
 * allocates the device buffers. */
int f3d_engine_create(const f3d_script_params* sp, const f3d_plane_geom* geom,
                      const f3d_options* opts, f3d_engine** out);
/* GpuRef::~GpuRef (src/cl/gpu.cpp:247-270). */
void f3d_engine_destroy(f3d_engine* e);
/* GpuRef::error (src/cl/gpu.h:23). */
const char* f3d_engine_error(const f3d_engine* e);
int f3d_engine_get_info(f3d_engine* e, f3d_engine_info* info);
/* Host copy of an engine table (F3D_TAB_*); returns the float count. */
int f3d_engine_get_table(f3d_engine* e, int which, float* dst);

enum {
  F3D_TAB_WIN_ANA = 0, F3D_TAB_WIN_SYN_A, F3D_TAB_WIN_SYN_B, F3D_TAB_PATTERN,
  F3D_TAB_SHARPEN, F3D_TAB_GS_RE, F3D_TAB_GS_IM, F3D_TAB_TWIDDLE_ROW, F3D_TAB_TWIDDLE_COL
};
/* The same tables computed on the host without a device (the PlaneRef
 * constructor, src/cpu/reference.cpp:19-80, and buildDegridSample :172-198). */
int f3d_compute_table(const f3d_script_params* sp, const f3d_plane_geom* geom, int which, float* dst);

/* GpuRef::forward (src/cl/gpu.cpp:326-347): forward transform of a host float
 * plane (width*height floats, packed), cached as frame fn. */
int f3d_forward(f3d_engine* e, int fn, const float* plane);
/* GpuRef::forwardRaw (src/cl/gpu.cpp:349-372): same from the plane's native
 * samples, `bytes` = width*height*bytes_per_sample, packed rows. */
int f3d_forward_raw(f3d_engine* e, int fn, const void* raw, size_t bytes);
/* Same from a plane already in device memory, rows `pitch` bytes apart. */
int f3d_forward_device(f3d_engine* e, int fn, const void* dev_plane, size_t pitch);
/* Host copy of the cached half spectra of frame fn: nblocks x bh x fbw
 * complex values, interleaved re, im (the device layout). For tests and
 * tooling; the reference keeps them device-only (src/cl/gpu.h:79). */
int f3d_get_spectra(f3d_engine* e, int fn, float* dst);
/* GpuRef::has (src/cl/gpu.h:35). */
int f3d_has(f3d_engine* e, int fn);
/* GpuRef::rawPath / bytesPerSample (src/cl/gpu.h:37-38). */
int f3d_raw_path(f3d_engine* e);
int f3d_bytes_per_sample(f3d_engine* e);
/* GpuRef::uploadDegridSample (src/cl/gpu.cpp:374-387). The engine builds the
 * degrid sample itself; this only makes it active (it is also made active by
 * the first process call when degrid is on). */
int f3d_upload_degrid_sample(f3d_engine* e);

/* GpuRef::process (src/cl/gpu.cpp:460-482): filter + inverse + overlap-add
 * of the window frames (frame numbers in temporal order, bt of them for
 * bt >= 2, else one); out receives width*height floats. */
int f3d_process(f3d_engine* e, const int* window, int n, float* out);
/* GpuRef::processRaw (src/cl/gpu.cpp:484-505): same, packed to the native
 * sample format into dst (`bytes` = width*height*bytes_per_sample). */
int f3d_process_raw(f3d_engine* e, const int* window, int n, void* dst, size_t bytes);
/* Same into device memory, rows `pitch` bytes apart; returns once queued. */
int f3d_process_device(f3d_engine* e, const int* window, int n, void* dev_dst, size_t pitch);

/* GpuRef::pruneCache (src/cl/gpu.cpp:507-517): drop cached spectra outside
 * [lo, hi]; a negative bound is disabled. */
int f3d_prune(f3d_engine* e, int lo, int hi);

/* Wait for all queued work of the engine. F3D_E_CUDA when a tensor-core
 * kernel's bounded wait gave up since the last call (the message names the
 * wait; the outputs queued since are invalid); the report clears it. */
int f3d_synchronize(f3d_engine* e);
/* Device time of the kernels of the last forward / process calls in ms
 * (CUDA events on the engine stream; valid after f3d_synchronize):
 * ms[0] forward transform;
 * ms[1] filter + inverse (separate kernels), the whole sweep (fused fast
 *       form) or the filter kernel (tensor-core form);
 * ms[2] overlap-add + pack (separate kernels), the seam merge (fused fast
 *       form) or inverse + overlap-add + seam merge (tensor-core form). */
int f3d_last_kernel_ms(f3d_engine* e, float* ms);

/* GpuRef::liveInstances / liveBytes (src/cl/gpu.cpp:44-57). */
int f3d_live_instances(void);
size_t f3d_live_bytes(void);

/* Number of kernel launches made by this library since load (all engines). */
uint64_t f3d_kernel_launches(void);

/* Denoise one frame without allocating device memory. No counterpart in the
 * reference: it exists for callers that cannot call cudaMalloc -- hosts that
 * hand out a fixed device-memory budget up front and own every byte of it,
 * and real-time threads that must not take cudaMalloc/cudaFree's device-wide
 * synchronisation.
 *
 * The caller passes the window frames (`nwin` device pointers in temporal
 * order, bt of them for bt >= 2, else one; rows `src_pitch` bytes apart) and
 * the output plane (`dst_pitch`); the work is queued on `stream` (NULL: the
 * default stream) with the current device's kernels of the exact form, and
 * the result has the same bits as f3d_forward_device + f3d_process_device.
 * Spectra, windowed blocks and tables live in one static device array of
 * F3D_NOALLOC_SCRATCH_BYTES that every GPU that loads this library holds
 * until the process exits. The first call on a device (and the first after a
 * cudaDeviceReset) looks the array's address up with cudaGetSymbolAddress,
 * that device current; make that first call before any stream capture. All
 * calls share the array and it keeps the last call's contents; every byte a
 * call reads is written by that call first, on its stream. Calls whose work
 * overlaps on a GPU race on the array: order them (one stream, or events).
 * Kalman (bt=0) needs state across frames and is refused, as are blocks above
 * 64 and any plane whose spectra and blocks do not fit the array
 * (F3D_E_UNSUPPORTED, the message says how many bytes it needs). What fits:
 * tables + nwin * round256(8 * nblocks * (bw/2+1) * bh) +
 * round256(4 * nblocks * bw * bh) bytes <= 64 MiB: with 32x32 blocks at
 * half overlap up to about 0.6 M samples at bt=4 (1024x576 fits, 1280x720
 * does not) and about 0.9 M at bt=3 (1280x720 fits). Calls no
 * cudaMalloc, cudaFree or other allocating routine and allocate no host
 * memory; the tables are built in about 110 KB of the calling thread's stack. */
#define F3D_NOALLOC_SCRATCH_BYTES ((size_t)64 << 20)
int f3d_denoise_noalloc(const f3d_script_params* sp, const f3d_plane_geom* geom,
                        const void* const* dev_window, int nwin, size_t src_pitch, void* dev_dst,
                        size_t dst_pitch, void* stream);

/* ---- Batches of planes -----------------------------------------------------
 * One temporal step of up to sixteen planes (the planes of a YUV frame,
 * planes of several streams, or consecutive outputs of one plane: the same
 * engine given several times) with one launch per kernel: the forward
 * transform of each plane's entering frame, then filter, inverse and
 * overlap-add of each plane's window. The engines must run the fused
 * tensor-core form (F3D_FORM_TC, half overlap, 16x16 or 32x32 blocks), or
 * all the fast form's fused sweep (F3D_FORM_FAST, half overlap, 8x8 to 32x32
 * blocks: one forward launch per entering frame, the sweeps of all planes in
 * one launch), on one device and one stream, with the same block size,
 * overlap, window type, temporal mode and sample format; plane sizes and bit
 * depths may differ.
 * F3D_BATCH_GRAPH (tensor-core form): each step shape is captured once as a
 * CUDA graph and replayed with its kernel nodes re-pointed at the step's
 * buffers.
 * F3D_BATCH_AUTOTUNE (tensor-core form): the first step in which every plane
 * enters a frame times the candidate launch shapes (forward CTAs per SM,
 * filter-kernel register budget) and keeps the fastest; results are cached
 * per batch shape for the process. Results are the same as the engines' own
 * calls. */
#define F3D_BATCH_GRAPH 1
#define F3D_BATCH_AUTOTUNE 2
typedef struct f3d_batch f3d_batch;
int f3d_batch_create(f3d_engine* const* engines, int n, int flags, f3d_batch** out);
void f3d_batch_destroy(f3d_batch* b);
const char* f3d_batch_error(f3d_batch* b);
/* Plane i: forward frame fns[i] from dev_src[i] (skipped when fns[i] < 0 or
 * the frame is cached), then the output of window windows[i] (nwin[i]
 * frames, as for f3d_process; nwin[i] = 0: no output) into dev_dst[i].
 * Queued on the engines' stream. When no entering frame is in its plane's
 * window (the caller forwards one frame ahead: frame n+2 with output n at
 * bt=4), the forward runs concurrently with the outputs on a second stream
 * and joins the engines' stream before the step ends. */
int f3d_batch_step(f3d_batch* b, const int* fns, const void* const* dev_src, const size_t* src_pitch,
                   const int* const* windows, const int* nwin, void* const* dev_dst, const size_t* dst_pitch);
/* Launch shape in use; returns 1 when the autotuner has chosen it. */
int f3d_batch_tune(f3d_batch* b, int* fwd_ctas_per_sm, int* filter_minb);
/* Pins the launch shape (the autotuner then keeps it): fwd_ctas_per_sm 1 to
 * 3 forward CTAs per SM, filter_minb 3..5 filter CTAs per SM. Every shape gives the same
 * results. F3D_E_PARAM for any other shape. */
int f3d_batch_set_tune(f3d_batch* b, int fwd_ctas_per_sm, int filter_minb);
/* Device times (ms) of the last step with outputs that ran outside a CUDA
 * graph (steps replayed as a graph are not timed): ms[0] the filter kernel,
 * ms[1] the inverse + overlap-add kernel and the seam merge (fast form:
 * ms[0] the fused sweep, ms[1] the seam merge). Waits for that step.
 * F3D_E_STATE when no such step ran. */
int f3d_batch_last_kernel_ms(f3d_batch* b, float* ms);

/* ---- Serving loop ----------------------------------------------------------
 * Replaces the reference's one-instance-per-clip model (src/fft3dcl.cpp:289,
 * :365-368: VapourSynth requests serialised per instance by a mutex) for
 * hosts that serve many streams at once. A server owns one GPU and one
 * scheduler thread. Each stream is one plane sequence with its own
 * parameters, size and format, and its own engine (window spectra and Kalman
 * state stay in HBM). Streams are admitted while the device memory of all open
 * streams fits `hbm_budget` and fewer than `max_streams` are open; otherwise
 * f3d_server_open returns F3D_E_BUSY. On every pass the scheduler launches
 * the next output of every stream whose window frames have arrived. Streams
 * whose engines run the fused tensor-core form and whose kernels take the
 * same parameters (block size, overlap, window, temporal mode, sample
 * format) form lanes of up to three streams in the order they open (the
 * planes of a YUV stream); each lane has one CUDA stream, and its ready
 * outputs go into shared steps: one launch per kernel for its planes of any
 * size. Lanes and the other streams (on CUDA streams of their own) run
 * concurrently on the device. Streams that open while others run join at once. Latency of
 * an output: from the arrival of the last input frame its window needs to
 * the end of its copy to host memory. A video stream of several planes (YUV)
 * is one server stream per plane. */
typedef struct {
  int device;
  int form;          /* F3D_FORM_* for every stream (per-stream fallbacks as in create) */
  int max_streams;
  size_t hbm_budget; /* bytes of device memory the open streams may hold */
} f3d_server_config;

typedef struct {
  long long frames;  /* outputs finished */
  double p50_ms, p99_ms, max_ms, mean_ms;
  double seconds;    /* first input ready to last output done */
  int open_streams;
  size_t used_bytes; /* admitted device memory */
  long long shared_steps;   /* steps launched for several streams at once */
  long long shared_outputs; /* outputs of those steps */
  int max_shared;           /* most outputs in one shared step */
  double busy_ms;           /* scheduler thread: time spent in passes that launched work */
} f3d_server_stats;

typedef struct f3d_server f3d_server;

int f3d_server_create(const f3d_server_config* cfg, f3d_server** out);
void f3d_server_destroy(f3d_server* sv);
/* Opens a stream of `nframes` frames (window clamping at both ends as in the
 * plugin, src/fft3dcl.cpp:303-331); *sid receives its id. */
int f3d_server_open(f3d_server* sv, const f3d_script_params* sp, const f3d_plane_geom* geom, int nframes,
                    int* sid);
/* Frame n (submit in frame order) from host memory; copied before return.
 * F3D_E_BUSY when the stream holds its maximum of frames not yet uploaded. */
int f3d_server_submit(f3d_server* sv, int sid, int n, const void* src, long long pitch);
/* Next finished output of the stream in frame order, waiting up to
 * timeout_ms; *n receives its frame number and dst (if not NULL) its samples.
 * F3D_E_BUSY when none finished in time. One thread polls a given stream. */
int f3d_server_poll(f3d_server* sv, int sid, int* n, void* dst, long long pitch, int timeout_ms);
/* The same, with the output's latency interval: *ready_ms when the last
 * input frame its window needs arrived, *done_ms when its copy to host
 * memory finished (milliseconds on one steady clock, the same for all
 * streams of the server; either pointer may be NULL). */
int f3d_server_poll_timed(f3d_server* sv, int sid, int* n, void* dst, long long pitch, int timeout_ms,
                          double* ready_ms, double* done_ms);
/* Releases the stream and its share of the budget. */
int f3d_server_close(f3d_server* sv, int sid);
int f3d_server_get_stats(f3d_server* sv, f3d_server_stats* st);

#ifdef __cplusplus
}
#endif
#endif
