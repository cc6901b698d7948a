// f3d_plugin.cpp -- VapourSynth API-4 plugin over the GB300 engine.
//
// Drop-in for the reference plugin (src/fft3dcl.cpp of HumbleUser33/FFT3dCL):
// same identifier, namespace, function name, argument string, defaults,
// clamping, plane semantics, temporal-window requests and cache pruning, and
// Kalman run in frame order (fmFrameState). The backend is the C ABI of
// include/fft3d_gb300.h; there is no CPU fallback, so device=0 and any GPU
// failure are reported as errors (mapSetError at create, setFilterError per
// frame). The arithmetic form is taken from FFT3DCL_FORM (exact | fast | tc,
// default tc: within the reference GPU path's tolerance of its CPU backend,
// +-1 LSB at 8 bits and +-4 at 10; exact gives the CPU backend's bits; Kalman
// always runs exact). FFT3DCL_LOG names a file that receives one line per
// instance created or released with the live engine count and device bytes.
// FFT3DCL_TIME names a file to which every released instance appends the
// process-wide time per stage of the frame path (src/timing.h:1-31 of the
// reference): wall-clock spans of getFrame, and the device time of the
// engine's kernels from its CUDA events.
#include "VSHelper4.h"
#include "VapourSynth4.h"
#include "fft3d_gb300.h"

#include <atomic>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <mutex>
#include <string>
#include <vector>

namespace {

// ---- stage timing (FFT3DCL_TIME) ----

enum Stage {
  kFetch,      // getFrameFilter of the window frames
  kAlloc,      // newVideoFrame
  kCopy,       // planes the filter does not process
  kLock,       // waiting for the instance mutex
  kForward,    // upload + forward launch of the frames entering the window
  kProcess,    // filter + inverse + overlap-add launches and the readback
  kPrune,      // spectra cache bookkeeping
  kGpuFwd,     // device time: forward transform
  kGpuFilter,  // the filter kernel (exact form: filter + inverse)
  kGpuSynth,   // inverse + overlap-add + pack (exact form: overlap-add + pack)
  kStages
};
const char* const kStageName[kStages] = {
    "fetch source frames", "allocate output frame", "copy untouched planes", "wait for instance lock",
    "upload + forward",    "filter .. readback",    "prune spectra cache",   "GPU: forward transform",
    "GPU: filter",         "GPU: synthesis"};
std::atomic<long long> g_stage_ns[kStages];
std::atomic<long long> g_stage_calls[kStages];

bool time_on() {
  static const bool on = [] {
    const char* p = std::getenv("FFT3DCL_TIME");
    return p && *p;
  }();
  return on;
}

long long now_ns() {
  return std::chrono::duration_cast<std::chrono::nanoseconds>(std::chrono::steady_clock::now().time_since_epoch())
      .count();
}

void add_stage(Stage s, long long ns) {
  g_stage_ns[s] += ns;
  g_stage_calls[s] += 1;
}

// Records the span from construction to destruction when timing is on.
struct Span {
  Stage s;
  long long t0;
  explicit Span(Stage st) : s(st), t0(time_on() ? now_ns() : 0) {}
  ~Span() {
    if (t0) add_stage(s, now_ns() - t0);
  }
};

void dump_stages(const char* tag) {
  if (!time_on()) return;
  FILE* f = std::fopen(std::getenv("FFT3DCL_TIME"), "a");
  if (!f) return;
  std::fprintf(f, "== %s ==\n", tag);
  long long total = 0;
  for (int i = 0; i < kStages; i++) {
    const long long ns = g_stage_ns[i].load(), calls = g_stage_calls[i].load();
    if (i < kGpuFwd) total += ns;
    std::fprintf(f, "  %-24s calls=%8lld  %9.4f s  %8.4f ms/call\n", kStageName[i], calls, ns / 1e9,
                 calls ? ns / 1e6 / (double)calls : 0.0);
  }
  std::fprintf(f, "  %-24s %21.4f s\n", "host stages total", total / 1e9);
  std::fclose(f);
}

struct Instance {
  f3d_script_params sp{};
  f3d_internal_params ip{};
  VSVideoInfo vi{};
  VSNode* clip = nullptr;
  std::vector<int> planes;
  std::vector<f3d_engine*> engines;
  std::vector<uint8_t> staging;  // rows packed when a frame's stride is not width*bps
  std::mutex mtx;
  ~Instance() {
    for (f3d_engine* e : engines) f3d_engine_destroy(e);
  }
};

void log_line(VSCore* core, const VSAPI* vsapi, int type, const std::string& msg) {
  vsapi->logMessage(type, msg.c_str(), core);
  const char* path = std::getenv("FFT3DCL_LOG");
  if (path && *path) {
    if (FILE* f = std::fopen(path, "a")) {
      char ts[16] = {};
      std::time_t now = std::time(nullptr);
      std::strftime(ts, sizeof(ts), "%H:%M:%S", std::localtime(&now));
      std::fprintf(f, "%s %s\n", ts, msg.c_str());
      std::fclose(f);
    }
  }
}

void log_usage(VSCore* core, const VSAPI* vsapi, const char* what) {
  char msg[160];
  std::snprintf(msg, sizeof(msg), "FFT3DCL: %s - %d GPU engine(s) alive, %.0f MiB of device buffers", what,
                f3d_live_instances(), (double)f3d_live_bytes() / 1048576.0);
  log_line(core, vsapi, mtInformation, msg);
}

int form_from_env() {
  const char* f = std::getenv("FFT3DCL_FORM");
  if (!f || !*f) return F3D_FORM_TC;
  if (!std::strcmp(f, "exact")) return F3D_FORM_EXACT;
  if (!std::strcmp(f, "fast")) return F3D_FORM_FAST;
  return F3D_FORM_TC;
}

inline int clamp_frame(int n, int num) { return n < 0 ? 0 : (n > num - 1 ? num - 1 : n); }

const VSFrame* VS_CC get_frame(int n, int reason, void* data, void**, VSFrameContext* ctx, VSCore* core,
                               const VSAPI* vsapi) {
  Instance* in = static_cast<Instance*>(data);
  const f3d_internal_params& ip = in->ip;
  const int num = in->vi.numFrames;
  if (reason == arInitial) {
    // src/fft3dcl.cpp:319-330: the clamped window as one contiguous range.
    if (ip.bm >= 2) {
      const int lo = clamp_frame(n - ip.current, num), hi = clamp_frame(n - ip.current + ip.bt - 1, num);
      for (int f = lo; f <= hi; f++) vsapi->requestFrameFilter(f, in->clip, ctx);
    } else {
      vsapi->requestFrameFilter(clamp_frame(n, num), in->clip, ctx);
    }
    return nullptr;
  }
  if (reason != arAllFramesReady) return nullptr;

  const VSFrame* src;
  {
    Span t(kFetch);
    src = vsapi->getFrameFilter(n, in->clip, ctx);
  }
  VSFrame* dst;
  {
    Span t(kAlloc);
    dst = vsapi->newVideoFrame(&in->vi.format, in->vi.width, in->vi.height, src, core);
  }
  const int bps = in->vi.format.bytesPerSample;
  const long long t_copy = time_on() ? now_ns() : 0;
  for (int p = 0; p < in->vi.format.numPlanes; p++) {  // untouched planes copied
    bool processed = false;
    for (int q : in->planes) processed |= q == p;
    if (processed) continue;
    const uint8_t* sp = vsapi->getReadPtr(src, p);
    uint8_t* dp = vsapi->getWritePtr(dst, p);
    const ptrdiff_t ss = vsapi->getStride(src, p), ds = vsapi->getStride(dst, p);
    const int h = vsapi->getFrameHeight(src, p), row = vsapi->getFrameWidth(src, p) * bps;
    for (int y = 0; y < h; y++) std::memcpy(dp + y * ds, sp + y * ss, row);
  }
  if (t_copy) add_stage(kCopy, now_ns() - t_copy);

  const long long t_lock = time_on() ? now_ns() : 0;
  std::lock_guard<std::mutex> lock(in->mtx);
  if (t_lock) add_stage(kLock, now_ns() - t_lock);
  for (size_t k = 0; k < in->planes.size(); k++) {
    const int p = in->planes[k];
    f3d_engine* e = in->engines[k];
    const int w = vsapi->getFrameWidth(src, p), h = vsapi->getFrameHeight(src, p);
    const size_t row = (size_t)w * bps, bytes = row * h;
    std::vector<int> window;
    if (ip.bm >= 2)
      for (int i = 0; i < ip.bt; i++) window.push_back(clamp_frame(n - ip.current + i, num));
    else
      window.push_back(clamp_frame(n, num));
    bool ok = true;
    int forwards = 0;
    for (int fn : window) {
      if (f3d_has(e, fn)) continue;
      const VSFrame* fr;
      {
        Span t(kFetch);
        fr = vsapi->getFrameFilter(fn, in->clip, ctx);
      }
      Span t(kForward);
      forwards++;
      const uint8_t* sp = vsapi->getReadPtr(fr, p);
      const ptrdiff_t ss = vsapi->getStride(fr, p);
      if ((size_t)ss == row) {
        ok = f3d_forward_raw(e, fn, sp, bytes) == F3D_OK;
      } else {
        in->staging.resize(bytes);
        for (int y = 0; y < h; y++) std::memcpy(in->staging.data() + (size_t)y * row, sp + y * ss, row);
        ok = f3d_forward_raw(e, fn, in->staging.data(), bytes) == F3D_OK;
      }
      vsapi->freeFrame(fr);
      if (!ok) break;
    }
    if (ok) {
      Span t(kProcess);
      uint8_t* dp = vsapi->getWritePtr(dst, p);
      const ptrdiff_t ds = vsapi->getStride(dst, p);
      if ((size_t)ds == row) {
        ok = f3d_process_raw(e, window.data(), (int)window.size(), dp, bytes) == F3D_OK;
      } else {
        in->staging.resize(bytes);
        ok = f3d_process_raw(e, window.data(), (int)window.size(), in->staging.data(), bytes) == F3D_OK;
        for (int y = 0; ok && y < h; y++) std::memcpy(dp + y * ds, in->staging.data() + (size_t)y * row, row);
      }
    }
    if (!ok) {
      const std::string msg = std::string("FFT3DCL: GPU processing failed at frame ") + std::to_string(n) + ": " +
                              f3d_engine_error(e);
      vsapi->setFilterError(msg.c_str(), ctx);
      vsapi->freeFrame(dst);
      vsapi->freeFrame(src);
      return nullptr;
    }
    if (time_on()) {
      // The readback has completed, so the engine's events are: the last
      // forward (this frame's, when one ran) and this output's kernels.
      float ms[3];
      if (f3d_last_kernel_ms(e, ms) == F3D_OK) {
        if (forwards > 0 && ms[0] >= 0.0f) add_stage(kGpuFwd, (long long)(ms[0] * 1e6));
        if (ms[1] >= 0.0f) add_stage(kGpuFilter, (long long)(ms[1] * 1e6));
        if (ms[2] >= 0.0f) add_stage(kGpuSynth, (long long)(ms[2] * 1e6));
      }
    }
    Span t(kPrune);
    // src/fft3dcl.cpp:457-466. Kalman keeps only the current frame; the
    // reference never prunes there and its cache grows with the clip.
    if (ip.bm >= 2)
      f3d_prune(e, n - ip.current - 1, n - ip.current + ip.bt);
    else if (ip.bm != 0)
      f3d_prune(e, -1, -2);
    else
      f3d_prune(e, n, n);
  }
  vsapi->freeFrame(src);
  return dst;
}

void VS_CC free_filter(void* data, VSCore* core, const VSAPI* vsapi) {
  Instance* in = static_cast<Instance*>(data);
  vsapi->freeNode(in->clip);
  delete in;
  log_usage(core, vsapi, "released");
  dump_stages("FFT3DCL instance released (process totals)");
}

void VS_CC create(const VSMap* inmap, VSMap* out, void*, VSCore* core, const VSAPI* vsapi) {
  int err = 0;
  VSNode* clip = vsapi->mapGetNode(inmap, "clip", 0, &err);
  if (err || !clip) {
    vsapi->mapSetError(out, "FFT3DCL: a video clip must be specified as the 'clip' argument");
    return;
  }
  struct NodeGuard {  // owns the node until createVideoFilter takes it
    const VSAPI* vsapi;
    VSNode* node;
    bool owned = true;
    ~NodeGuard() {
      if (owned && node) vsapi->freeNode(node);
    }
  } guard{vsapi, clip};
  const VSVideoInfo* vi = vsapi->getVideoInfo(clip);
  if (!vsh::isConstantVideoFormat(vi) || (vi->format.numPlanes != 1 && vi->format.numPlanes != 3)) {
    vsapi->mapSetError(out, "FFT3DCL: only constant-format gray, YUV and planar RGB clips are supported");
    return;
  }
  const VSVideoFormat& f = vi->format;
  if (f.sampleType == stFloat && f.bitsPerSample != 32) {
    vsapi->mapSetError(out, "FFT3DCL: only 32-bit float clips supported (16-bit float not ported yet)");
    return;
  }
  if (f.sampleType == stInteger && (f.bitsPerSample < 8 || f.bitsPerSample > 16)) {
    vsapi->mapSetError(out, "FFT3DCL: integer bit depths 8-16 only");
    return;
  }
  auto getF = [&](const char* key, float def) {
    int e = 0;
    double v = vsapi->mapGetFloat(inmap, key, 0, &e);
    return e ? def : (float)v;
  };
  auto getI = [&](const char* key, int64_t def) {
    int e = 0;
    int64_t v = vsapi->mapGetInt(inmap, key, 0, &e);
    return e ? def : v;
  };
  // Argument defaults, src/fft3dcl.cpp:171-198.
  f3d_script_params sp;
  sp.sigma = getF("sigma", 2.0f);
  sp.beta = getF("beta", 1.0f);
  sp.bw = (int)getI("bw", 32);
  sp.bh = (int)getI("bh", 32);
  sp.bt = (int)getI("bt", 3);
  sp.sharpen = getF("sharpen", 0.0f);
  sp.plane = (int)getI("plane", 0);
  sp.mode = (int)getI("mode", 1);
  sp.bordersize = (int)getI("bordersize", 1);
  sp.precision = (int)getI("precision", 0);
  sp.degrid = getF("degrid", sp.mode == 1 ? 1.0f : 0.0f);
  sp.scutoff = getF("scutoff", 0.3f);
  sp.svr = getF("svr", 1.0f);
  sp.smin = getF("smin", 4.0f);
  sp.smax = getF("smax", 20.0f);
  sp.kratio = getF("kratio", 2.0f);
  sp.ow = (int)getI("ow", sp.bw / 2);
  sp.oh = (int)getI("oh", sp.bh / 2);
  sp.wintype = (int)getI("wintype", 0);
  sp.interlaced = (int)getI("interlaced", 0);
  sp.sigma2 = getF("sigma2", sp.sigma);
  sp.sigma3 = getF("sigma3", sp.sigma);
  sp.sigma4 = getF("sigma4", sp.sigma);
  sp.oldfft = (int)getI("oldfft", -1);
  const int device = (int)getI("device", 2);
  if (device == 0) {
    vsapi->mapSetError(out, "FFT3DCL: device=0 (CPU backend) is not available: there is no CPU path; use device=1 or 2");
    return;
  }

  // Plane semantics, src/fft3dcl.cpp:200-225.
  int plane = sp.plane;
  if (f.colorFamily == cfRGB) plane = 4;
  if (f.colorFamily == cfGray) {
    if (plane == 1) {
      vsapi->mapSetError(out, "FFT3DCL: cannot set chroma processing for a greyscale clip");
      return;
    }
    if (plane == 4) plane = 0;
  }
  if (plane == 2 || plane == 3) plane = 1;
  if (plane != 0 && plane != 1 && plane != 4) {
    vsapi->mapSetError(out, "FFT3DCL: plane must be 0 (luma), 1 (chroma) or 4 (all)");
    return;
  }
  auto in = new Instance();
  in->sp = sp;
  in->vi = *vi;
  if (f.colorFamily == cfGray || plane == 0)
    in->planes = {0};
  else if (plane == 1)
    in->planes = {1, 2};
  else
    in->planes = {0, 1, 2};
  f3d_options opts{0, form_from_env(), nullptr};
  for (int p : in->planes) {
    f3d_plane_geom g{vi->width >> (p ? f.subSamplingW : 0), vi->height >> (p ? f.subSamplingH : 0),
                     f.bitsPerSample, f.sampleType, f.colorFamily == cfYUV && p > 0};
    f3d_internal_params ip;
    if (f3d_validate_params(&sp, g.width, g.height, f.bitsPerSample, &ip) != F3D_OK) {
      vsapi->mapSetError(out, f3d_last_error());
      delete in;
      return;
    }
    in->ip = ip;
    f3d_engine* e = nullptr;
    if (f3d_engine_create(&sp, &g, &opts, &e) != F3D_OK) {
      const std::string msg = std::string("FFT3DCL: GPU setup failed: ") + f3d_last_error();
      vsapi->mapSetError(out, msg.c_str());
      delete in;
      return;
    }
    in->engines.push_back(e);
  }
  in->clip = clip;
  VSFilterDependency deps[] = {{clip, rpGeneral}};
  const int fm = sp.bt == 0 ? fmFrameState : fmParallelRequests;
  vsapi->createVideoFilter(out, "FFT3DCL", vi, get_frame, free_filter, fm, deps, 1, in, core);
  guard.owned = false;
  log_usage(core, vsapi, "created");
}

}  // namespace

static const char* const kArgs =
    "clip:vnode;"
    "sigma:float:opt;beta:float:opt;bw:int:opt;bh:int:opt;bt:int:opt;sharpen:float:opt;"
    "plane:int:opt;mode:int:opt;bordersize:int:opt;precision:int:opt;degrid:float:opt;"
    "scutoff:float:opt;svr:float:opt;smin:float:opt;smax:float:opt;kratio:float:opt;"
    "ow:int:opt;oh:int:opt;wintype:int:opt;interlaced:int:opt;sigma2:float:opt;"
    "sigma3:float:opt;sigma4:float:opt;oldfft:int:opt;device:int:opt";

// Plugin entry, src/fft3dcl.cpp:548-552.
VS_EXTERNAL_API(void) VapourSynthPluginInit2(VSPlugin* plugin, const VSPLUGINAPI* vspapi) {
  vspapi->configPlugin("com.github.humbleuser33.fft3dcl", "fft3dcl", "FFT3DCL denoiser (GB300 CUDA)",
                       VS_MAKE_VERSION(1, 1), VAPOURSYNTH_API_VERSION, 0, plugin);
  vspapi->registerFunction("FFT3DCL", kArgs, "clip:vnode;", create, nullptr, plugin);
}
