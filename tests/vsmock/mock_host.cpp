// mock_host.cpp -- a minimal VapourSynth API-4 host for testing the plugin
// without VapourSynth (test infrastructure). It loads the plugin, records
// configPlugin and registerFunction, and calls the registered create function
// with argument maps, printing one JSON line per case.
//
//   mock_host <plugin.so>
//       registration, then argument-error cases over synthetic 96x64 clips;
//   mock_host <plugin.so> clip <in.raw> <out.raw> <gray|yuv|rgb> <int|float>
//             <bits> <width> <height> <frames> <forward|reverse|shuffle>
//             [name=value ...]
//       one filter over a clip read from in.raw (frames in order, planes in
//       order, rows packed), its output frames requested the way VapourSynth
//       requests them and written to out.raw in the same layout.
//
// Frame requests follow the API-4 protocol: getFrame(n, arInitial) lets the
// filter request its input frames (requestFrameFilter), then
// getFrame(n, arAllFramesReady) may fetch only those (getFrameFilter). A
// fetch of a frame that was not requested is recorded as a protocol error,
// as is a source frame the filter never frees. Filters created as
// fmFrameState get their frames in order (VapourSynth serialises them); the
// others in the order asked for. Source frames have row strides rounded up to
// 64 bytes, as VapourSynth's frames do, so rows are not packed.
#include "VapourSynth4.h"

#include <dlfcn.h>

#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <set>
#include <string>
#include <vector>

struct VSMap {
  std::map<std::string, int64_t> ints;
  std::map<std::string, double> floats;
  std::map<std::string, VSNode*> nodes;
  std::string error;
  bool created = false;
};
struct VSNode {
  VSVideoInfo vi;
  std::vector<uint8_t>* clip = nullptr;  // packed source frames, or null: a synthetic pattern
};
struct VSFrame {
  VSVideoFormat fmt;
  int w[3], h[3];
  ptrdiff_t stride[3];
  std::vector<uint8_t> data[3];
  bool source = false;
};
struct VSCore {};
struct VSFrameContext {
  std::string err;
  std::set<int> requested;
  std::vector<int> unrequested;
};
struct VSPlugin {};

namespace {
std::string g_id, g_ns, g_fname, g_args, g_ret;
VSPublicFunction g_create = nullptr;
VSFilterGetFrame g_getframe = nullptr;
VSFilterFree g_free = nullptr;
void* g_inst = nullptr;
int g_filter_mode = -1, g_dep_mode = -1, g_num_deps = 0;
int g_frames_alive = 0, g_source_alive = 0, g_nodes_freed = 0;
int (*g_live_engines)() = nullptr;  // the plugin library's f3d_live_instances, when exported

int VS_CC configPlugin(const char* id, const char* ns, const char*, int, int, int, VSPlugin*) noexcept {
  g_id = id;
  g_ns = ns;
  return 1;
}
int VS_CC registerFunction(const char* name, const char* args, const char* ret, VSPublicFunction f, void*,
                           VSPlugin*) noexcept {
  g_fname = name;
  g_args = args;
  g_ret = ret;
  g_create = f;
  return 1;
}
VSNode* VS_CC mapGetNode(const VSMap* m, const char* k, int, int* err) noexcept {
  auto it = m->nodes.find(k);
  if (err) *err = it == m->nodes.end();
  return it == m->nodes.end() ? nullptr : it->second;
}
int64_t VS_CC mapGetInt(const VSMap* m, const char* k, int, int* err) noexcept {
  auto it = m->ints.find(k);
  if (err) *err = it == m->ints.end();
  return it == m->ints.end() ? 0 : it->second;
}
double VS_CC mapGetFloat(const VSMap* m, const char* k, int, int* err) noexcept {
  auto it = m->floats.find(k);
  if (err) *err = it == m->floats.end();
  return it == m->floats.end() ? 0.0 : it->second;
}
void VS_CC mapSetError(VSMap* m, const char* msg) noexcept { m->error = msg; }
const VSVideoInfo* VS_CC getVideoInfo(VSNode* n) noexcept { return &n->vi; }
void VS_CC freeNode(VSNode*) noexcept { g_nodes_freed++; }
void VS_CC createVideoFilter(VSMap* out, const char*, const VSVideoInfo*, VSFilterGetFrame gf, VSFilterFree fr,
                             int mode, const VSFilterDependency* deps, int ndeps, void* inst, VSCore*) noexcept {
  out->created = true;
  g_getframe = gf;
  g_free = fr;
  g_inst = inst;
  g_filter_mode = mode;
  g_num_deps = ndeps;
  g_dep_mode = ndeps > 0 ? deps[0].requestPattern : -1;
}
VSFrame* make_frame(const VSVideoFormat& f, int w, int h) {
  auto* fr = new VSFrame();
  fr->fmt = f;
  for (int p = 0; p < f.numPlanes; p++) {
    fr->w[p] = p ? w >> f.subSamplingW : w;
    fr->h[p] = p ? h >> f.subSamplingH : h;
    fr->stride[p] = (fr->w[p] * f.bytesPerSample + 63) / 64 * 64;
    fr->data[p].assign(fr->stride[p] * fr->h[p], 0);
  }
  g_frames_alive++;
  return fr;
}
VSFrame* VS_CC newVideoFrame(const VSVideoFormat* f, int w, int h, const VSFrame*, VSCore*) noexcept {
  return make_frame(*f, w, h);
}
void VS_CC freeFrame(const VSFrame* f) noexcept {
  if (!f) return;
  g_frames_alive--;
  if (f->source) g_source_alive--;
  delete f;
}
ptrdiff_t VS_CC getStride(const VSFrame* f, int p) noexcept { return f->stride[p]; }
const uint8_t* VS_CC getReadPtr(const VSFrame* f, int p) noexcept { return f->data[p].data(); }
uint8_t* VS_CC getWritePtr(VSFrame* f, int p) noexcept { return f->data[p].data(); }
const VSVideoFormat* VS_CC getVideoFrameFormat(const VSFrame* f) noexcept { return &f->fmt; }
int VS_CC getFrameWidth(const VSFrame* f, int p) noexcept { return f->w[p]; }
int VS_CC getFrameHeight(const VSFrame* f, int p) noexcept { return f->h[p]; }

size_t frame_bytes(const VSVideoInfo& vi) {
  size_t b = 0;
  for (int p = 0; p < vi.format.numPlanes; p++) {
    const int w = p ? vi.width >> vi.format.subSamplingW : vi.width;
    const int h = p ? vi.height >> vi.format.subSamplingH : vi.height;
    b += (size_t)w * h * vi.format.bytesPerSample;
  }
  return b;
}

const VSFrame* VS_CC getFrameFilter(int n, VSNode* node, VSFrameContext* ctx) noexcept {
  const VSVideoInfo& vi = node->vi;
  if (ctx && !ctx->requested.count(n)) ctx->unrequested.push_back(n);
  n = n < 0 ? 0 : (n >= vi.numFrames ? vi.numFrames - 1 : n);
  VSFrame* f = make_frame(vi.format, vi.width, vi.height);
  f->source = true;
  g_source_alive++;
  if (node->clip) {
    const uint8_t* src = node->clip->data() + frame_bytes(vi) * n;
    for (int p = 0; p < vi.format.numPlanes; p++) {
      const size_t row = (size_t)f->w[p] * vi.format.bytesPerSample;
      for (int y = 0; y < f->h[p]; y++) std::memcpy(f->data[p].data() + y * f->stride[p], src + y * row, row);
      src += row * f->h[p];
    }
    return f;
  }
  // Synthetic 8-bit pattern (moving diagonal bands).
  for (int p = 0; p < vi.format.numPlanes; p++)
    for (int y = 0; y < f->h[p]; y++)
      for (int x = 0; x < f->w[p]; x++) f->data[p][y * f->stride[p] + x] = (uint8_t)(64 + ((x + y + 3 * n) % 97));
  return f;
}
void VS_CC requestFrameFilter(int n, VSNode*, VSFrameContext* ctx) noexcept {
  if (ctx) ctx->requested.insert(n);
}
void VS_CC setFilterError(const char* msg, VSFrameContext* ctx) noexcept { ctx->err = msg; }
void VS_CC logMessage(int, const char*, VSCore*) noexcept {}

void json_str(const std::string& s) {
  std::putchar('"');
  for (char c : s) {
    if (c == '"' || c == '\\') std::putchar('\\');
    std::putchar(c);
  }
  std::putchar('"');
}

VSAPI make_api() {
  VSAPI api{};
  api.createVideoFilter = createVideoFilter;
  api.freeNode = freeNode;
  api.getVideoInfo = getVideoInfo;
  api.newVideoFrame = newVideoFrame;
  api.freeFrame = freeFrame;
  api.getStride = getStride;
  api.getReadPtr = getReadPtr;
  api.getWritePtr = getWritePtr;
  api.getVideoFrameFormat = getVideoFrameFormat;
  api.getFrameWidth = getFrameWidth;
  api.getFrameHeight = getFrameHeight;
  api.getFrameFilter = getFrameFilter;
  api.requestFrameFilter = requestFrameFilter;
  api.setFilterError = setFilterError;
  api.mapSetError = mapSetError;
  api.mapGetInt = mapGetInt;
  api.mapGetFloat = mapGetFloat;
  api.mapGetNode = mapGetNode;
  api.logMessage = logMessage;
  return api;
}

void set_format(VSNode& node, int family, int sample_type, int bits) {
  node.vi.format.colorFamily = family;
  node.vi.format.sampleType = sample_type;
  node.vi.format.bitsPerSample = bits;
  node.vi.format.bytesPerSample = sample_type == stFloat ? 4 : (bits <= 8 ? 1 : 2);
  node.vi.format.subSamplingW = family == cfYUV ? 1 : 0;
  node.vi.format.subSamplingH = family == cfYUV ? 1 : 0;
  node.vi.format.numPlanes = family == cfGray ? 1 : 3;
  node.vi.fpsNum = 25;
  node.vi.fpsDen = 1;
}

// Requests output frame n the way VapourSynth does: initial, then all ready.
const VSFrame* request(int n, VSCore& core, const VSAPI& api, std::string* err, std::vector<int>* unrequested) {
  VSFrameContext ctx;
  void* fd = nullptr;
  g_getframe(n, arInitial, g_inst, &fd, &ctx, &core, &api);
  const VSFrame* f = g_getframe(n, arAllFramesReady, g_inst, &fd, &ctx, &core, &api);
  if (!f) *err = ctx.err;
  for (int u : ctx.unrequested) unrequested->push_back(u);
  return f;
}

int register_plugin(const char* path) {
  void* h = dlopen(path, RTLD_NOW | RTLD_LOCAL);
  if (!h) {
    std::printf("{\"case\": \"load\", \"error\": ");
    json_str(dlerror());
    std::printf("}\n");
    return 1;
  }
  using Init = void (*)(VSPlugin*, const VSPLUGINAPI*);
  auto init = reinterpret_cast<Init>(dlsym(h, "VapourSynthPluginInit2"));
  if (!init) return 3;
  VSPLUGINAPI papi{};
  papi.configPlugin = configPlugin;
  papi.registerFunction = registerFunction;
  static VSPlugin plugin;
  init(&plugin, &papi);
  g_live_engines = reinterpret_cast<int (*)()>(dlsym(h, "f3d_live_instances"));
  return 0;
}

int argument_cases() {
  std::printf("{\"case\": \"register\", \"id\": ");
  json_str(g_id);
  std::printf(", \"namespace\": ");
  json_str(g_ns);
  std::printf(", \"function\": ");
  json_str(g_fname);
  std::printf(", \"args\": ");
  json_str(g_args);
  std::printf(", \"returns\": ");
  json_str(g_ret);
  std::printf("}\n");
  VSAPI api = make_api();
  struct Case {
    const char* name;
    int family, bits;
    std::map<std::string, int64_t> ints;
    std::map<std::string, double> floats;
    bool clip = true;
  };
  const Case cases[] = {
      {"no_clip", cfGray, 8, {}, {}, false},
      {"bad_bt", cfGray, 8, {{"bt", 7}}, {}},
      {"bad_bw", cfGray, 8, {{"bw", 0}}, {}},
      {"device0", cfGray, 8, {{"device", 0}}, {}},
      {"gray_chroma", cfGray, 8, {{"plane", 1}}, {}},
      {"bad_plane", cfYUV, 8, {{"plane", 7}}, {}},
      {"bad_bits", cfGray, 6, {}, {}},
      {"valid_gray", cfGray, 8, {{"bt", 3}}, {{"sigma", 2.0}}},
      {"valid_yuv_all", cfYUV, 8, {{"bt", 4}, {"plane", 4}}, {{"sharpen", 0.4}}},
  };
  VSCore core;
  for (const Case& c : cases) {
    VSNode node{};
    set_format(node, c.family, stInteger, c.bits);
    node.vi.width = 96;
    node.vi.height = 64;
    node.vi.numFrames = 6;
    VSMap in, out;
    if (c.clip) in.nodes["clip"] = &node;
    in.ints = c.ints;
    in.floats = c.floats;
    g_getframe = nullptr;
    g_create(&in, &out, nullptr, &core, &api);
    std::printf("{\"case\": \"%s\", \"created\": %s, \"error\": ", c.name, out.created ? "true" : "false");
    json_str(out.error);
    if (out.created && g_getframe) {
      uint64_t sum = 0;
      std::string ferr;
      std::vector<int> unreq;
      for (int n = 0; n < node.vi.numFrames; n++) {
        const VSFrame* f = request(n, core, api, &ferr, &unreq);
        if (!f) break;
        for (int p = 0; p < f->fmt.numPlanes; p++)
          for (int y = 0; y < f->h[p]; y++)
            for (int x = 0; x < f->w[p]; x++) sum = sum * 1099511628211ull + f->data[p][y * f->stride[p] + x];
        freeFrame(f);
      }
      std::printf(", \"frames_checksum\": %llu, \"frame_error\": ", (unsigned long long)sum);
      json_str(ferr);
      if (g_free) g_free(g_inst, &core, &api);
    }
    std::printf("}\n");
  }
  return 0;
}

// Argument types of the plugin's signature.
bool is_int_arg(const std::string& k) {
  static const char* ints[] = {"bw", "bh", "bt", "plane", "mode", "bordersize", "precision", "ow", "oh",
                               "wintype", "interlaced", "oldfft", "device"};
  for (const char* s : ints)
    if (k == s) return true;
  return false;
}

int clip_case(int argc, char** argv) {
  if (argc < 12) return 2;
  const char* in_path = argv[3];
  const char* out_path = argv[4];
  const std::string fam = argv[5], st = argv[6], order = argv[11];
  const int family = fam == "yuv" ? cfYUV : (fam == "rgb" ? cfRGB : cfGray);
  const int sample_type = st == "float" ? stFloat : stInteger;
  VSNode node{};
  set_format(node, family, sample_type, std::atoi(argv[7]));
  node.vi.width = std::atoi(argv[8]);
  node.vi.height = std::atoi(argv[9]);
  node.vi.numFrames = std::atoi(argv[10]);
  std::vector<uint8_t> clip(frame_bytes(node.vi) * node.vi.numFrames);
  FILE* fi = std::fopen(in_path, "rb");
  if (!fi || std::fread(clip.data(), 1, clip.size(), fi) != clip.size()) return 4;
  std::fclose(fi);
  node.clip = &clip;
  VSMap in, out;
  in.nodes["clip"] = &node;
  for (int i = 12; i < argc; i++) {
    const std::string kv = argv[i];
    const size_t eq = kv.find('=');
    if (eq == std::string::npos) return 2;
    const std::string k = kv.substr(0, eq), v = kv.substr(eq + 1);
    if (is_int_arg(k)) in.ints[k] = std::atoll(v.c_str());
    else in.floats[k] = std::atof(v.c_str());
  }
  VSAPI api = make_api();
  VSCore core;
  g_create(&in, &out, nullptr, &core, &api);
  std::printf("{\"case\": \"clip\", \"created\": %s, \"error\": ", out.created ? "true" : "false");
  json_str(out.error);
  if (!out.created || !g_getframe) {
    std::printf("}\n");
    return 0;
  }
  const int nf = node.vi.numFrames;
  std::vector<int> seq(nf);
  for (int i = 0; i < nf; i++) seq[i] = i;
  // VapourSynth runs fmFrameState filters one frame at a time, in order.
  const bool in_order = g_filter_mode == fmFrameState;
  if (!in_order && order == "reverse") std::reverse(seq.begin(), seq.end());
  if (!in_order && order == "shuffle") {
    uint64_t s = 0x9E3779B97F4A7C15ull;
    for (int i = nf - 1; i > 0; i--) {
      s = s * 6364136223846793005ull + 1442695040888963407ull;
      std::swap(seq[i], seq[(int)((s >> 33) % (uint64_t)(i + 1))]);
    }
  }
  std::vector<uint8_t> res(clip.size(), 0);
  std::string ferr;
  std::vector<int> unreq;
  int done = 0;
  for (int n : seq) {
    const VSFrame* f = request(n, core, api, &ferr, &unreq);
    if (!f) break;
    uint8_t* dst = res.data() + frame_bytes(node.vi) * n;
    for (int p = 0; p < f->fmt.numPlanes; p++) {
      const size_t row = (size_t)f->w[p] * f->fmt.bytesPerSample;
      for (int y = 0; y < f->h[p]; y++) std::memcpy(dst + y * row, f->data[p].data() + y * f->stride[p], row);
      dst += row * f->h[p];
    }
    freeFrame(f);
    done++;
  }
  const int source_left = g_source_alive;
  if (g_free) g_free(g_inst, &core, &api);
  FILE* fo = std::fopen(out_path, "wb");
  if (!fo || std::fwrite(res.data(), 1, res.size(), fo) != res.size()) return 5;
  std::fclose(fo);
  std::printf(", \"frames_done\": %d, \"frame_error\": ", done);
  json_str(ferr);
  std::printf(", \"filter_mode\": \"%s\", \"dependency\": \"%s\", \"deps\": %d, \"unrequested\": [",
              g_filter_mode == fmFrameState ? "fmFrameState"
              : g_filter_mode == fmParallelRequests ? "fmParallelRequests"
                                                  : "other",
              g_dep_mode == rpGeneral ? "rpGeneral" : "other", g_num_deps);
  for (size_t i = 0; i < unreq.size(); i++) std::printf("%s%d", i ? ", " : "", unreq[i]);
  std::printf("], \"source_frames_not_freed\": %d, \"frames_alive\": %d, \"nodes_freed\": %d, "
              "\"live_engines_after_free\": %d}\n",
              source_left, g_frames_alive, g_nodes_freed, g_live_engines ? g_live_engines() : -1);
  return 0;
}
}  // namespace

int main(int argc, char** argv) {
  if (argc < 2) return 2;
  const int rc = register_plugin(argv[1]);
  if (rc) return rc;
  if (argc >= 3 && std::strcmp(argv[2], "clip") == 0) return clip_case(argc, argv);
  return argument_cases();
}
