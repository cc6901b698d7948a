// mock_host.cpp -- a minimal VapourSynth API-4 host for testing the plugin's
// registration and argument handling without VapourSynth (test
// infrastructure). It loads the plugin, records configPlugin and
// registerFunction, then calls the registered create function with argument
// maps over synthetic clips and prints one JSON line per case: the error the
// plugin set, or that it created its filter (and, where it did, a checksum of
// the frames it returns).
#include "VapourSynth4.h"

#include <dlfcn.h>

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <map>
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
};
struct VSFrame {
  VSVideoFormat fmt;
  int w[3], h[3];
  ptrdiff_t stride[3];
  std::vector<uint8_t> data[3];
};
struct VSCore {};
struct VSFrameContext {
  std::string err;
};
struct VSPlugin {};

namespace {
std::string g_id, g_ns, g_fname, g_args, g_ret;
VSPublicFunction g_create = nullptr;
VSFilterGetFrame g_getframe = nullptr;
VSFilterFree g_free = nullptr;
void* g_inst = nullptr;
VSNode* g_src = nullptr;

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
void VS_CC freeNode(VSNode*) noexcept {}
void VS_CC createVideoFilter(VSMap* out, const char*, const VSVideoInfo*, VSFilterGetFrame gf, VSFilterFree fr, int,
                             const VSFilterDependency*, int, void* inst, VSCore*) noexcept {
  out->created = true;
  g_getframe = gf;
  g_free = fr;
  g_inst = inst;
}
VSFrame* make_frame(const VSVideoFormat& f, int w, int h) {
  auto* fr = new VSFrame();
  fr->fmt = f;
  for (int p = 0; p < f.numPlanes; p++) {
    fr->w[p] = p ? w >> f.subSamplingW : w;
    fr->h[p] = p ? h >> f.subSamplingH : h;
    fr->stride[p] = (fr->w[p] * f.bytesPerSample + 31) / 32 * 32;
    fr->data[p].assign(fr->stride[p] * fr->h[p], 0);
  }
  return fr;
}
VSFrame* VS_CC newVideoFrame(const VSVideoFormat* f, int w, int h, const VSFrame*, VSCore*) noexcept {
  return make_frame(*f, w, h);
}
void VS_CC freeFrame(const VSFrame* f) noexcept { delete f; }
ptrdiff_t VS_CC getStride(const VSFrame* f, int p) noexcept { return f->stride[p]; }
const uint8_t* VS_CC getReadPtr(const VSFrame* f, int p) noexcept { return f->data[p].data(); }
uint8_t* VS_CC getWritePtr(VSFrame* f, int p) noexcept { return f->data[p].data(); }
const VSVideoFormat* VS_CC getVideoFrameFormat(const VSFrame* f) noexcept { return &f->fmt; }
int VS_CC getFrameWidth(const VSFrame* f, int p) noexcept { return f->w[p]; }
int VS_CC getFrameHeight(const VSFrame* f, int p) noexcept { return f->h[p]; }
// Source frames: a deterministic 8-bit pattern (moving diagonal bands).
const VSFrame* VS_CC getFrameFilter(int n, VSNode* node, VSFrameContext*) noexcept {
  const VSVideoInfo& vi = node->vi;
  n = n < 0 ? 0 : (n >= vi.numFrames ? vi.numFrames - 1 : n);
  VSFrame* f = make_frame(vi.format, vi.width, vi.height);
  for (int p = 0; p < vi.format.numPlanes; p++)
    for (int y = 0; y < f->h[p]; y++)
      for (int x = 0; x < f->w[p]; x++) f->data[p][y * f->stride[p] + x] = (uint8_t)(64 + ((x + y + 3 * n) % 97));
  return f;
}
void VS_CC requestFrameFilter(int, VSNode*, VSFrameContext*) noexcept {}
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
}  // namespace

int main(int argc, char** argv) {
  if (argc < 2) return 2;
  void* h = dlopen(argv[1], RTLD_NOW | RTLD_LOCAL);
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
  VSPlugin plugin;
  init(&plugin, &papi);
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

  // Cases: name, colour family, sample bits, int args, float args.
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
    node.vi.format.colorFamily = c.family;
    node.vi.format.sampleType = stInteger;
    node.vi.format.bitsPerSample = c.bits;
    node.vi.format.bytesPerSample = c.bits <= 8 ? 1 : 2;
    node.vi.format.subSamplingW = c.family == cfYUV ? 1 : 0;
    node.vi.format.subSamplingH = c.family == cfYUV ? 1 : 0;
    node.vi.format.numPlanes = c.family == cfGray ? 1 : 3;
    node.vi.fpsNum = 25;
    node.vi.fpsDen = 1;
    node.vi.width = 96;
    node.vi.height = 64;
    node.vi.numFrames = 6;
    VSMap in, out;
    if (c.clip) in.nodes["clip"] = &node;
    in.ints = c.ints;
    in.floats = c.floats;
    g_src = &node;
    g_getframe = nullptr;
    g_create(&in, &out, nullptr, &core, &api);
    std::printf("{\"case\": \"%s\", \"created\": %s, \"error\": ", c.name, out.created ? "true" : "false");
    json_str(out.error);
    if (out.created && g_getframe) {
      // Request every frame the way VapourSynth does: initial, then all ready.
      uint64_t sum = 0;
      std::string ferr;
      for (int n = 0; n < node.vi.numFrames; n++) {
        VSFrameContext ctx;
        void* fd = nullptr;
        g_getframe(n, arInitial, g_inst, &fd, &ctx, &core, &api);
        const VSFrame* f = g_getframe(n, arAllFramesReady, g_inst, &fd, &ctx, &core, &api);
        if (!f) {
          ferr = ctx.err;
          break;
        }
        for (int p = 0; p < f->fmt.numPlanes; p++)
          for (int y = 0; y < f->h[p]; y++)
            for (int x = 0; x < f->w[p]; x++) sum = sum * 1099511628211ull + f->data[p][y * f->stride[p] + x];
        delete f;
      }
      std::printf(", \"frames_checksum\": %llu, \"frame_error\": ", (unsigned long long)sum);
      json_str(ferr);
      if (g_free) g_free(g_inst, &core, &api);
    }
    std::printf("}\n");
  }
  return 0;
}
