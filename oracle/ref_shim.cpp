// ref_shim.cpp -- C entry points over the reference's own CPU backend.
//
// TEST INFRASTRUCTURE ONLY. Compiled by oracle/Makefile together with the
// reference's unmodified sources (src/cpu/fft.cpp, src/cpu/tables.cpp,
// src/cpu/reference.cpp, src/params.h) where they lie, into oracle/_ref/. It
// exists to pin the C oracle (fft3d_oracle.c) to the reference bit for bit and
// to generate the golden vectors under tests/golden/. Nothing here is shipped.
//
// The clip driver below follows the CPU branch of the reference plugin's frame
// callback (src/fft3dcl.cpp:471-521): clamped temporal window, spectra cache
// pruned to [n-current-1, n-current+bt], filterAndSynthesize, download.
#include "params.h"
#include "reference.h"

#include <cstdint>
#include <cstring>
#include <map>
#include <memory>
#include <vector>

using namespace fft3dcl;

extern "C" {

// Field order matches orc_script_params in fft3d_oracle.h.
struct ref_script_params {
  float sigma, beta;
  int bw, bh, bt;
  float sharpen;
  int plane, mode, bordersize, precision;
  float degrid, scutoff, svr, smin, smax, kratio;
  int ow, oh, wintype, interlaced;
  float sigma2, sigma3, sigma4;
  int oldfft;
};

static ScriptParams to_sp(const ref_script_params* s) {
  ScriptParams sp;
  sp.sigma = s->sigma;
  sp.beta = s->beta;
  sp.bw = s->bw;
  sp.bh = s->bh;
  sp.bt = s->bt;
  sp.sharpen = s->sharpen;
  sp.plane = s->plane;
  sp.mode = s->mode;
  sp.bordersize = s->bordersize;
  sp.precision = s->precision;
  sp.degrid = s->degrid;
  sp.scutoff = s->scutoff;
  sp.svr = s->svr;
  sp.smin = s->smin;
  sp.smax = s->smax;
  sp.kratio = s->kratio;
  sp.ow = s->ow;
  sp.oh = s->oh;
  sp.wintype = s->wintype;
  sp.interlaced = s->interlaced;
  sp.sigma2 = s->sigma2;
  sp.sigma3 = s->sigma3;
  sp.sigma4 = s->sigma4;
  sp.oldfft = s->oldfft;
  return sp;
}

// Validated parameters as 36 numbers, in the order of orc_internal_params.
int ref_validate(const ref_script_params* s, int width, int height, int bits, double* vals,
                 const char** err) {
  ScriptParams sp = to_sp(s);
  InternalParams ip;
  if (!validateParams(sp, width, height, bits, ip, err)) return 0;
  double v[] = {ip.sigma,     ip.beta,     (double)ip.bw, (double)ip.bh, (double)ip.bm,
                (double)ip.bt, ip.sharpen, (double)ip.sharpenOn, (double)ip.mode,
                (double)ip.bordersize, (double)ip.precision, ip.degrid, (double)ip.degridOn,
                ip.scutoff,   ip.svr,      ip.smin,       ip.smax,       ip.kratio,
                (double)ip.ow, (double)ip.oh, (double)ip.wintype, (double)ip.interlaced,
                ip.sigma2,    ip.sigma3,   ip.sigma4,     (double)ip.usePattern,
                (double)ip.current, (double)ip.nx, (double)ip.ny, (double)ip.totw,
                (double)ip.toth, (double)ip.oldfft, ip.wienerS, ip.betaX, ip.kalmanCN,
                ip.ssmin,     ip.ssmax};
  std::memcpy(vals, v, sizeof(v));
  return 1;
}

void ref_fft1d(int n, const float* in, float* out, int inverse) {
  FftPlan p(n);
  const auto* a = reinterpret_cast<const std::complex<float>*>(in);
  auto* b = reinterpret_cast<std::complex<float>*>(out);
  if (inverse)
    p.inverse(a, b);
  else
    p.forward(a, b);
}

// Tables of one plane: 0 winAna, 1 winSynA, 2 winSynB, 3 pattern, 4 sharpen,
// 5 gsRe, 6 gsIm (first block only). Returns the element count.
int ref_get_table(const ref_script_params* s, int width, int height, int bits, int sampleType,
                  int chroma, int which, float* dst) {
  ScriptParams sp = to_sp(s);
  InternalParams ip;
  const char* e = nullptr;
  if (!validateParams(sp, width, height, bits, ip, &e)) return -1;
  PlaneGeom g{width, height, bits, sampleType, chroma != 0};
  PlaneRef ref(ip, g);
  if (which >= 5) ref.buildDegridSample();
  const std::vector<float>* t = nullptr;
  size_t n = 0;
  switch (which) {
  case 0: t = &ref.winAna(); n = t->size(); break;
  case 1: t = &ref.winSynA(); n = t->size(); break;
  case 2: t = &ref.winSynB(); n = t->size(); break;
  case 3: t = &ref.pattern(); n = t->size(); break;
  case 4: t = &ref.sharpenLut(); n = t->size(); break;
  case 5: t = &ref.gsRe(); n = (size_t)ref.fbw() * ip.bh; break;
  case 6: t = &ref.gsIm(); n = (size_t)ref.fbw() * ip.bh; break;
  default: return -1;
  }
  if (dst && n) std::memcpy(dst, t->data(), n * sizeof(float));
  return (int)n;
}

// Forward spectra of one float plane (re, im: nblocks*fbw*bh each).
int ref_spectra(const ref_script_params* s, int width, int height, int bits, int sampleType,
                int chroma, const float* plane, float* re, float* im) {
  ScriptParams sp = to_sp(s);
  InternalParams ip;
  const char* e = nullptr;
  if (!validateParams(sp, width, height, bits, ip, &e)) return -1;
  PlaneGeom g{width, height, bits, sampleType, chroma != 0};
  PlaneRef ref(ip, g);
  std::vector<float> pl(plane, plane + (size_t)width * height);
  auto sp2 = ref.computeSpectra(pl);
  std::memcpy(re, sp2->re.data(), sp2->re.size() * sizeof(float));
  std::memcpy(im, sp2->im.data(), sp2->im.size() * sizeof(float));
  return (int)sp2->re.size();
}

static int clampFrame(int n, int num) { return n < 0 ? 0 : (n > num - 1 ? num - 1 : n); }

// Output frames first..first+count-1 of one plane through the reference's
// PlaneRef, following the CPU path of src/fft3dcl.cpp:471-521.
int ref_run_clip(const ref_script_params* s, int width, int height, int bits, int sampleType,
                 int chroma, int nframes, const uint8_t* const* frames, ptrdiff_t pitch,
                 int first, int count, uint8_t* const* out, ptrdiff_t opitch, const char** err) {
  ScriptParams sp = to_sp(s);
  InternalParams ip;
  if (!validateParams(sp, width, height, bits, ip, err)) return -1;
  PlaneGeom g{width, height, bits, sampleType, chroma != 0};
  PlaneRef ref(ip, g);
  if (ip.degridOn) ref.buildDegridSample();
  std::map<int, std::shared_ptr<PlaneRef::Spectra>> cache;
  std::vector<float> planeBuf, outBuf;
  int start = ip.bm == 0 ? 0 : first;
  for (int n = start; n < first + count; n++) {
    auto getSpectra = [&](int fn) {
      fn = clampFrame(fn, nframes);
      auto it = cache.find(fn);
      if (it != cache.end()) return it->second;
      planeBuf.clear();
      ref.upload(frames[fn], pitch, planeBuf);
      auto sp3 = ref.computeSpectra(planeBuf);
      cache[fn] = sp3;
      return sp3;
    };
    std::vector<std::shared_ptr<PlaneRef::Spectra>> window;
    if (ip.bm >= 2) {
      for (int i = 0; i < ip.bt; i++) window.push_back(getSpectra(n - ip.current + i));
    } else {
      window.push_back(getSpectra(n));
    }
    outBuf.clear();
    ref.filterAndSynthesize(window, outBuf);
    if (n >= first) ref.download(outBuf, out[n - first], opitch);
    if (ip.bm >= 2) {
      int lo = n - ip.current - 1, hi = n - ip.current + ip.bt;
      for (auto it = cache.begin(); it != cache.end();)
        it = (it->first < lo || it->first > hi) ? cache.erase(it) : std::next(it);
    } else if (ip.bm != 0 && !cache.empty()) {
      cache.clear();
    }
  }
  return 0;
}

} // extern "C"
