// Host-side checks of the batched launch plan (tensor-core and fast forms,
// fft3dcl_gb300/csrc/f3d_batch_plan.hpp): per-plane CTA prefixes, the
// filter's runs of one geometry and its shifted-window bits, the batches
// the plan refuses, and the autotuner's choice. Built and run by
// tests/test_batch_plan_cpu.py; prints "ok" or the first failed check.
#include "f3d_batch_plan.hpp"

#include <cstdio>
#include <cstdlib>
#include <vector>

using namespace f3d;

static int g_fail = 0;
#define CHECK(c)                                                    \
  do {                                                              \
    if (!(c)) {                                                     \
      std::printf("FAILED line %d: %s\n", __LINE__, #c);            \
      g_fail = 1;                                                   \
    }                                                               \
  } while (0)

// Stand-in device addresses: the plan only compares and copies pointers.
static float2* spec(int frame, int plane) {
  return reinterpret_cast<float2*>(static_cast<uintptr_t>(0x100000u + 0x1000u * (16 * plane + frame)));
}
static uint8_t* fake(uintptr_t v) { return reinterpret_cast<uint8_t*>(v); }

// A plane of size w x h (32x32 blocks, half overlap), output of frame n of
// plane p with the window of bm frames, n - cur .. .
static SweepArgs plane(int w, int h, int p, int n, int bm, int cur) {
  SweepArgs a{};
  a.inv.g.W = w;
  a.inv.g.H = h;
  a.inv.g.bw = a.inv.g.bh = 32;
  a.inv.g.mode = 1;
  a.inv.bm = bm;
  const int nf = bm >= 2 ? bm : 1;
  for (int k = 0; k < nf; k++) a.inv.s[k] = spec(n - cur + k + 8, p);
  a.cells_x = (w + 15) / 16;
  a.cells_y = (h + 15) / 16;
  a.strips = (a.cells_x + 6) / 7;
  a.segs = 1 + a.cells_y / 10;
  a.tab = fake(0x10);
  a.err = reinterpret_cast<int*>(fake(0x20));
  a.img = fake(0x30 + 0x100 * (16 * p + n));
  return a;
}

static int groups(const SweepArgs& a) { return a.strips * (a.cells_y + 1); }

int main() {
  SweepBatch Bf, Bs, Bm;
  // Ten consecutive outputs of one 4K plane (bt = 4): one run, every entry
  // after the first shifted.
  {
    std::vector<SweepArgs> v;
    for (int n = 0; n < 10; n++) v.push_back(plane(3840, 2160, 0, n, 4, 2));
    CHECK(sweep_batches(v.data(), 10, Bf, Bs, Bm));
    CHECK(Bf.rlen[0] == 10);
    for (int i = 0; i < 10; i++) {
      CHECK(Bf.run[i] == 0);
      CHECK(Bf.cta0[i] == i * groups(v[0]));
      CHECK(Bs.cta0[i] == i * v[0].strips * v[0].segs);
      CHECK(Bm.cta0[i] == i * (v[0].segs - 1));
    }
    CHECK(Bf.shifted == 0x3FE);
    for (int i = 10; i <= kMaxBatch; i++) CHECK(Bf.cta0[i] == 10 * groups(v[0]));
  }
  // Two YUV 4:2:0 frames by plane, [Y, Y, U, U, V, V]: a luma run and a
  // chroma run of four; each second output of a plane is shifted, V0 (after
  // U1, another plane's buffers) is not.
  {
    std::vector<SweepArgs> v = {plane(1920, 1080, 0, 5, 4, 2), plane(1920, 1080, 0, 6, 4, 2),
                                plane(960, 540, 1, 5, 4, 2),   plane(960, 540, 1, 6, 4, 2),
                                plane(960, 540, 2, 5, 4, 2),   plane(960, 540, 2, 6, 4, 2)};
    CHECK(sweep_batches(v.data(), 6, Bf, Bs, Bm));
    const int run[6] = {0, 0, 2, 2, 2, 2};
    for (int i = 0; i < 6; i++) CHECK(Bf.run[i] == run[i]);
    CHECK(Bf.rlen[0] == 2 && Bf.rlen[2] == 4);
    CHECK(Bf.shifted == ((1 << 1) | (1 << 3) | (1 << 5)));
    CHECK(Bf.cta0[2] == 2 * groups(v[0]));
    CHECK(Bf.cta0[6] == 2 * groups(v[0]) + 4 * groups(v[2]));
  }
  // The same frames by frame, [Y, U, V, Y, U, V]: the chroma pairs are runs,
  // nothing is shifted.
  {
    std::vector<SweepArgs> v = {plane(1920, 1080, 0, 5, 4, 2), plane(960, 540, 1, 5, 4, 2),
                                plane(960, 540, 2, 5, 4, 2),   plane(1920, 1080, 0, 6, 4, 2),
                                plane(960, 540, 1, 6, 4, 2),   plane(960, 540, 2, 6, 4, 2)};
    CHECK(sweep_batches(v.data(), 6, Bf, Bs, Bm));
    const int run[6] = {0, 1, 1, 3, 4, 4};
    for (int i = 0; i < 6; i++) CHECK(Bf.run[i] == run[i]);
    CHECK(Bf.rlen[0] == 1 && Bf.rlen[1] == 2 && Bf.rlen[3] == 1 && Bf.rlen[4] == 2);
    CHECK(Bf.shifted == 0);
  }
  // One window frame (bt = 1): consecutive outputs share nothing.
  {
    std::vector<SweepArgs> v = {plane(640, 360, 0, 0, 1, 0), plane(640, 360, 0, 1, 1, 0)};
    CHECK(sweep_batches(v.data(), 2, Bf, Bs, Bm));
    CHECK(Bf.rlen[0] == 2 && Bf.shifted == 0);
  }
  // Windows that are not one frame apart are not shifted.
  {
    std::vector<SweepArgs> v = {plane(640, 360, 0, 0, 3, 1), plane(640, 360, 0, 2, 3, 1)};
    CHECK(sweep_batches(v.data(), 2, Bf, Bs, Bm));
    CHECK(Bf.rlen[0] == 2 && Bf.shifted == 0);
  }
  // Refused: no planes, more than kMaxBatch, mixed temporal modes, another
  // block size, a plane without its operand tiles.
  {
    std::vector<SweepArgs> v(kMaxBatch + 1, plane(640, 360, 0, 0, 3, 1));
    CHECK(!sweep_batches(v.data(), 0, Bf, Bs, Bm));
    CHECK(sweep_batches(v.data(), kMaxBatch, Bf, Bs, Bm));
    CHECK(!sweep_batches(v.data(), kMaxBatch + 1, Bf, Bs, Bm));
    std::vector<SweepArgs> m = {plane(640, 360, 0, 0, 3, 1), plane(640, 360, 1, 0, 2, 1)};
    CHECK(!sweep_batches(m.data(), 2, Bf, Bs, Bm));
    m[1] = plane(640, 360, 1, 0, 3, 1);
    m[1].inv.g.bw = 16;
    CHECK(!sweep_batches(m.data(), 2, Bf, Bs, Bm));
    m[1] = plane(640, 360, 1, 0, 3, 1);
    m[1].img = nullptr;
    CHECK(!sweep_batches(m.data(), 2, Bf, Bs, Bm));
  }
  // The fast form's sweep plan: no tables or operand tiles needed, 8x8 to
  // 32x32 blocks; the same prefixes and runs.
  {
    std::vector<SweepArgs> v;
    for (int n = 0; n < 4; n++) {
      SweepArgs a = plane(1920, 1080, 0, n, 4, 2);
      a.tab = nullptr;
      a.err = nullptr;
      a.img = nullptr;
      v.push_back(a);
    }
    CHECK(!sweep_batches(v.data(), 4, Bf, Bs, Bm));  // the tensor-core plan needs them
    CHECK(sweep_batches(v.data(), 4, Bf, Bs, Bm, false));
    CHECK(Bs.rlen[0] == 4 && Bs.shifted == 0xE);
    for (int i = 0; i <= 4; i++) CHECK(Bs.cta0[i] == i * v[0].strips * v[0].segs);
    for (auto& a : v) a.inv.g.bw = a.inv.g.bh = 8;
    CHECK(sweep_batches(v.data(), 4, Bf, Bs, Bm, false));
    CHECK(!sweep_batches(v.data(), 4, Bf, Bs, Bm));  // no 8x8 tensor-core sweep
    v[1].inv.g.bw = v[1].inv.g.bh = 16;
    CHECK(!sweep_batches(v.data(), 4, Bf, Bs, Bm, false));  // one block size per batch
    v[1].inv.g.bw = v[1].inv.g.bh = 64;
    CHECK(!sweep_batches(v.data(), 2, Bf, Bs, Bm, false));  // 64x64: no fused fast sweep
  }
  // Forward: block-group prefix, one group per 8 blocks of 32 x 32 (16 of
  // 16 x 16); the planes of a batch share the block size.
  {
    TcFwdArgs f[3] = {};
    const int nb[3] = {32912, 8540, 2232};
    for (int i = 0; i < 3; i++) {
      f[i].g.bw = f[i].g.bh = 32;
      f[i].g.mode = 1;
      f[i].g.nb = nb[i];
      f[i].fmt = FMT_U16;
    }
    TcFwdBatch B;
    CHECK(forward_batch(f, 3, B));
    CHECK(B.grp0[1] == 4114 && B.grp0[2] == 4114 + 1068 && B.grp0[3] == 4114 + 1068 + 279);
    CHECK(B.grp0[kMaxBatch] == B.grp0[3]);
    f[2].fmt = FMT_U8;
    CHECK(!forward_batch(f, 3, B));
    f[2].fmt = FMT_U16;
    f[2].g.bw = f[2].g.bh = 16;
    CHECK(!forward_batch(f, 3, B));
    for (int i = 0; i < 3; i++) f[i].g.bw = f[i].g.bh = 16;
    CHECK(forward_batch(f, 3, B));
    CHECK(B.grp0[1] == 2057 && B.grp0[2] == 2057 + 534 && B.grp0[3] == 2057 + 534 + 140);
  }
  // Autotuner: the default shape (index 0) unless another is over 1 % faster.
  {
    const float same[3] = {1.0f, 1.0f, 1.0f}, close[3] = {1.0f, 0.995f, 1.2f}, clear[3] = {1.0f, 1.1f, 0.97f};
    CHECK(autotune_pick(same, 3) == 0);
    CHECK(autotune_pick(close, 3) == 0);
    CHECK(autotune_pick(clear, 3) == 2);
  }
  if (!g_fail) std::printf("ok\n");
  return g_fail;
}
