// f3d_batch_plan.hpp -- host-side planning of the batched tensor-core
// launches: the by-value batch parameters of the forward and of the filter,
// inverse and seam-merge kernels, with each kernel's per-plane prefix of CTA
// (or block-group) counts, the filter's runs of one geometry and its
// shifted-window bits. Plain host code, also compiled by the CPU tests.
#pragma once

#include "f3d_kernels.hpp"

namespace f3d {

// Blocks per tensor-core forward group: one M = 128 tile of blocks x n/2
// packed columns (8 blocks of 32 x 32, 16 of 16 x 16).
constexpr int tc_group_size(int bw) { return 256 / bw; }

// The forward batch parameter of `planes` (false: not one batch).
inline bool forward_batch(const TcFwdArgs* planes, int n, TcFwdBatch& B) {
  if (n < 1 || n > kMaxBatch) return false;
  B = TcFwdBatch{};
  B.n = n;
  for (int i = 0; i < n; i++) {
    const TcFwdArgs& a = planes[i];
    if ((a.g.bw != 16 && a.g.bw != 32) || a.g.bh != a.g.bw || a.g.bw != planes[0].g.bw || a.g.mode != 1 ||
        a.fmt != planes[0].fmt)
      return false;
    B.p[i] = a;
    const int gs = tc_group_size(a.g.bw);
    B.grp0[i + 1] = B.grp0[i] + (a.g.nb + gs - 1) / gs;
  }
  for (int i = n + 1; i <= kMaxBatch; i++) B.grp0[i] = B.grp0[n];
  return true;
}

// The three sweep-side batch parameters (filter, inverse, seam merge) of
// `planes`: the same planes, with the prefix of each kernel's CTA counts.
// tc: the tensor-core sweep (16x16 or 32x32 blocks, tables, operand tiles);
// otherwise the fast form's fused sweep (8x8 to 32x32 blocks; only Bs and Bm
// are used).
inline bool sweep_batches(const SweepArgs* planes, int n, SweepBatch& Bf, SweepBatch& Bs, SweepBatch& Bm,
                          bool tc = true) {
  if (n < 1 || n > kMaxBatch) return false;
  SweepBatch B{};
  B.n = n;
  for (int i = 0; i < n; i++) {
    const SweepArgs& a = planes[i];
    const int bw = a.inv.g.bw;
    const bool size_ok = tc ? (bw == 16 || bw == 32) : (bw == 8 || bw == 16 || bw == 32);
    if (!size_ok || a.inv.g.bh != bw || bw != planes[0].inv.g.bw || (tc && (!a.tab || !a.err || !a.img)) ||
        a.inv.bm != planes[0].inv.bm || a.inv.half != planes[0].inv.half)
      return false;
    B.p[i] = a;
  }
  // Runs of consecutive planes of one geometry (the same group and segment
  // counts). A run of consecutive outputs of one plane is shifted: every
  // window frame but the newest is the previous entry's (the same spectrum
  // buffers). The filter kernel interleaves the CTAs of a run's planes.
  const int nf = B.p[0].inv.bm >= 2 ? B.p[0].inv.bm : 1;
  B.shifted = 0;
  for (int i = 0; i < n; i++) {
    const SweepArgs& a = B.p[i];
    const bool same = i > 0 && a.inv.g.W == B.p[i - 1].inv.g.W && a.inv.g.H == B.p[i - 1].inv.g.H &&
                      a.strips == B.p[i - 1].strips && a.segs == B.p[i - 1].segs;
    B.run[i] = same ? B.run[i - 1] : i;
    B.rlen[i] = 0;
    B.rlen[B.run[i]]++;
    bool shift = same && nf > 1;
    for (int k = 0; k + 1 < nf && shift; k++) shift = a.inv.s[k] == B.p[i - 1].inv.s[k + 1];
    if (shift) B.shifted |= 1 << i;
  }
  auto prefix = [&](SweepBatch& out, auto count) {
    out = B;
    for (int i = 0; i < n; i++) out.cta0[i + 1] = out.cta0[i] + count(out.p[i]);
    for (int i = n + 1; i <= kMaxBatch; i++) out.cta0[i] = out.cta0[n];
  };
  prefix(Bf, [](const SweepArgs& a) { return a.strips * (a.cells_y + 1); });  // (row, strip) groups
  prefix(Bs, [](const SweepArgs& a) { return a.strips * a.segs; });          // (strip, segment)
  prefix(Bm, [](const SweepArgs& a) { return a.segs > 1 ? a.segs - 1 : 0; });  // seams
  return true;
}

// Autotuner choice among n timed launch shapes (fastest[i]: the fastest of
// shape i's runs; shape 0 is the default): the fastest shape, unless the
// default is within `margin` of it (single-step timings vary by about 1 %).
inline int autotune_pick(const float* fastest, int n, float margin = 0.01f) {
  int pick = 0;
  for (int c = 1; c < n; c++)
    if (fastest[c] < fastest[pick]) pick = c;
  return fastest[0] <= (1.0f + margin) * fastest[pick] ? 0 : pick;
}

}  // namespace f3d
