#!/usr/bin/env python
"""Throughput of the FFT3D block-FFT denoise path on GB300.

Workload: 3840x2160 10-bit luma, sigma=3 bt=4 bw=bh=32 ow=oh=16 sharpen=0.4
precision=2, a seeded synthetic 48-frame clip (ramp + moving rectangles in
64..940, Gaussian noise 12 LSB). One step of the tensor-core headline is one
batch step of --outputs-per-step (default 10) consecutive output frames in
steady state: the forward transforms of the frames that enter the temporal
window, then filter + inverse + overlap-add + 10-bit packing of each output.
The other forms run one output frame per step.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--form exact|fast|tc]
    python bench.py --impl reference ...   # the reference CPU path on the host cores

Prints one JSON line (rank 0). `value` is device throughput with the clip
resident in HBM; `e2e` is the same metric through the C ABI with host
buffers (host->device upload of the new frame and device->host readback of
the output inside the timed region). For N > 1 each rank runs an independent
replica on its own GPU (the path does not shard across GPUs).
"""
from __future__ import annotations

import argparse
import gc
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "4K 10-bit frames/s (bt=4,bw=32) plain vs batched-TC; p99 frame latency @16 streams"
UNIT = "frames/s"
W, H, BITS, NFRAMES = 3840, 2160, 10, 48
PARAMS = dict(sigma=3.0, bt=4, bw=32, bh=32, ow=16, oh=16, sharpen=0.4, precision=2)
WORKLOAD = ("3840x2160 YUV420P10 luma, sigma=3 bt=4 bw=bh=32 ow=oh=16 sharpen=0.4 precision=2, "
            "48-frame seeded clip, one output frame per step")

# dram__bytes_read.sum + dram__bytes_write.sum per launch of the dominant
# kernel from one ncu capture of this workload (launch list of
# `bench.py --steps 2 --warmup 3`), keyed by form; None until captured.
NCU_TRAFFIC = {"tc": 571806464 + 130638592}
# The same for the filter launch of a batch step of k consecutive outputs
# (k -> bytes): captured on the 1920x1080 case of this workload (`--size
# 1920x1080 --steps 1 --warmup 3 --no-cpu --serve-streams 0 --no-yuv
# --compare tc --outputs-per-step k`, mean of the k-output launches; k=4:
# 260.2 MB read + 124.4 MB written, k=8: 410.5 + 286.0 MB, k=10 (with the
# filter's current column mapping): 490.3 + 366.7 MB) and scaled to
# 3840x2160 by the block count (32912 / 8540).
NCU_TRAFFIC_BATCH = {4: 1002927925 + 479516689, 8: 1581975962 + 1102231724, 10: 1889588860 + 1413116250}
# Consecutive outputs per batch step of the tensor-core headline (4K sweeps:
# ten beat eight and twelve); its traffic must be in NCU_TRAFFIC_BATCH.
DEFAULT_OUTPUTS_PER_STEP = 10


# Arithmetic of each form's block transforms: the tensor-core form contracts
# fp16 hi/lo operand parts (hi*hi + hi*lo + lo*hi) with fp32 accumulation;
# the filter and everything outside the contractions is fp32.
DTYPE_OF_FORM = {"exact": "f32", "fast": "f32",
                 "tc": "f16 hi/lo split operands (3 products), f32 accumulate; f32 filter"}


def algorithmic_bytes(nb: int, fbw: int, bh: int, bt: int) -> dict:
    """Bytes one output frame must move with resident spectra: the raw plane
    in, the packed plane out, the new frame's spectrum written once and the
    bt window spectra read once. Intermediates (filtered spectra, inverse
    blocks) do not count."""
    plane = W * H * 2
    spec = nb * fbw * bh * 8
    return {"plane": plane, "spectrum": spec, "frame": 2 * plane + spec * (1 + bt),
            "filter_inverse": spec * bt}


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class Clocks:
    """nvidia-smi samples every 200 ms while the timed region runs."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits", "-lms", "200",
                 "-i", str(self.device)], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        time.sleep(0.3)

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.3)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for name, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(smax) if smax else None, "reasons": sorted(reasons),
                "samples": len(sm)}


def make_clip(nframes: int = NFRAMES):
    from fft3dcl_gb300 import synth
    return synth.clip_yuv420p10_luma(W, H, nframes)


# --------------------------------------------------------------- CPU leg --

def cpu_steady_state(frames, threads: int, budget_s: float, max_steps: int, min_steps: int = 1,
                     bits: int = BITS, params: dict | None = None, chroma: bool = False):
    """Oracle (the C restatement of the reference CPU backend) in steady
    state: per step one new frame is uploaded and transformed, then the
    window is filtered, inverted, overlap-added and downloaded (Kalman:
    the state carries over from step to step). Returns (frames/s, steps)."""
    import ctypes as C
    import oracle
    params = PARAMS if params is None else params
    L = oracle.lib()
    h, w = frames[0].shape
    st = 1 if frames[0].dtype == np.float32 else 0
    pl = oracle.Plane(w, h, bits, st, chroma=chroma, **params)
    pl.build_degrid()
    n = pl.nb * pl.fbw * pl.ip.bh
    bm = pl.ip.bm
    bt = pl.ip.bt if bm >= 2 else 1
    cur = pl.ip.current if bm >= 2 else 0
    slots = [(np.empty(n, np.float32), np.empty(n, np.float32)) for _ in range(bt + 1)]
    plane = np.empty((h, w), np.float32)
    out = np.empty((h, w), np.float32)
    dst = np.empty((h, w), frames[0].dtype)

    def spectra(fn, slot):
        f = frames[fn % len(frames)]
        L.orc_upload(pl.h, oracle._ptr(f), f.strides[0], oracle._ptr(plane))
        L.orc_compute_spectra(pl.h, oracle._ptr(plane), oracle._ptr(slot[0]), oracle._ptr(slot[1]), threads)

    def step(nout):
        # window of output frame nout: nout-cur .. nout-cur+bt-1; the last is new
        new = nout - cur + bt - 1
        spectra(new, slots[new % (bt + 1)])
        win = [slots[(nout - cur + i) % (bt + 1)] for i in range(bt)]
        wr = (C.c_void_p * bt)(*[x[0].ctypes.data for x in win])
        wi = (C.c_void_p * bt)(*[x[1].ctypes.data for x in win])
        L.orc_filter_and_synthesize(pl.h, wr, wi, bt, oracle._ptr(out), threads)
        L.orc_download(pl.h, oracle._ptr(out), oracle._ptr(dst), dst.strides[0])

    base = cur + 10
    for i in range(bt - 1):  # window warm-up, untimed
        spectra(base - cur + i, slots[(base - cur + i) % (bt + 1)])
    t0 = time.perf_counter()
    steps = 0
    while steps < max_steps and (steps < min_steps or time.perf_counter() - t0 < budget_s):
        step(base + steps)
        steps += 1
    dt = time.perf_counter() - t0
    return steps / dt, steps


# The two other single-plane workloads: the plain method on 640x360 GRAY8
# and Kalman on 1280x720 float with the sigma pattern and scene cuts.
GRAY8_PARAMS = dict(sigma=2.0, beta=1.0, bt=3, bw=32, bh=32, ow=16, oh=16, degrid=1.0, sharpen=0.0)
KALMAN_PARAMS = dict(bt=0, kratio=2.0, bw=64, bh=64, ow=32, oh=32, sigma=2.0, sigma2=1.5, sigma3=2.5, sigma4=3.0)
# Algorithmic bytes per output frame with resident spectra: 640x360 GRAY8
# bt=3: 2 x 230,400 + 4,386,816 x (1 + 3); 720p float Kalman: 2 x 3,686,400
# + 2 x 16 B of state x 2,128,896 bins.
AB_GRAY8 = 2 * 640 * 360 + 1008 * 17 * 32 * 8 * 4
AB_KALMAN = 2 * 1280 * 720 * 4 + 2 * 16 * 1008 * 33 * 64
# 1920x1080 YUV420P8 bt=4, all planes: luma 2 x 2,073,600 + 37,167,360 x
# (1 + 4), each chroma plane 2 x 518,400 + 9,713,664 x (1 + 4).
AB_YUV1080 = 2 * 1920 * 1080 + 8540 * 17 * 32 * 8 * 5 + 2 * (2 * 960 * 540 + 2232 * 17 * 32 * 8 * 5)


def config_section(args, dev, local_rank, frames, bits, params, forms, ab_bytes, peak, kbatch=1):
    """Device throughput of one single-plane workload in steady state with the
    clip resident in HBM (engine calls per output; for the tensor-core form
    also batch steps of kbatch consecutive outputs, CUDA graph), its step
    roofline on algorithmic bytes, and the oracle on the host's threads over
    a bounded sample."""
    import torch
    import fft3dcl_gb300 as F
    h, w = frames[0].shape
    st = 1 if frames[0].dtype == np.float32 else 0
    bps = frames[0].itemsize
    clip = torch.from_numpy(np.stack(frames)).to(dev)
    nfr = clip.shape[0]
    ip = F.validate(w, h, bits, **params)
    bm = ip.bm
    need = ip.bt if bm >= 2 else 1
    cur = ip.current if bm >= 2 else 0
    pitch = w * bps
    res = {}
    for form, k in [(f, 1) for f in forms] + ([("tc", kbatch)] if kbatch > 1 and "tc" in forms else []):
        stream = torch.cuda.Stream(device=dev)
        eng = F.Engine(w, h, bits, st, form=form, device=local_rank, stream=stream.cuda_stream, **params)
        outs = [torch.empty((h, w), dtype=clip.dtype, device=dev) for _ in range(k)]
        batch = F.Batch([eng] * k, graph=True, autotune=True) if k > 1 else None

        def step(n):
            wins = [[m - cur + i for i in range(need)] for m in range(n, n + k)]
            for wnd in wins:  # only the first step finds frames missing
                for fn in wnd:
                    if not eng.has(fn):
                        eng.forward_device(fn, clip[fn % nfr].data_ptr(), pitch)
            if batch is None:
                eng.process_device(wins[0], outs[0].data_ptr(), pitch)
            else:
                # The frames the next step's windows add, forwarded in this
                # step concurrently with its outputs.
                ahead = [n + k - 1 - cur + need + i for i in range(k)]
                batch.step(ahead, [clip[a % nfr].data_ptr() for a in ahead], [pitch] * k, wins,
                           [o.data_ptr() for o in outs], [pitch] * k)
            if bm == 0:  # Kalman keeps only the current frame
                eng.prune(n + k - 1, n + k - 1)
            else:
                eng.prune(n - cur - 1, n + 2 * k - 1 - cur + need)

        n = max(cur, 1)
        # Batches: the autotuner's step and the graph capture come first.
        for _ in range(max(3 if batch is None else 6, args.warmup)):
            step(n)
            n += k
        torch.cuda.synchronize(dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            step(n)
            n += k
        e1.record(stream)
        torch.cuda.synchronize(dev)
        fps = args.steps * k / (e0.elapsed_time(e1) / 1000.0)
        info = eng.info()
        key = form if k == 1 else f"{form}_batch{k}"
        res[key] = {"frames_per_s": round(fps, 1), "form_run": ["exact", "fast", "tc"][info.form],
                    "roofline_step": {"algorithmic_bytes": ab_bytes, "achieved": round(ab_bytes * fps / 1e9, 1),
                                      "unit": "GB/s", "frac": round(ab_bytes * fps / 1e9 / peak, 4)}}
        if batch is not None:
            res[key]["how"] = (f"batch steps of {k} consecutive outputs, the next step's frames forwarded "
                               "concurrently, CUDA graph replay, autotuned launch shape")
            res[key]["tune"] = batch.tune()
            batch.close()
        eng.close()
    if not args.no_cpu:
        threads = os.cpu_count() or 1
        fps_cpu, steps = cpu_steady_state(frames, threads, 5.0, 200, bits=bits, params=params)
        res["cpu_baseline"] = {"value": round(fps_cpu, 3), "unit": UNIT, "cores": threads, "kind": "port",
                               "sample": f"{steps} steady-state output frames (about 5 s) on {threads} host "
                                         "threads, C restatement of src/cpu, bit-identical to the reference"}
    return res


YUV_PARAMS = dict(sigma=2.5, bt=4, bw=32, bh=32, ow=16, oh=16, sharpen=0.4, scutoff=0.3, svr=1.0, smin=4.0,
                  smax=20.0, degrid=1.0)


def yuv_batched(args, dev, local_rank, peak):
    """1920x1080 YUV420P8, all three planes: the tensor-core form as one
    batch (one launch per kernel for the three planes, or for four consecutive
    frames' twelve planes, replayed as a CUDA graph, autotuned) against the fast
    form's per-plane engines."""
    import torch
    import fft3dcl_gb300 as F
    from fft3dcl_gb300 import synth
    w, h, nd = 1920, 1080, 8
    planes = [synth.moving_rects(w, h, nd, 0xF3D0 + 1, lo=16, hi=235, noise=2.5),
              synth.moving_rects(w // 2, h // 2, nd, 0xF3D0 + 11, lo=16, hi=240, noise=1.5, ramp=False),
              synth.moving_rects(w // 2, h // 2, nd, 0xF3D0 + 12, lo=16, hi=240, noise=1.5, ramp=False)]
    src = [torch.from_numpy(np.stack(p)).to(dev) for p in planes]
    ip = F.validate(w, h, 8, **YUV_PARAMS)
    bt, cur = ip.bt, ip.current
    res = {}
    # name: (form, storage flags, frames per step)
    variants = {"tc": ("tc", 0, 1), "tc_4frames": ("tc", 0, 4), "tc_5frames": ("tc", 0, 5),
                "tc_half": ("tc", F.FLAG_HALF_SPECTRA, 1), "tc_half_4frames": ("tc", F.FLAG_HALF_SPECTRA, 4),
                "fast": ("fast", 0, 1)}
    for name, (form, flags, k) in variants.items():
        st = torch.cuda.Stream(device=dev)
        engs = [F.Engine(p[0].shape[1], p[0].shape[0], 8, chroma=i > 0, form=form, device=local_rank,
                         stream=st.cuda_stream, flags=flags, **YUV_PARAMS) for i, p in enumerate(planes)]
        if flags:
            assert all(e.info().half_spectra for e in engs)
        # Batch slots by plane: [Y, U, V] for one frame, [Y, Y, Y, Y, U, ..., V] for four.
        slots = [(i, r) for i in range(3) for r in range(k)]
        dst = [torch.empty(planes[i][0].shape, dtype=torch.uint8, device=dev) for i, _ in slots]
        pitch = [planes[i][0].shape[1] for i, _ in slots]
        batch = F.Batch([engs[i] for i, _ in slots], graph=True, autotune=True) if form == "tc" else None

        def step(n):
            wins = [[n + r - cur + j for j in range(bt)] for _, r in slots]
            for (i, _), win in zip(slots, wins):
                for fn in (win if batch is not None else win[:-1]):
                    if not engs[i].has(fn):
                        engs[i].forward_device(fn, src[i][fn % nd].data_ptr(), pitch[i * k])
            if batch is not None:
                # Forward the next step's entering frames, concurrent with this
                # step's outputs.
                ahead = [n + k - 1 - cur + bt + r for _, r in slots]
                batch.step(ahead, [src[i][a % nd].data_ptr() for (i, _), a in zip(slots, ahead)], pitch, wins,
                           [d.data_ptr() for d in dst], pitch)
            else:
                last = wins[0][-1]
                for i, e in enumerate(engs):
                    if not e.has(last):
                        e.forward_device(last, src[i][last % nd].data_ptr(), pitch[i])
                    e.process_device(wins[0], dst[i].data_ptr(), pitch[i])
            for e in engs:
                e.prune(n - cur - 1, n + k - 1 - cur + bt + k)

        n = cur
        for _ in range(max(3 if batch is None else 6, args.warmup)):
            step(n)
            n += k
        torch.cuda.synchronize(dev)
        l0 = F.kernel_launches()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        nsteps = max(60, args.steps) // k  # at least 60 frames per variant
        for _ in range(nsteps):
            step(n)
            n += k
        e1.record(st)
        torch.cuda.synchronize(dev)
        ms = e0.elapsed_time(e1)
        fps = nsteps * k / (ms / 1000.0)
        res[name] = {"frames_per_s": round(fps, 1),
                     "launches_per_frame": round((F.kernel_launches() - l0) / (nsteps * k), 2),
                     "roofline_step": {"algorithmic_bytes": AB_YUV1080, "achieved": round(AB_YUV1080 * fps / 1e9, 1),
                                       "unit": "GB/s", "frac": round(AB_YUV1080 * fps / 1e9 / peak, 4)}}
        if batch is not None:
            res[name]["tune"] = batch.tune()
            batch.close()
        for e in engs:
            e.close()
    res["tc"]["form"] = ("tensor cores, 3 planes per launch, CUDA graph per frame, forward one frame ahead "
                         "concurrent with the outputs")
    res["tc_4frames"]["form"] = ("as tc, four consecutive frames per step: 12 planes per launch "
                                 "([Y x4, U x4, V x4]; each plane's outputs share window spectra in L2)")
    res["tc_5frames"]["form"] = "as tc_4frames with five consecutive frames per step: 15 planes per launch"
    res["tc_half"]["form"] = ("as tc, spectra cached as fp16 pairs (F3D_FLAG_HALF_SPECTRA: the original's "
                              "storage at precision 0, the default; opt-in, within +-1 LSB of the fp32 path)")
    res["tc_half_4frames"]["form"] = "as tc_4frames with fp16 spectrum storage"
    res["fast"]["form"] = "fp32 radix FFT, per-plane engines"
    if not args.no_cpu:
        # The oracle on every host thread, plane after plane: a frame takes
        # the sum of its three planes' times.
        threads = os.cpu_count() or 1
        secs, steps = 0.0, []
        for i, p in enumerate(planes):
            fps_p, n_p = cpu_steady_state(p, threads, 2.0, 100, bits=8, params=YUV_PARAMS, chroma=i > 0)
            secs += 1.0 / fps_p
            steps.append(n_p)
        res["cpu_baseline"] = {"value": round(1.0 / secs, 3), "unit": UNIT, "cores": threads, "kind": "port",
                               "sample": f"steady-state output frames per plane (Y, U, V: {steps}, about 2 s "
                                         f"each) on {threads} host threads, C restatement of src/cpu, "
                                         "bit-identical to the reference"}
    return res


SECTIONS = ("yuv1080p_all_planes", "gray8_640x360_bt3", "grays_1280x720_kalman_bw64")


def extra_section(name, args, dev, local_rank, peak):
    """One of the workloads measured beside the headline (the other
    configurations of the path), by name."""
    from fft3dcl_gb300 import synth
    if name == "yuv1080p_all_planes":
        return dict(workload="1920x1080 YUV420P8 all planes, sigma=2.5 bt=4 bw=bh=32 ow=oh=16 sharpen=0.4 "
                             "scutoff=0.3 svr=1 smin=4 smax=20 degrid=1, clip resident in HBM",
                    **yuv_batched(args, dev, local_rank, peak))
    if name == "gray8_640x360_bt3":
        return dict(workload="640x360 GRAY8, 16-frame clip, sigma=2 beta=1 bt=3 bw=bh=32 ow=oh=16 degrid=1 "
                             "sharpen=0 (the plain method), clip resident in HBM",
                    **config_section(args, dev, local_rank, synth.clip_gray8(), 8, GRAY8_PARAMS,
                                     ("exact", "fast", "tc"), AB_GRAY8, peak, kbatch=16))
    if name == "grays_1280x720_kalman_bw64":
        return dict(workload="1280x720 GRAYS float, 64-frame clip with scene cuts at 20 and 45, Kalman bt=0 "
                             "kratio=2 bw=bh=64 ow=oh=32, sigma pattern 2/1.5/2.5/3, state resident in HBM "
                             "(Kalman runs the exact form in every form)",
                    **config_section(args, dev, local_rank, synth.clip_grays(), 32, KALMAN_PARAMS, ("exact",),
                                     AB_KALMAN, peak))
    raise ValueError(f"unknown section {name}")


def run_section(args, local_rank):
    """--section NAME: that workload alone, one JSON line (for profiling
    captures of its kernels)."""
    import torch
    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    peak, _ = load_peaks()
    print(json.dumps({"section": args.section, **extra_section(args.section, args, dev, local_rank, peak)}),
          flush=True)


def fast_batch_run(args, dev, local_rank, clip_dev, k):
    """Steady-state batch steps of k consecutive outputs in the fast form,
    the clip resident in HBM, the frames after the windows forwarded in the
    same step (concurrently with the sweeps)."""
    import torch
    import fft3dcl_gb300 as F
    ip = F.validate(W, H, BITS, **PARAMS)
    bt, cur = ip.bt, ip.current
    pitch, nfr = W * 2, clip_dev.shape[0]
    stream = torch.cuda.Stream(device=dev)
    eng = F.Engine(W, H, BITS, form="fast", device=local_rank, stream=stream.cuda_stream, **PARAMS)
    outs = [torch.empty((H, W), dtype=torch.uint16, device=dev) for _ in range(k)]
    batch = F.Batch([eng] * k, graph=False, autotune=False)

    def step(n):
        wins = [[m - cur + i for i in range(bt)] for m in range(n, n + k)]
        for w in wins:
            for fn in w:
                if not eng.has(fn):
                    eng.forward_device(fn, clip_dev[fn % nfr].data_ptr(), pitch)
        ahead = [n + k - 1 - cur + bt + i for i in range(k)]
        batch.step(ahead, [clip_dev[a % nfr].data_ptr() for a in ahead], [pitch] * k, wins,
                   [o.data_ptr() for o in outs], [pitch] * k)
        eng.prune(n - cur - 1, n + k - 1 - cur + bt + k)

    n = cur
    for _ in range(max(3, args.warmup)):
        step(n)
        n += k
    torch.cuda.synchronize(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        step(n)
        n += k
    e1.record(stream)
    torch.cuda.synchronize(dev)
    fps = args.steps * k / (e0.elapsed_time(e1) / 1000.0)
    batch.close()
    eng.close()
    return {"value": round(fps, 3), "how": f"batch steps of {k} consecutive outputs: one forward launch per entering "
                                          "frame, the fused sweeps of the outputs in one launch, no graph"}


def run_reference(args):
    """--impl reference: the reference's CPU path on the host cores. The
    reference sources compile only here, so on the GPU host this is the C
    restatement (oracle/), bit-identical to the reference by its tests."""
    import oracle
    oracle.build(ref=False)
    frames = make_clip(args.frames)
    threads = os.cpu_count() or 1
    fps_warm, _ = cpu_steady_state(frames, threads, 0.0, max(1, args.warmup), max(1, args.warmup))
    fps, steps = cpu_steady_state(frames, threads, 0.0, args.steps, args.steps)
    kind = "port"
    line = {"metric": METRIC, "value": round(fps, 4), "unit": UNIT, "impl": "reference",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(1000.0 / fps, 3), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": WORKLOAD, "cpu_threads": threads},
            "cpu_baseline": {"value": round(fps, 4), "unit": UNIT, "cores": threads, "kind": kind,
                             "sample": f"{steps} steady-state 4K output frames, all {threads} host threads, "
                                       "C restatement of src/cpu (bit-identical to the reference)"},
            "e2e": {"value": round(fps, 4), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# --------------------------------------------------------------- GPU leg --

def slowest_rank(times_ms: list, world: int) -> list:
    """Replicas: each timing taken as the maximum over the ranks (the job
    ends when its slowest replica does), so that whole-job throughput is the
    units all ranks processed divided by that time."""
    if world <= 1:
        return list(times_ms)
    import torch
    t = torch.tensor(times_ms, dtype=torch.float64)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return [float(x) for x in t]


def replica_throughput(units_per_rank: float, world: int, ms: float) -> float:
    """Whole-job throughput of `world` replicas that each processed
    units_per_rank units in at most ms milliseconds."""
    return units_per_rank * world / (ms / 1000.0)


def run_gpu(args, rank, world, local_rank):
    import torch
    import fft3dcl_gb300 as F

    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    frames = make_clip(args.frames)
    clip_dev = torch.from_numpy(np.stack(frames)).to(dev)  # [48, H, W] uint16, resident
    ip = F.validate(W, H, BITS, **PARAMS)
    bt, cur = ip.bt, ip.current
    pitch = W * 2
    out = torch.empty((H, W), dtype=torch.uint16, device=dev)
    nfr = clip_dev.shape[0]

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    kout = args.outputs_per_step if (args.form == "tc" and not args.no_batch) else 1
    outs = [out] + [torch.empty((H, W), dtype=torch.uint16, device=dev) for _ in range(kout - 1)]

    def device_run(form, with_clocks=False, batched=False):
        """Steady-state steps with the clip resident in HBM: (ms for
        args.steps steps, per-kernel ms, launches, clocks, engine). Batched
        (tensor-core form): each step is one batch step of kout consecutive
        outputs - the forwards of the frames after their windows run
        concurrently with the outputs - replayed as a CUDA graph, launch
        shape autotuned; the per-kernel times come from the engine's own
        calls. Returns the frames per step too."""
        stream = torch.cuda.Stream(device=dev)
        eng = F.Engine(W, H, BITS, form=form, device=local_rank, stream=stream.cuda_stream, **PARAMS)
        k = kout if batched else 1
        batch = F.Batch([eng] * k, graph=True, autotune=True) if batched else None

        def step_engine(n):
            win = [n - cur + i for i in range(bt)]
            for fn in win:
                if not eng.has(fn):
                    eng.forward_device(fn, clip_dev[fn % nfr].data_ptr(), pitch)
            eng.process_device(win, out.data_ptr(), pitch)
            eng.prune(n - cur - 1, n - cur + bt)

        def step_batch(n, b=None, ahead_in_step=True):
            b = batch if b is None else b
            wins = [[m - cur + i for i in range(bt)] for m in range(n, n + k)]
            for w in wins:
                for fn in w:
                    if not eng.has(fn):
                        eng.forward_device(fn, clip_dev[fn % nfr].data_ptr(), pitch)
            # The frames after the last window, forwarded concurrently with the
            # outputs (or, for kernel timing, by the next step's engine calls).
            ahead = [n + k - 1 - cur + bt + i for i in range(k)] if ahead_in_step else [-1] * k
            b.step(ahead, [clip_dev[a % nfr].data_ptr() for a in ahead], [pitch] * k, wins,
                   [o.data_ptr() for o in outs[:k]], [pitch] * k)
            eng.prune(n - cur - 1, n + k - 1 - cur + bt + k)

        step = step_batch if batched else step_engine

        n = cur
        for _ in range(max(3, args.warmup)):
            step(n)
            n += k
        torch.cuda.synchronize(dev)
        clocks = Clocks(local_rank) if with_clocks else None
        if clocks:
            clocks.start()
        barrier()
        torch.cuda.synchronize(dev)
        l0 = F.kernel_launches()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            step(n)
            n += k
        e1.record(stream)
        torch.cuda.synchronize(dev)
        barrier()
        launches = F.kernel_launches() - l0
        clk = clocks.stop() if clocks else None
        ms = e0.elapsed_time(e1)
        # Per-kernel device time over the same number of steps (a synchronize
        # after each step so that the engine's events can be read).
        kt = np.zeros(3)
        for _ in range(args.steps):
            step_engine(n)
            n += 1
            eng.synchronize()
            kt += np.array(eng.last_kernel_ms())
        kt /= args.steps
        if batch is not None:
            tune = batch.tune()
            forms_extra["tune"] = tune
            batch.close()
            # The batch step's own filter and inverse launches (k outputs per
            # launch), same launch shape, without a graph so that events
            # bracket them, and with the forwards outside the step so that no
            # concurrent kernel shares the GPU while they run.
            tb = F.Batch([eng] * k, graph=False, autotune=False)
            tb.set_tune(tune["fwd_ctas_per_sm"], tune["filter_minb"])
            bkt = np.zeros(2)
            for _ in range(max(3, args.warmup)):
                step_batch(n, tb, ahead_in_step=False)
                n += k
            for _ in range(args.steps):
                step_batch(n, tb, ahead_in_step=False)
                n += k
                bkt += np.array(tb.last_kernel_ms())
            tb.close()
            forms_extra["batch_kernel_ms"] = [float(x) for x in bkt / args.steps]
        return ms, kt, launches, clk, eng, stream, n, k

    # Other forms first (device throughput only), then the headline form.
    forms = {}
    forms_extra = {}
    for f in [x for x in args.compare.split(",") if x and x != args.form]:
        ms_f, kt_f, _, _, eng_f, _, _, _ = device_run(f)
        forms[f] = {"value": round(args.steps * world / (ms_f / 1000.0), 3),
                    "kernel_ms": [round(float(x), 4) for x in kt_f]}
        eng_f.close()
    batched = args.form == "tc" and not args.no_batch
    if batched and "fast" in args.compare.split(","):
        # The plain form batched the same way: k consecutive outputs per step
        # (one forward launch per entering frame, the k fused sweeps in one
        # launch with their CTAs interleaved), launched directly.
        forms["fast_batch"] = fast_batch_run(args, dev, local_rank, clip_dev, kout)
    if batched:
        # The tensor-core engine's own calls, for comparison with its batch.
        ms_d, kt_d, _, _, eng_d, _, _, _ = device_run("tc")
        forms["tc_direct"] = {"value": round(args.steps * world / (ms_d / 1000.0), 3),
                              "kernel_ms": [round(float(x), 4) for x in kt_d],
                              "how": "engine calls, forward then output, no graph"}
        eng_d.close()
    ms, kt, launches, clk, eng, stream, n, kframes = device_run(args.form, with_clocks=True, batched=batched)
    info = eng.info()
    forms[args.form] = {"value": round(args.steps * kframes * world / (ms / 1000.0), 3),
                        "kernel_ms": [round(float(x), 4) for x in kt]}
    if batched:
        forms[args.form]["how"] = (f"batch step of {kout} consecutive outputs, the forwards of the frames after "
                                   "their windows concurrent with them, CUDA graph replay, autotuned launch shape")
        forms[args.form]["tune"] = forms_extra.get("tune")

    # End to end with host buffers: pinned source planes, upload of the
    # entering frame and readback of the packed output inside the timed
    # region. Tensor-core form: the pipeline a host-buffer user runs with the
    # batch API - the upload of frame n+2 (upload stream), the batch step
    # (forward n+2 concurrent with output n) and the readback of output n
    # (readback stream) overlap across steps. Other forms: the engine's
    # synchronous forward_raw / process_raw calls.
    host = [torch.from_numpy(frames[i]).pin_memory() for i in range(min(8, nfr))]
    hnp = [h.numpy() for h in host]
    eng.prune(-1, -2)
    e2e_how = "engine forward_raw + process_raw per step (synchronous)"
    if batched:
        k = kframes
        up = torch.cuda.Stream(device=dev)    # uploads
        down = torch.cuda.Stream(device=dev)  # readbacks
        dsrc = [[torch.empty((H, W), dtype=torch.uint16, device=dev) for _ in range(k)] for _ in range(3)]
        dout = [[torch.empty((H, W), dtype=torch.uint16, device=dev) for _ in range(k)] for _ in range(2)]
        hout = [[torch.empty((H, W), dtype=torch.uint16).pin_memory() for _ in range(k)] for _ in range(2)]
        ev_up = [torch.cuda.Event() for _ in range(3)]
        ev_comp = [torch.cuda.Event() for _ in range(3)]
        ev_read = [torch.cuda.Event() for _ in range(2)]
        pbatch = F.Batch([eng] * k, graph=True, autotune=True)
        e2e_how = (f"batch API pipeline, {k} outputs per step: uploads of the entering frames and readbacks of "
                   "the outputs on two copy streams, overlapping the batch steps (forwards concurrent with the "
                   "outputs, CUDA graph)")
        step_no = [0]

        def step_host(n):
            wins = [[m - cur + i for i in range(bt)] for m in range(n, n + k)]
            for w in wins:
                for fn in w:
                    if not eng.has(fn):
                        eng.forward_raw(fn, hnp[fn % len(hnp)])
            ahead = [n + k - 1 - cur + bt + i for i in range(k)]
            k3, k2 = step_no[0] % 3, step_no[0] % 2
            step_no[0] += 1
            with torch.cuda.stream(up):
                up.wait_event(ev_comp[k3])  # the forwards that read these slots three steps ago
                for i, a in enumerate(ahead):
                    dsrc[k3][i].copy_(host[a % len(host)], non_blocking=True)
                ev_up[k3].record(up)
            stream.wait_event(ev_up[k3])
            stream.wait_event(ev_read[k2])    # output slots read back two steps ago
            pbatch.step(ahead, [d.data_ptr() for d in dsrc[k3]], [pitch] * k, wins,
                        [d.data_ptr() for d in dout[k2]], [pitch] * k)
            ev_comp[k3].record(stream)
            with torch.cuda.stream(down):
                down.wait_event(ev_comp[k3])
                for i in range(k):
                    hout[k2][i].copy_(dout[k2][i], non_blocking=True)
                ev_read[k2].record(down)
            eng.prune(n - cur - 1, n + k - 1 - cur + bt + k)
    else:
        hout = torch.empty((H, W), dtype=torch.uint16).pin_memory()
        hout_np = hout.numpy()

        def step_host(n):
            win = [n - cur + i for i in range(bt)]
            for fn in win:
                if not eng.has(fn):
                    eng.forward_raw(fn, hnp[fn % len(hnp)])
            eng.process_raw(win, hout_np)
            eng.prune(n - cur - 1, n - cur + bt)

    kstep = kframes if batched else 1
    for _ in range(max(3, args.warmup)):
        step_host(n)
        n += kstep
    barrier()
    torch.cuda.synchronize(dev)
    h0, h1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    gc.disable()  # no collector pause inside the host-driven timed loop
    h0.record(stream)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step_host(n)
        n += kstep
    if batched:
        stream.wait_stream(down)  # the last readbacks
    h1.record(stream)
    torch.cuda.synchronize(dev)
    wall = time.perf_counter() - t0
    gc.enable()
    barrier()
    ms_e2e = max(h0.elapsed_time(h1), wall * 1000.0)
    if batched:
        pbatch.close()
    eng.close()

    ms, ms_e2e = slowest_rank([ms, ms_e2e], world)
    if rank != 0:
        return
    fps = replica_throughput(args.steps * kframes, world, ms)
    fps_e2e = replica_throughput(args.steps * kframes, world, ms_e2e)
    ab = algorithmic_bytes(info.nblocks, info.fbw, ip.bh, bt)
    peak, peak_kind = load_peaks()
    inv_ms = float(kt[1])
    # The dominant kernel, timed between the engine's events: the tensor-core
    # filter (window spectra in; its operand tiles are an intermediate), the
    # fused fast-form sweep (window spectra in, packed plane out) or, unfused,
    # the filter+inverse kernel (window spectra in).
    if info.form == 2 and info.fused:
        kname, kbytes = "k_filter_tc (temporal filter of the window spectra)", ab["filter_inverse"]
        kt_names = ("forward", "filter", "inverse_overlap_add")
    elif info.fused:
        kname, kbytes = "k_sweep_fast (filter+inverse+overlap-add+pack)", ab["filter_inverse"] + ab["plane"]
        kt_names = ("forward", "sweep", "seam_merge")
    else:
        kname, kbytes = "k_inverse (filter+inverse)", ab["filter_inverse"]
        kt_names = ("forward", "filter_inverse", "overlap_add")
    achieved = kbytes / (inv_ms / 1000.0) / 1e9 if inv_ms > 0 else None
    roof_single = {"kernel": kname, "bound": "hbm",
                   "achieved": achieved and round(achieved, 1), "peak": peak, "unit": "GB/s",
                   "frac": achieved and round(achieved / peak, 4),
                   "traffic": NCU_TRAFFIC.get(args.form), "algorithmic_bytes": kbytes,
                   "peak_source": f"{peak_kind} hbm_gbs"}
    roof = roof_single
    bkt = forms_extra.get("batch_kernel_ms")
    if bkt and kframes > 1 and info.form == 2 and info.fused:
        # The headline step's own filter launch: kframes consecutive outputs,
        # each reading its bt window spectra (shared ones from L2).
        bbytes = kframes * kbytes
        bach = bbytes / (bkt[0] / 1000.0) / 1e9
        roof = {"kernel": f"k_filter_tc, {kframes} consecutive outputs per launch (the headline batch step)",
                "bound": "hbm", "achieved": round(bach, 1), "peak": peak, "unit": "GB/s",
                "frac": round(bach / peak, 4), "traffic": NCU_TRAFFIC_BATCH.get(kframes),
                "algorithmic_bytes": bbytes, "peak_source": f"{peak_kind} hbm_gbs"}
    line = {
        "metric": METRIC, "value": round(fps, 3), "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms / args.steps, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": DTYPE_OF_FORM[args.form],
        "data": "synthetic (seeded ramp + moving rectangles, Gaussian noise 12 LSB, 10-bit)",
        "config": {"workload": WORKLOAD if kframes == 1 else WORKLOAD.replace(
                       "one output frame per step", f"{kframes} consecutive output frames per step"),
                   "form": args.form, "parallelism": f"replicas x{world}",
                   "inputs": f"clip resident in HBM ({len(frames)} x 16.6 MB)",
                   "l2": "working set per step ~750 MB: four 143 MB window spectra, larger than the 129 MB L2"},
        "kernel_ms": {kt_names[i]: round(float(kt[i]), 4) for i in range(3)},
        "batch_kernel_ms": bkt and {"filter": round(bkt[0], 4), "inverse_overlap_add_merge": round(bkt[1], 4),
                                    "outputs_per_launch": kframes},
        "forms": forms,
        "roofline": roof,
        "roofline_single_output": roof_single,
        "roofline_step": {"algorithmic_bytes": ab["frame"],
                          "achieved": round(ab["frame"] * fps / world / 1e9, 1), "unit": "GB/s",
                          "frac": round(ab["frame"] * fps / world / 1e9 / peak, 4)},
        "e2e": {"value": round(fps_e2e, 3), "unit": UNIT, "h2d_bytes_per_step": W * H * 2 * kframes,
                "d2h_bytes_per_step": W * H * 2 * kframes, "how": e2e_how},
        "frames_per_step": kframes,
        "gpu_launches": int(launches), "clocks": clk,
    }
    if world == 1 and not args.no_yuv:
        line["yuv1080p_all_planes"] = extra_section("yuv1080p_all_planes", args, dev, local_rank, peak)
    if world == 1 and not args.no_configs:
        for name in ("gray8_640x360_bt3", "grays_1280x720_kalman_bw64"):
            line[name] = extra_section(name, args, dev, local_rank, peak)
    if world == 1 and args.serve_streams > 0:
        # The serving workload: YUV 4:2:0 video streams (all planes) with
        # Poisson frame arrivals through the serving loop (shared steps for
        # the tensor-core streams, HBM-budget admission); then the same
        # streams with the arrival rates scaled up until the delivered rate
        # falls behind the offered one (saturation).
        from fft3dcl_gb300 import serving
        specs = serving.mixed_streams(args.serve_streams, args.serve_frames)
        sframes = [serving.stream_frames(s, distinct=4) for s in specs]

        def serve(rate):
            with F.Server(form=args.form, device=local_rank, max_streams=3 * len(specs),
                          hbm_budget=200 << 30) as sv:
                return serving.run(sv, specs, sframes, realtime=True, rate=rate, timeout_s=300, keep_outputs=False)[1]

        # Warm-up, untimed: the same mix with a few frames per stream, all at
        # once, so that every kernel of the mix is loaded before the timed runs.
        wspecs = serving.mixed_streams(args.serve_streams, 8)
        with F.Server(form=args.form, device=local_rank, max_streams=3 * len(wspecs), hbm_budget=200 << 30) as sv:
            serving.run(sv, wspecs, [serving.stream_frames(s, distinct=4) for s in wspecs], realtime=False,
                        timeout_s=300, keep_outputs=False)

        def point(rate, st):
            return {"rate_x": rate, "offered_frames_per_s": round(st["offered_frames_per_s"], 1),
                    "frames_per_s": round(st["frames_per_s"], 1), "p50_ms": round(st["p50_ms"], 3),
                    "p99_ms": round(st["p99_ms"], 3), "server_p99_ms": round(st["server_p99_ms"], 3),
                    "submit_lag_p99_ms": round(st["submit_lag_p99_ms"], 3),
                    "shared_steps": st["shared_steps"], "outputs_per_shared_step":
                        round(st["shared_outputs"] / st["shared_steps"], 2) if st["shared_steps"] else None,
                    "scheduler_busy": round(st["scheduler_busy"], 3) if st["scheduler_busy"] is not None else None}

        st = serve(1.0)
        sweep = [point(1.0, st)]
        for rate in (2.0, 4.0, 8.0, 16.0, 32.0, 64.0, 128.0):
            sweep.append(point(rate, serve(rate)))
            # Saturated: the delivered rate falls behind the offered one, or
            # frames queue for longer than a tenth of a second.
            if sweep[-1]["frames_per_s"] < 0.9 * sweep[-1]["offered_frames_per_s"] or sweep[-1]["p99_ms"] > 100.0:
                break
        capacity = max(p["frames_per_s"] for p in sweep)
        line["serving"] = {
            "streams": len(specs), "frames_per_stream": args.serve_frames,
            "p50_ms": round(st["p50_ms"], 3), "p99_ms": round(st["p99_ms"], 3), "max_ms": round(st["max_ms"], 3),
            "server_p50_ms": round(st["server_p50_ms"], 3), "server_p99_ms": round(st["server_p99_ms"], 3),
            "frames_per_s": round(st["frames_per_s"], 1),
            "offered_frames_per_s": round(st["offered_frames_per_s"], 1),
            "shared_steps": st["shared_steps"], "max_outputs_per_shared_step": st["max_shared"],
            "capacity_frames_per_s": capacity,
            "load_sweep": sweep,
            "mix": "YUV420P8/P10 video streams, all three planes (one server stream per plane), resolutions "
                   "640x360..3840x2160, bt in {1,3,4}, bw in {16,32}; every stream runs the tensor-core form and "
                   "streams with the same block size, bt and depth share steps",
            "arrivals": "Poisson, 24-60 frames/s per stream (rate_x scales every stream's rate)",
            "latency": "per video frame: scheduled arrival of the last frame its temporal window needs -> last "
                       "plane's output copied to host memory (server_*: from that frame's arrival at the server)",
            "form": args.form}
    if world == 1 and not args.no_cpu:
        cpu_threads = os.cpu_count() or 1
        fps_cpu, steps = cpu_steady_state(frames, cpu_threads, 12.0, 30)
        fps_cpu1, steps1 = cpu_steady_state(frames, 1, 0.0, 1)
        line["cpu_baseline"] = {
            "value": round(fps_cpu, 4), "unit": UNIT, "cores": cpu_threads, "kind": "port",
            "sample": f"{steps} steady-state 4K output frames on {cpu_threads} host threads "
                      f"(1 thread: {fps_cpu1:.4f} frames/s over {steps1} frame), C restatement of "
                      "src/cpu, bit-identical to the reference"}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--form", default="tc", choices=["exact", "fast", "tc"],
                    help="arithmetic form of the headline line")
    ap.add_argument("--compare", default="exact,fast",
                    help="comma-separated forms whose device throughput is reported under 'forms'")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--serve-streams", type=int, default=16, help="streams of the serving run (0: skip it)")
    ap.add_argument("--no-yuv", action="store_true", help="skip the batched 1080p YUV measurement")
    ap.add_argument("--no-configs", action="store_true",
                    help="skip the 640x360 GRAY8 and 720p float Kalman measurements")
    ap.add_argument("--no-batch", action="store_true",
                    help="tensor-core headline through the engine's own calls instead of a batch step")
    ap.add_argument("--outputs-per-step", type=int, default=DEFAULT_OUTPUTS_PER_STEP, choices=list(range(1, 17)),
                    help="tensor-core batch: consecutive output frames per step")
    ap.add_argument("--size", default=None,
                    help="WxH of the luma plane instead of 3840x2160 (small cases for profiling)")
    ap.add_argument("--serve-frames", type=int, default=120, help="frames per serving stream")
    ap.add_argument("--frames", type=int, default=NFRAMES,
                    help="frames of the resident clip (fewer only to keep profiler captures small)")
    ap.add_argument("--section", default=None, choices=SECTIONS,
                    help="run only this workload of the extra sections and print its results")
    args = ap.parse_args()
    if args.size:
        global W, H, WORKLOAD
        W, H = (int(v) for v in args.size.lower().split("x"))
        WORKLOAD = WORKLOAD.replace("3840x2160", f"{W}x{H}")
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        if rank == 0:
            run_reference(args)
        return
    if args.section:
        run_section(args, local_rank)
        return
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    try:
        run_gpu(args, rank, world, local_rank)
    finally:
        if world > 1:
            import torch.distributed as dist
            dist.destroy_process_group()


if __name__ == "__main__":
    main()
