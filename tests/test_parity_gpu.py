"""GPU parity: the CUDA engine through its C ABI against the oracle.

Exact form: the reference's radix-2 operation order without fused
multiply-add, so the bar is bit equality with the oracle (itself bit-equal to
the reference CPU backend). Tolerances for the other forms are stated where
they are used: +-1 LSB at 8 bit, +-4 LSB at 10 bit, 1e-4 absolute for float
output (samples in [0, 1])."""
import glob
import json
import os

import numpy as np
import pytest

import fft3dcl_gb300 as F
import oracle
from fft3dcl_gb300 import synth

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = sorted(p for p in glob.glob(os.path.join(GOLDEN, "*.npz")) if not p.endswith("fft8_kat.npz"))
THREADS = min(16, os.cpu_count() or 1)


def load_case(path):
    z = np.load(path)
    return (list(z["frames"]), list(z["out"]), int(z["bits"]), bool(int(z["chroma"])),
            json.loads(str(z["params"])))


def gpu_clip(frames, bits, chroma=False, form="exact", **params):
    """Run one plane through the engine the way the reference plugin drives
    GpuRef: forward the window frames that are not cached, process, prune."""
    h, w = frames[0].shape
    st = 1 if frames[0].dtype == np.float32 else 0
    if chroma:
        # A chroma plane: a YUV clip whose planes 1 and 2 are this plane.
        clip = [[np.zeros((h, w), f.dtype), f, f] for f in frames]
        flt = F.Filter(clip, F.VideoFormat("yuv", bits, st), form=form, plane=1, **params)
        k = 1
    else:
        flt = F.Filter([[f] for f in frames], F.VideoFormat("gray", bits, st), form=form, **params)
        k = 0
    try:
        return [flt.get_frame(n)[k] for n in range(len(frames))]
    finally:
        flt.close()


@pytest.mark.parametrize("path", CASES, ids=[os.path.basename(p)[:-4] for p in CASES])
def test_exact_form_matches_golden_bit_for_bit(path):
    frames, out, bits, chroma, params = load_case(path)
    got = gpu_clip(frames, bits, chroma=chroma, **params)
    for n, (g, o) in enumerate(zip(got, out)):
        np.testing.assert_array_equal(g, o, err_msg=f"frame {n}")
    assert F.live_instances() == 0 and F.live_bytes() == 0


SIZES = [(4, 4), (8, 8), (16, 16), (32, 32), (64, 64), (8, 32), (32, 8), (64, 16), (16, 64), (4, 64)]


@pytest.mark.parametrize("bw,bh", SIZES)
def test_forward_spectra_exact(bw, bh):
    rng = np.random.default_rng(bw * 100 + bh)
    plane = rng.integers(0, 256, (97, 131)).astype(np.uint8)
    with F.Engine(131, 97, 8, bw=bw, bh=bh) as e:
        e.forward_raw(7, plane)
        spec = e.spectra(7)
    pl = oracle.Plane(131, 97, 8, bw=bw, bh=bh)
    ref = pl.spectra(pl.upload(plane))
    np.testing.assert_array_equal(spec, ref)


@pytest.mark.parametrize("bw,bh,bt,extra", [
    (32, 32, 3, {}), (16, 16, 4, {"sharpen": 0.5}), (64, 64, 1, {}), (8, 16, 2, {"degrid": 0.7}),
    (64, 32, 0, {"sigma2": 3.0}), (4, 4, -1, {"sharpen": 0.3}), (32, 64, 4, {"wintype": 1}),
    (16, 8, 3, {"ow": 4, "oh": 2}), (32, 16, 3, {"mode": 0}),
    # 64 x 64 blocks run their transforms on lane pairs: every temporal mode
    # family, sharpen, pattern, window types, mode 0.
    (64, 64, 4, {"sharpen": 0.4, "sigma2": 2.5}), (64, 64, 3, {"mode": 0}),
    (64, 64, 2, {"wintype": 2, "degrid": 0.5}), (64, 64, -1, {"sharpen": 0.2, "wintype": 1}),
])
def test_block_sizes_and_modes_exact(bw, bh, bt, extra):
    frames = synth.moving_rects(150, 90, 6, bw + bh + bt, lo=16, hi=235, noise=4.0, n_rects=6)
    params = dict(bw=bw, bh=bh, bt=bt, **extra)
    got = gpu_clip(frames, 8, **params)
    ref = oracle.run_clip(frames, 8, threads=THREADS, **params)
    for g, r in zip(got, ref):
        np.testing.assert_array_equal(g, r)


# Blocks above 64, up to the reference CPU backend's 512 (src/params.h:62-72):
# the exact form's large-block kernels (one CTA per block, transforms through
# global memory), in every temporal mode, mode 0, general overlap, 16-bit and
# float samples; every form asked for runs them.
BIG = [
    (128, 128, 3, {}, 8, "exact"), (256, 64, 2, {"sharpen": 0.3}, 8, "fast"),
    (512, 512, 1, {}, 8, "tc"), (128, 32, 0, {"sigma2": 3.0}, 8, "exact"),
    (16, 256, 4, {"mode": 0}, 8, "exact"), (128, 128, 4, {"ow": 48, "oh": 40}, 8, "exact"),
    (256, 256, -1, {"sharpen": 0.4}, 8, "exact"), (128, 64, 3, {"wintype": 2, "degrid": 0.6}, 12, "exact"),
    (64, 128, 2, {"wintype": 1}, 32, "fast"),
]


@pytest.mark.parametrize("bw,bh,bt,extra,bits,form", BIG,
                         ids=[f"{c[0]}x{c[1]}_bt{c[2]}_{c[4]}bit_{c[5]}" for c in BIG])
def test_large_blocks_exact(bw, bh, bt, extra, bits, form):
    w, h = (600, 400) if max(bw, bh) >= 256 else (300, 210)
    seed = bw * 7 + bh + bt
    if bits == 32:
        frames = synth.moving_rects(w, h, 5, seed, lo=0.06, hi=0.92, noise=0.01, dtype=np.float32, n_rects=5)
    elif bits > 8:
        frames = synth.moving_rects(w, h, 5, seed, lo=200, hi=3900, noise=20.0, dtype=np.uint16,
                                    maxval=(1 << bits) - 1, n_rects=5)
    else:
        frames = synth.moving_rects(w, h, 5, seed, lo=16, hi=235, noise=4.0, n_rects=5)
    params = dict(bw=bw, bh=bh, bt=bt, **extra)
    with F.Engine(w, h, bits, 1 if bits == 32 else 0, form=form, **params) as e:
        assert e.info().form == F.FORMS["exact"]
    got = gpu_clip(frames, bits, form=form, **params)
    ref = oracle.run_clip(frames, bits, threads=THREADS, **params)
    for g, r in zip(got, ref):
        np.testing.assert_array_equal(g, r)
    assert F.live_instances() == 0 and F.live_bytes() == 0


@pytest.mark.parametrize("bw,bh", [(128, 128), (512, 256), (8, 512)])
def test_large_block_spectra_exact(bw, bh):
    rng = np.random.default_rng(bw + bh)
    plane = rng.integers(0, 256, (230, 301)).astype(np.uint8)
    with F.Engine(301, 230, 8, bw=bw, bh=bh) as e:
        e.forward_raw(3, plane)
        spec = e.spectra(3)
    pl = oracle.Plane(301, 230, 8, bw=bw, bh=bh)
    np.testing.assert_array_equal(spec, pl.spectra(pl.upload(plane)))


@pytest.mark.parametrize("nframes,bt", [(1, 3), (1, 4), (2, 3), (2, 4), (3, 4), (3, 2), (1, 0)])
def test_short_clips_clamp_the_window(nframes, bt):
    # Clips of 1-3 frames with bt=3/4: window indices clamp to the clip
    # (src/fft3dcl.cpp:303-331, :424-430).
    frames = synth.moving_rects(70, 50, nframes, 9 + nframes, lo=16, hi=235, noise=3.0, n_rects=3)
    got = gpu_clip(frames, 8, bt=bt)
    ref = oracle.run_clip(frames, 8, bt=bt)
    for g, r in zip(got, ref):
        np.testing.assert_array_equal(g, r)


@pytest.mark.parametrize("w,h", [(1, 1), (5, 3), (17, 40), (33, 1), (2, 70)])
def test_planes_smaller_than_a_block(w, h):
    # Mirror addressing wraps several times when the plane is smaller than
    # the block (src/cpu/reference.cpp:10-17).
    frames = synth.moving_rects(w, h, 4, w * 7 + h, lo=16, hi=235, noise=5.0, n_rects=1)
    got = gpu_clip(frames, 8, bt=2, sharpen=0.2)
    ref = oracle.run_clip(frames, 8, bt=2, sharpen=0.2)
    for g, r in zip(got, ref):
        np.testing.assert_array_equal(g, r)


def test_gray8_640x360_bt3_exact():
    # Plain-method workload: 640x360 GRAY8, 16 frames, sigma=2 bt=3 32x32/16.
    frames = synth.clip_gray8()
    params = dict(sigma=2.0, beta=1.0, bt=3, bw=32, bh=32, ow=16, oh=16, degrid=1.0, sharpen=0.0)
    got = gpu_clip(frames, 8, **params)
    ref = oracle.run_clip(frames, 8, threads=THREADS, **params)
    for g, r in zip(got, ref):
        np.testing.assert_array_equal(g, r)


def test_yuv420p8_1080p_all_planes_exact():
    y, u, v = synth.clip_yuv420p8(frames=6)
    params = dict(sigma=2.5, bt=4, bw=32, bh=32, ow=16, oh=16, sharpen=0.4, scutoff=0.3, svr=1.0,
                  smin=4.0, smax=20.0, degrid=1.0)
    clip = [[a, b, c] for a, b, c in zip(y, u, v)]
    flt = F.Filter(clip, F.VideoFormat("yuv", 8, 0, 1, 1), plane=4, **params)
    got = [flt.get_frame(n) for n in range(len(clip))]
    flt.close()
    for p, (plane, chroma) in enumerate(((y, False), (u, True), (v, True))):
        ref = oracle.run_clip(plane, 8, chroma=chroma, threads=THREADS, **params)
        for n in range(len(clip)):
            np.testing.assert_array_equal(got[n][p], ref[n], err_msg=f"plane {p} frame {n}")


def test_yuv420p10_4k_luma_exact():
    frames = synth.clip_yuv420p10_luma(frames=5)
    params = dict(sigma=3.0, bt=4, bw=32, bh=32, ow=16, oh=16, sharpen=0.4, precision=2)
    got = gpu_clip(frames, 10, **params)
    ref = oracle.run_clip(frames, 10, first=1, count=3, threads=THREADS, **params)
    for g, r in zip(got[1:4], ref):
        np.testing.assert_array_equal(g, r)


def test_grays_720p_kalman_pattern_exact():
    frames = synth.clip_grays(frames=26, cuts=(20,))
    params = dict(bt=0, kratio=2.0, bw=64, bh=64, ow=32, oh=32, sigma=2.0, sigma2=1.5, sigma3=2.5,
                  sigma4=3.0)
    got = gpu_clip(frames, 32, **params)
    ref = oracle.run_clip(frames, 32, threads=THREADS, **params)
    for n, (g, r) in enumerate(zip(got, ref)):
        np.testing.assert_array_equal(g, r, err_msg=f"frame {n}")


def test_round_trip_identity_at_4k():
    # Size-independent property at full size: bt=-1 without sharpen is
    # analysis window -> FFT -> inverse FFT -> synthesis window -> overlap-add,
    # and the half-cosine windows of wintype 0 add up to one at half overlap,
    # so 10-bit samples come back within one LSB.
    frames = synth.clip_yuv420p10_luma(frames=2)
    got = gpu_clip(frames, 10, bt=-1, sharpen=0.0)
    for g, f in zip(got, frames):
        d = np.abs(g.astype(np.int64) - f.astype(np.int64))
        assert d.max() <= 1


def test_deterministic_across_runs():
    frames = synth.clip_gray8(frames=6)
    a = gpu_clip(frames, 8, bt=4, sharpen=0.4)
    b = gpu_clip(frames, 8, bt=4, sharpen=0.4)
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x, y)


def test_device_memory_returns_to_zero():
    e = F.Engine(1280, 720, 8, bt=4)
    info = e.info()
    assert info.device_bytes > 0 and F.live_bytes() >= info.device_bytes
    rng = np.random.default_rng(0)
    for fn in range(6):
        e.forward_raw(fn, rng.integers(0, 256, (720, 1280)).astype(np.uint8))
    assert e.info().cached_frames == 6
    e.prune(2, 3)
    assert e.info().cached_frames == 2
    e.close()
    assert F.live_instances() == 0 and F.live_bytes() == 0


def test_missing_window_frame_is_an_error():
    with F.Engine(64, 64, 8, bt=3) as e:
        e.forward_raw(0, np.zeros((64, 64), np.uint8))
        with pytest.raises(F.F3DError, match="missing spectra"):
            e.process_raw([0, 1, 2])


def test_float_process_matches_oracle_filter_and_synthesize():
    # GpuRef::process returns the float plane before packing.
    rng = np.random.default_rng(3)
    frames = [rng.uniform(0, 1, (72, 88)).astype(np.float32) for _ in range(3)]
    pl = oracle.Plane(88, 72, 8, bt=3)
    pl.build_degrid()
    specs = [pl.spectra(f) for f in frames]
    ref = pl.filter_and_synthesize(specs)
    with F.Engine(88, 72, 8, bt=3) as e:
        for i, f in enumerate(frames):
            e.forward(i, f)
        got = e.process([0, 1, 2])
    np.testing.assert_array_equal(got, ref)
