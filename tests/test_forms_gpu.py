"""GPU parity of the non-exact arithmetic forms against the oracle.

Tolerances (the ones the path is specified with): +-1 LSB for 8-bit output,
+-4 LSB for 10-bit output (10-bit samples in 16-bit words), 1e-4 absolute for
float output with samples in [0, 1]. Each case also checks run-to-run
determinism of the form."""
import numpy as np
import pytest

import fft3dcl_gb300 as F
import oracle
from fft3dcl_gb300 import synth

pytestmark = pytest.mark.gpu

FORMS = ["fast", "tc"]


def tol_for(frames, bits):
    if frames[0].dtype == np.float32:
        return 1e-4
    return 1 if bits <= 8 else 4


def run(frames, bits, form, **params):
    return F.FFT3DCL(frames, bits=bits, form=form, **params)


def check(got, ref, tol):
    worst = 0.0
    for g, r in zip(got, ref):
        d = np.abs(g.astype(np.float64) - r.astype(np.float64)).max()
        worst = max(worst, d)
    assert worst <= tol, f"max |diff| {worst} > {tol}"
    return worst


CASES = [
    ("gray8_bt3", lambda: synth.clip_gray8(frames=8), 8, dict(bt=3)),
    ("gray8_bt4_sharpen", lambda: synth.clip_gray8(frames=6), 8, dict(bt=4, sharpen=0.4)),
    ("gray8_bt2_beta", lambda: synth.clip_gray8(frames=5), 8, dict(bt=2, beta=1.5, degrid=0.5)),
    ("gray8_bt1_pattern", lambda: synth.clip_gray8(frames=3), 8,
     dict(bt=1, sigma2=1.0, sigma3=3.0, sigma4=4.0)),
    ("gray8_btm1", lambda: synth.clip_gray8(frames=2), 8, dict(bt=-1, sharpen=0.7)),
    ("gray8_bw16_wintype1", lambda: synth.clip_gray8(frames=5), 8, dict(bw=16, bh=16, wintype=1)),
    # 16x16 blocks: the tensor-core form's 16-point DFT matrices, every temporal mode.
    ("gray8_bw16_bt4_sharpen", lambda: synth.clip_gray8(frames=6), 8, dict(bt=4, bw=16, bh=16, sharpen=0.4)),
    ("p10_bw16_bt3", lambda: synth.moving_rects(1280, 720, 5, 21, lo=64, hi=940, noise=10.0, dtype=np.uint16,
                                                maxval=1023), 10, dict(bt=3, bw=16, bh=16, sigma=3.0)),
    ("p10_bw16_bt2_pattern", lambda: synth.moving_rects(400, 232, 4, 22, lo=64, hi=940, noise=10.0,
                                                        dtype=np.uint16, maxval=1023), 10,
     dict(bt=2, bw=16, bh=16, sigma2=1.0, sigma3=3.0, sigma4=4.0)),
    ("gray8_bw16_bt1_wintype2", lambda: synth.clip_gray8(frames=3), 8, dict(bt=1, bw=16, bh=16, wintype=2)),
    ("gray8_bw16_btm1", lambda: synth.clip_gray8(frames=2), 8, dict(bt=-1, bw=16, bh=16, sharpen=0.6)),
    ("float_bw16_bt3", lambda: synth.clip_grays(frames=5), 32, dict(bt=3, bw=16, bh=16, sharpen=0.3)),
    ("p16_bw16_bt4", lambda: synth.moving_rects(224, 128, 6, 9, lo=4096, hi=60000, noise=300.0, dtype=np.uint16,
                                                maxval=65535), 16, dict(bt=4, bw=16, bh=16)),
    # 32x32 blocks: the tensor-core form folds these windows into its DFT matrices.
    ("gray8_wintype1", lambda: synth.clip_gray8(frames=5), 8, dict(bt=3, wintype=1, sharpen=0.3)),
    ("gray8_wintype2", lambda: synth.clip_gray8(frames=5), 8, dict(bt=4, wintype=2)),
    ("p10_wintype2", lambda: synth.moving_rects(320, 176, 5, 11, lo=64, hi=960, noise=8.0,
                                                            dtype=np.uint16, maxval=1023), 10,
     dict(bt=2, wintype=2, sharpen=0.2)),
    ("gray8_bw8x64_overlap", lambda: synth.clip_gray8(frames=5), 8, dict(bw=8, bh=64, ow=2, oh=16)),
    ("gray8_mode0", lambda: synth.clip_gray8(frames=5), 8, dict(mode=0, bw=16, bh=32)),
    ("p10_4k_bt4", lambda: synth.clip_yuv420p10_luma(frames=5), 10, dict(sigma=3.0, bt=4, sharpen=0.4)),
    ("float_bt3", lambda: synth.clip_grays(frames=5), 32, dict(bt=3, sharpen=0.3)),
    ("p12_bt2", lambda: synth.moving_rects(160, 96, 4, 7, lo=256, hi=3800, noise=20.0, dtype=np.uint16,
                                           maxval=4095), 12, dict(bt=2)),
    ("p16_bt3_sharpen", lambda: synth.moving_rects(224, 128, 5, 8, lo=4096, hi=60000, noise=300.0, dtype=np.uint16,
                                                   maxval=65535), 16, dict(bt=3, sharpen=0.3)),
    ("float_kalman_bw64", lambda: synth.clip_grays(frames=24, cuts=(12,)), 32,
     dict(bt=0, bw=64, bh=64, sigma2=1.5, sigma3=2.5, sigma4=3.0)),
]


@pytest.mark.parametrize("form", FORMS)
@pytest.mark.parametrize("name,make,bits,params", CASES, ids=[c[0] for c in CASES])
def test_form_within_tolerance(form, name, make, bits, params):
    frames = make()
    got = run(frames, bits, form, **params)
    ref = oracle.run_clip(frames, bits, threads=16, **params)
    check(got, ref, tol_for(frames, bits))
    again = run(frames, bits, form, **params)
    for a, b in zip(got, again):
        np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize("form", FORMS)
def test_form_spectra_close_to_oracle(form):
    rng = np.random.default_rng(1)
    plane = rng.integers(0, 256, (97, 131)).astype(np.uint8)
    for bw, bh in [(8, 8), (16, 16), (16, 32), (32, 32), (64, 16), (64, 64)]:
        with F.Engine(131, 97, 8, form=form, bw=bw, bh=bh) as e:
            e.forward_raw(0, plane)
            spec = e.spectra(0)
        pl = oracle.Plane(131, 97, 8, bw=bw, bh=bh)
        ref = pl.spectra(pl.upload(plane))
        # spectra scale with the block area (sums of up to bw*bh samples <= 1)
        assert np.abs(spec - ref).max() <= 2e-6 * bw * bh, (bw, bh)


@pytest.mark.parametrize("w,h,bits,params", [
    (3840, 2160, 10, dict(sigma=3.0, bt=4, sharpen=0.4)),
    (640, 360, 8, dict(bt=3)),
    (333, 177, 8, dict(bt=2, bw=16, bh=16, sharpen=0.5)),
    (97, 61, 8, dict(bt=1, bw=8, bh=8)),
    (1000, 37, 8, dict(bt=-1, sharpen=0.3)),
    (41, 700, 8, dict(bt=3, sigma2=1.0, sigma3=3.0, sigma4=4.0)),
])
def test_fused_sweep_equals_separate_kernels(w, h, bits, params):
    # The fused kernel adds each cell's four quadrants in the order of the
    # separate overlap-add kernel, so the two paths agree bit for bit.
    if bits == 8:
        frames = synth.moving_rects(w, h, 5, w + h, lo=16, hi=235, noise=4.0, n_rects=5)
    else:
        frames = synth.moving_rects(w, h, 5, w + h, lo=64, hi=940, noise=12.0, dtype=np.uint16, maxval=1023)
    outs = []
    for fused in (True, False):
        flt = F.Filter([[f] for f in frames], F.VideoFormat("gray", bits, 0), form="fast", fused=fused, **params)
        assert flt.engines[0].info().form == 1
        outs.append([flt.get_frame(n)[0] for n in range(len(frames))])
        flt.close()
    for a, b in zip(*outs):
        np.testing.assert_array_equal(a, b)


from test_parity_gpu import CASES as GOLDEN_CASES, gpu_clip, load_case  # noqa: E402


@pytest.mark.parametrize("form", FORMS)
@pytest.mark.parametrize("path", GOLDEN_CASES, ids=[p.rsplit("/", 1)[-1][:-4] for p in GOLDEN_CASES])
def test_form_golden_within_tolerance(form, path):
    # The golden outputs come from the reference's CPU backend; chroma planes,
    # 16-bit and float samples and every temporal mode are among them.
    frames, out, bits, chroma, params = load_case(path)
    got = gpu_clip(frames, bits, chroma=chroma, form=form, **params)
    check(got, out, tol_for(frames, bits))


@pytest.mark.parametrize("bw", [16, 32])
@pytest.mark.parametrize("w,h,params", [
    (640, 360, dict(bt=3)),
    (333, 177, dict(bt=2, sharpen=0.5)),
    (1000, 37, dict(bt=-1, sharpen=0.3)),
    (41, 700, dict(bt=4, sigma2=1.0, sigma3=3.0, sigma4=4.0)),
    (1920, 1080, dict(bt=1, degrid=0.0)),
    (24, 20, dict(bt=3)),
    (16, 16, dict(bt=4, sharpen=0.4)),
])
def test_tc_sweep_sizes(w, h, params, bw):
    # The tensor-core sweep on planes with ragged edges, one and many
    # segments (seam rows) and strips, against the oracle.
    frames = synth.moving_rects(w, h, 5, w + 3 * h, lo=16, hi=235, noise=4.0, n_rects=5)
    params = dict(params, bw=bw, bh=bw)
    flt = F.Filter([[f] for f in frames], F.VideoFormat("gray", 8, 0), form="tc", **params)
    info = flt.engines[0].info()
    assert info.form == 2 and info.fused == 1
    got = [flt.get_frame(n)[0] for n in range(len(frames))]
    flt.close()
    ref = oracle.run_clip(frames, 8, threads=16, **params)
    check(got, ref, 1)


@pytest.mark.parametrize("form", FORMS)
@pytest.mark.parametrize("bits", [8, 10, 32])
def test_form_yuv_planes_within_tolerance(form, bits):
    # All three planes of a YUV 4:2:0 clip: the chroma planes take the mode-1
    # chroma offset (src/cpu/reference.cpp:72-79; in the tensor-core form, the
    # window spectrum's correction), each plane against the oracle. bits=32:
    # float samples.
    w, h, n = 352, 208, 6
    if bits == 32:
        kw, s = dict(dtype=np.float32, maxval=1.0), 1.0 / 255.0
    elif bits == 8:
        kw, s = {}, 1
    else:
        kw, s = dict(dtype=np.uint16, maxval=(1 << bits) - 1), 4
    y = synth.moving_rects(w, h, n, 91 + bits, lo=16 * s, hi=235 * s, noise=2.5 * s, **kw)
    u = synth.moving_rects(w // 2, h // 2, n, 92 + bits, lo=16 * s, hi=240 * s, noise=1.5 * s, ramp=False, **kw)
    v = synth.moving_rects(w // 2, h // 2, n, 93 + bits, lo=16 * s, hi=240 * s, noise=1.5 * s, ramp=False, **kw)
    params = dict(sigma=2.5, bt=4, sharpen=0.4, plane=4)
    clip = [[y[i], u[i], v[i]] for i in range(n)]
    fmt = F.VideoFormat("yuv", bits, 1 if bits == 32 else 0, 1, 1)
    got = F.FFT3DCL(clip, fmt, form=form, **params)
    tol = 1e-4 if bits == 32 else (1 if bits == 8 else 4)
    for p, plane in enumerate([y, u, v]):
        ref = oracle.run_clip([plane[i] for i in range(n)], bits, threads=16, chroma=p > 0, **params)
        check([g[p] for g in got], ref, tol)
