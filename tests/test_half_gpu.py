"""Half-precision spectrum storage (F3D_FLAG_HALF_SPECTRA): where it applies
(8-bit planes at precision 0 or 1 in the fused tensor-core form, the storage
of the original filter's precision 0/1), the spectra are cached as fp16 pairs
and the output stays within the 8-bit tolerance (+-1 LSB) of the oracle;
where it does not apply, the flag changes nothing."""
import json

import numpy as np
import pytest

import fft3dcl_gb300 as F
import oracle
from oracle import fp64
from fft3dcl_gb300 import synth

pytestmark = pytest.mark.gpu

HALF = F.FLAG_HALF_SPECTRA


def worst_diff(got, ref):
    return max(float(np.abs(g.astype(np.float64) - r.astype(np.float64)).max()) for g, r in zip(got, ref))


@pytest.mark.parametrize("bits,form,params,applies", [
    (8, "tc", dict(precision=0), True),
    (8, "tc", dict(precision=1), True),
    (8, "tc", dict(precision=2), False),
    (10, "tc", dict(precision=0), False),     # forced to precision 2 above 8 bits
    (8, "fast", dict(precision=0), False),
    (8, "tc", dict(precision=0, bw=16, bh=16), True),
    (8, "tc", dict(precision=0, ow=8, oh=8), False),  # tensor-core forward, fast-form inverse
])
def test_half_storage_applies_where_the_original_used_it(bits, form, params, applies):
    with F.Engine(320, 192, bits, form=form, flags=HALF, **params) as e:
        info = e.info()
        assert bool(info.half_spectra) == applies
        bins = info.nblocks * info.fbw * e.sp_bh
        assert info.spectrum_bytes == bins * (4 if applies else 8)


CASES = [
    ("gray8_bt3_p0", lambda: synth.clip_gray8(frames=8), dict(bt=3, precision=0)),
    ("gray8_bt4_sharpen_p1", lambda: synth.clip_gray8(frames=6), dict(bt=4, sharpen=0.4, precision=1)),
    ("gray8_bt2_degrid", lambda: synth.clip_gray8(frames=5), dict(bt=2, beta=1.5, degrid=0.5, precision=0)),
    ("gray8_bt1_pattern", lambda: synth.clip_gray8(frames=3), dict(bt=1, sigma2=1.0, sigma3=3.0, sigma4=4.0,
                                                                   precision=0)),
    ("gray8_btm1", lambda: synth.clip_gray8(frames=2), dict(bt=-1, sharpen=0.7, precision=0)),
    ("gray8_bw16_bt4", lambda: synth.clip_gray8(frames=6), dict(bt=4, bw=16, bh=16, sharpen=0.3, precision=0)),
]


@pytest.mark.parametrize("name,make,params", CASES, ids=[c[0] for c in CASES])
def test_half_storage_within_8bit_tolerance(name, make, params):
    frames = make()
    got = F.FFT3DCL(frames, bits=8, form="tc", flags=HALF, **params)
    ref = oracle.run_clip(frames, 8, threads=16, **params)
    worst = worst_diff(got, ref)
    print("half_storage", name, "max |diff| LSB", worst)
    assert worst <= 1
    again = F.FFT3DCL(frames, bits=8, form="tc", flags=HALF, **params)
    for a, b in zip(got, again):
        np.testing.assert_array_equal(a, b)


def test_half_storage_yuv_planes_within_tolerance():
    w, h = 480, 272
    y = synth.moving_rects(w, h, 6, 71, lo=16, hi=235, noise=2.5)
    u = synth.moving_rects(w // 2, h // 2, 6, 72, lo=16, hi=240, noise=1.5, ramp=False)
    v = synth.moving_rects(w // 2, h // 2, 6, 73, lo=16, hi=240, noise=1.5, ramp=False)
    clip = [[y[n], u[n], v[n]] for n in range(6)]
    params = dict(sigma=2.5, bt=4, sharpen=0.4, plane=4, precision=0)
    fmt = F.VideoFormat("yuv", 8, 0, 1, 1)
    got = F.FFT3DCL(clip, fmt, form="tc", flags=HALF, **params)
    for p, plane in enumerate([y, u, v]):
        ref = oracle.run_clip([plane[n] for n in range(6)], 8, threads=16, chroma=p > 0, **params)
        assert worst_diff([g[p] for g in got], ref) <= 1, p


def test_flag_without_effect_changes_nothing():
    frames = synth.clip_gray8(frames=5)
    params = dict(bt=3, precision=2)
    a = F.FFT3DCL(frames, bits=8, form="tc", flags=HALF, **params)
    b = F.FFT3DCL(frames, bits=8, form="tc", **params)
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x, y)


def test_half_spectra_error_against_fp64():
    # fp16 storage rounds each value to 11 significant bits (relative error
    # <= 2^-11); the relative RMS over a frame is well below that.
    plane = synth.clip_gray8(frames=1)[0]
    h, w = plane.shape
    params = dict(sigma=2.0, bt=3, precision=0)
    ref = fp64.spectra_fp64(plane, 8, **params)
    with F.Engine(w, h, 8, form="tc", flags=HALF, **params) as e:
        assert e.info().half_spectra
        e.forward_raw(0, plane)
        err = fp64.spectral_error(e.spectra(0), ref)
    print("spectral_error half", json.dumps(err))
    assert err["rel_rms"] < 5e-4


@pytest.mark.parametrize("graph", [False, True])
def test_half_batch_equals_engine(graph):
    import torch
    frames = synth.moving_rects(320, 192, 9, 81, lo=16, hi=235, noise=2.5)
    params = dict(sigma=2.0, bt=4, sharpen=0.3, precision=0)
    ref = F.FFT3DCL(frames, bits=8, form="tc", flags=HALF, **params)
    dev = torch.device("cuda", 0)
    st = torch.cuda.Stream(device=dev)
    e = F.Engine(320, 192, 8, form="tc", stream=st.cuda_stream, flags=HALF, **params)
    assert e.info().half_spectra
    src = torch.from_numpy(np.stack(frames)).to(dev)
    k = 2
    dst = [torch.empty((192, 320), dtype=torch.uint8, device=dev) for _ in range(k)]
    b = F.Batch([e] * k, graph=graph, autotune=True)
    nfr, pitch = len(frames), 320
    got = []
    with torch.cuda.stream(st):
        for n in range(0, nfr, k):
            wins = [[min(max(m - 2 + i, 0), nfr - 1) for i in range(4)] for m in range(n, n + k)]
            for wdw in wins:
                for fn in wdw:
                    if not e.has(fn):
                        e.forward_device(fn, src[fn].data_ptr(), pitch)
            ahead = [a if a < nfr else -1 for a in (n + k + 1 + i for i in range(k))]
            b.step(ahead, [src[min(a, nfr - 1)].data_ptr() for a in ahead], [pitch] * k, wins,
                   [d.data_ptr() for d in dst], [pitch] * k)
            st.synchronize()
            got += [d.cpu().numpy() for d in dst]
            e.prune(n - 3, n + 2 * k + 1)
    b.close()
    e.close()
    for n in range(nfr):
        np.testing.assert_array_equal(got[n], ref[n], err_msg=f"frame {n}")


def test_batch_rejects_mixed_spectrum_storage():
    with F.Engine(96, 64, 8, form="tc", bt=3, precision=0, flags=HALF) as e1, \
            F.Engine(96, 64, 8, form="tc", bt=3, precision=0) as e2:
        with pytest.raises(F.F3DError):
            F.Batch([e1, e2])
