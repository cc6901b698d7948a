"""The FP64 restatement of the forward transform against the fp32 oracle
(which is pinned to the reference's CPU backend): they agree to fp32
rounding, so the FP64 spectra can stand as the exact values the forms'
spectral errors are measured against."""
import numpy as np
import pytest

import oracle
from oracle import fp64
from fft3dcl_gb300 import synth

CASES = [
    ("u8_bw32", 131, 97, 8, False, dict(bw=32, bh=32)),
    ("p10_chroma_bw16_wintype1", 160, 96, 10, True, dict(bw=16, bh=16, wintype=1)),
    ("float_bw32x16_wintype2", 200, 120, 32, False, dict(bw=32, bh=16, ow=8, oh=4, wintype=2)),
    ("u16_bw8", 64, 40, 16, False, dict(bw=8, bh=8)),
]


def plane_for(w, h, bits, seed):
    if bits == 32:
        return synth.moving_rects(w, h, 1, seed, lo=0.06, hi=0.9, noise=0.01, dtype=np.float32)[0]
    if bits == 8:
        return synth.moving_rects(w, h, 1, seed, lo=16, hi=235, noise=3.0)[0]
    maxv = (1 << bits) - 1
    return synth.moving_rects(w, h, 1, seed, lo=maxv * 0.06, hi=maxv * 0.92, noise=maxv / 80.0,
                              dtype=np.uint16, maxval=maxv)[0]


@pytest.mark.parametrize("name,w,h,bits,chroma,params", CASES, ids=[c[0] for c in CASES])
def test_fp64_restatement_matches_fp32_oracle(name, w, h, bits, chroma, params):
    plane = plane_for(w, h, bits, w + h)
    st = 1 if bits == 32 else 0
    pl = oracle.Plane(w, h, bits, sample_type=st, chroma=chroma, **params)
    ref32 = pl.spectra(pl.upload(plane))
    ref64 = fp64.spectra_fp64(plane, bits, chroma=chroma, **params)
    assert ref32.shape == ref64.shape
    err = fp64.spectral_error(ref32, ref64)
    assert err["rel_rms"] < 5e-7 and err["max_rel"] < 5e-7, err
