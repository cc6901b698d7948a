"""Spectral error of each arithmetic form against the FP64 restatement of
the forward transform, on the plain 640x360 8-bit configuration and the 4K
10-bit configuration. Bounds: the fp32 radix forms stay within a few fp32
ulps (rel. RMS < 1e-6); the tensor-core form, fp16 hi/lo operands with fp32
accumulation, within 1e-5. The measured figures are printed."""
import json

import numpy as np
import pytest

import fft3dcl_gb300 as F
from oracle import fp64
from fft3dcl_gb300 import synth

pytestmark = pytest.mark.gpu

BOUND = {"exact": 1e-6, "fast": 1e-6, "tc": 1e-5}
CONFIGS = [
    ("640x360_gray8_bt3", lambda: synth.clip_gray8(frames=1)[0], 8, dict(sigma=2.0, bt=3)),
    ("4k_p10_bt4", lambda: synth.clip_yuv420p10_luma(frames=1)[0], 10, dict(sigma=3.0, bt=4, sharpen=0.4)),
    ("4k_p10_bt4_bw16", lambda: synth.clip_yuv420p10_luma(frames=1)[0], 10,
     dict(sigma=3.0, bt=4, bw=16, bh=16, sharpen=0.4)),
]


@pytest.mark.parametrize("name,make,bits,params", CONFIGS, ids=[c[0] for c in CONFIGS])
def test_spectral_error_per_form(name, make, bits, params):
    plane = make()
    h, w = plane.shape
    ref = fp64.spectra_fp64(plane, bits, **params)
    res = {}
    for form in ("exact", "fast", "tc"):
        with F.Engine(w, h, bits, form=form, **params) as e:
            assert e.info().form == F.FORMS[form]
            e.forward_raw(0, plane)
            res[form] = fp64.spectral_error(e.spectra(0), ref)
    print("spectral_error", name, json.dumps(res))
    for form, err in res.items():
        assert err["rel_rms"] < BOUND[form], (form, err)
