"""The oracle (C restatement of the reference CPU backend) pinned against the
reference: the 8-point FFT known answer and round trips of tools/fft_test.cpp,
the golden vectors generated from the reference's own build, and -- where the
reference sources are present -- live bit-for-bit comparisons."""
import glob
import json
import os

import numpy as np
import pytest

import oracle
from fft3dcl_gb300 import synth

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = sorted(p for p in glob.glob(os.path.join(GOLDEN, "*.npz")) if not p.endswith("fft8_kat.npz"))


def load_case(path):
    z = np.load(path)
    return (list(z["frames"]), list(z["out"]), int(z["bits"]), bool(int(z["chroma"])),
            json.loads(str(z["params"])))


def test_fft_known_answer():
    # tools/fft_test.cpp:42-47: forward of [0..7], X[1] = -4 + 9.6569i
    x = np.arange(8).astype(np.complex64)
    y = oracle.fft1d(x)
    assert abs(y[1] - (-4 + 9.6569j)) < 1e-4
    z = np.load(os.path.join(GOLDEN, "fft8_kat.npz"))
    np.testing.assert_array_equal(y, z["y"])
    back = oracle.fft1d(y, inverse=True)
    assert np.abs(back - x).max() < 1e-6


def test_fft2d_round_trip_and_dc():
    # tools/fft_test.cpp:10-39: DC = sum, 32x32 R2C -> C2R round trip
    rng = np.random.default_rng(12345)
    blk = rng.uniform(-1, 1, (32, 32)).astype(np.float32)
    full = np.zeros((32, 32), np.complex64)
    oracle.lib().orc_fft2d_forward(oracle._ptr(blk), 32, 32, oracle._ptr(full))
    assert abs(full[0, 0].real - blk.sum(dtype=np.float64)) < 1e-3
    half = np.ascontiguousarray(full[:, :17])
    back = np.zeros((32, 32), np.float32)
    oracle.lib().orc_fft2d_inverse_half(oracle._ptr(half), 32, 32, oracle._ptr(back))
    assert np.abs(back - blk).max() < 1e-5


@pytest.mark.parametrize("path", CASES, ids=[os.path.basename(p)[:-4] for p in CASES])
def test_oracle_matches_golden(path):
    frames, out, bits, chroma, params = load_case(path)
    got = oracle.run_clip(frames, bits, chroma=chroma, **params)
    for g, o in zip(got, out):
        np.testing.assert_array_equal(g, o)


@pytest.mark.parametrize("path", CASES[:4], ids=[os.path.basename(p)[:-4] for p in CASES[:4]])
def test_oracle_thread_count_invariant(path):
    frames, out, bits, chroma, params = load_case(path)
    got = oracle.run_clip(frames, bits, chroma=chroma, threads=3, **params)
    for g, o in zip(got, out):
        np.testing.assert_array_equal(g, o)


needs_ref = pytest.mark.skipif(not oracle.ref_available(), reason="reference sources not built here")


@needs_ref
@pytest.mark.parametrize("params", [
    {}, {"bt": 4, "sharpen": 0.4, "degrid": 0.5}, {"bt": 0, "kratio": 1.5},
    {"bw": 8, "bh": 4, "ow": 2, "oh": 2}, {"mode": 0, "bw": 32, "bh": 16},
])
def test_oracle_matches_reference_live(params):
    frames = synth.moving_rects(77, 53, 5, 7, lo=16, hi=235, noise=3.0, n_rects=5)
    a = oracle.run_clip(frames, 8, **params)
    b = oracle.run_clip(frames, 8, impl="ref", **params)
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x, y)


@needs_ref
def test_validate_params_matches_reference():
    import ctypes as C
    R = oracle.ref()
    rng = np.random.default_rng(5)
    for _ in range(400):
        kw = dict(bw=int(rng.integers(1, 700)), bh=int(rng.integers(1, 700)), bt=int(rng.integers(-2, 6)),
                  mode=int(rng.integers(-1, 4)), sigma=float(rng.uniform(0, 10)),
                  sharpen=float(rng.choice([0.0, 0.5])), wintype=int(rng.integers(-1, 4)))
        kw["ow"] = int(rng.integers(0, kw["bw"] + 2))
        kw["oh"] = int(rng.integers(0, kw["bh"] + 2))
        w, h, bits = int(rng.integers(1, 4000)), int(rng.integers(1, 3000)), int(rng.choice([8, 10, 16, 32]))
        sp = oracle.script_params(**kw)
        vals = (C.c_double * 37)()
        err1, err2 = C.c_char_p(), C.c_char_p()
        ok_ref = R.ref_validate(C.byref(sp), w, h, bits, vals, C.byref(err1))
        ip = oracle.InternalParams()
        ok_orc = oracle.lib().orc_validate_params(C.byref(sp), w, h, bits, C.byref(ip), C.byref(err2))
        assert ok_ref == ok_orc
        if not ok_ref:
            assert err1.value == err2.value
            continue
        mine = [getattr(ip, f) for f, _ in oracle.InternalParams._fields_]
        assert np.array_equal(np.array(mine, np.float64).astype(np.float32),
                              np.array(list(vals), np.float64).astype(np.float32)), kw


@needs_ref
@pytest.mark.parametrize("params", [{}, {"wintype": 1, "bw": 16, "ow": 6}, {"wintype": 2, "bh": 64},
                                    {"mode": 0}, {"sigma2": 3.0, "sharpen": 0.7, "svr": 0.5}])
def test_tables_match_reference(params):
    import ctypes as C
    sp = oracle.script_params(**params)
    ip = oracle.validate(sp, 200, 120, 8)
    pl = oracle.Plane(200, 120, 8, **params)
    pl.build_degrid()
    for which in range(7):
        n = oracle.ref().ref_get_table(C.byref(sp), 200, 120, 8, 0, 0, which, None)
        ref = np.zeros(max(n, 0), np.float32)
        if n > 0:
            oracle.ref().ref_get_table(C.byref(sp), 200, 120, 8, 0, 0, which, oracle._ptr(ref))
        mine = pl.table(which)
        if which in (1, 2) and ip.mode == 0:
            assert mine.size == 0 and ref.size == 0
            continue
        np.testing.assert_array_equal(mine, ref)
