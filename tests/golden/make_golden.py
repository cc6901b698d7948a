"""Generate the golden vectors of tests/golden/ from the reference itself.

Runs the reference's own CPU backend (src/cpu/*.cpp + src/params.h of
HumbleUser33/FFT3dCL, compiled where it lies by `make -C oracle ref` into
oracle/_ref/) on small seeded clips and stores inputs, parameters and outputs
as compressed .npz files. The tests pin the C oracle to these vectors, so the
oracle stays pinned on machines where the reference sources are absent.

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from fft3dcl_gb300 import synth  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))
W, H, N = 40, 32, 6

# (name, sample kind, bits, chroma, params): every temporal mode, degrid on
# and off, sharpen, sigma pattern, beta, window types, general overlap,
# mode 0, 10-bit, float and chroma centering.
CASES = [
    ("default_bt3", "u8", 8, False, {}),
    ("bt2", "u8", 8, False, {"bt": 2}),
    ("bt4_sharpen", "u8", 8, False, {"bt": 4, "sharpen": 0.4}),
    ("bt1", "u8", 8, False, {"bt": 1}),
    ("bt0_kalman", "u8", 8, False, {"bt": 0}),
    ("btm1_sharpen", "u8", 8, False, {"bt": -1, "sharpen": 1.0}),
    ("pattern", "u8", 8, False, {"sigma2": 1.5, "sigma3": 2.5, "sigma4": 3.0}),
    ("beta2_nodegrid", "u8", 8, False, {"beta": 2.0, "degrid": 0.0}),
    ("wintype1_bw16", "u8", 8, False, {"bw": 16, "bh": 16, "wintype": 1}),
    ("wintype2_bw8x16", "u8", 8, False, {"bw": 8, "bh": 16, "wintype": 2}),
    ("overlap_general", "u8", 8, False, {"bw": 16, "bh": 16, "ow": 4, "oh": 6}),
    ("mode0", "u8", 8, False, {"mode": 0, "bw": 16, "bh": 16}),
    ("p10_bt4", "u16", 10, False, {"bt": 4, "sharpen": 0.4, "sigma": 3.0}),
    ("p16_bt3", "u16", 16, False, {"sigma": 4.0}),
    ("float_kalman_bw64_pattern", "f32", 32, False,
     {"bt": 0, "bw": 64, "bh": 64, "sigma2": 1.5, "sigma3": 2.5, "sigma4": 3.0}),
    ("float_bt2", "f32", 32, False, {"bt": 2, "sharpen": -0.3}),
    ("chroma_u8_bt3", "u8", 8, True, {}),
    ("chroma_p10_bt1", "u16", 10, True, {"bt": 1}),
]


def frames_for(kind: str, seed: int):
    if kind == "u8":
        return synth.moving_rects(W, H, N, seed, lo=16, hi=235, noise=6.0, n_rects=4)
    if kind == "u16":
        return synth.moving_rects(W, H, N, seed, lo=64, hi=940, noise=24.0, dtype=np.uint16,
                                  maxval=1023, n_rects=4)
    return synth.moving_rects(W, H, N, seed, lo=0.06, hi=0.92, noise=6 / 255, dtype=np.float32,
                              n_rects=4, cuts=(3,))


def main():
    oracle.build(ref=True)
    if not oracle.ref_available():
        raise SystemExit("the reference CPU backend is not available here")
    for k, (name, kind, bits, chroma, params) in enumerate(CASES):
        frames = frames_for(kind, 1000 + k)
        if kind == "u16" and bits == 16:
            frames = [np.clip(f.astype(np.int64) * 64, 0, 65535).astype(np.uint16) for f in frames]
        out = oracle.run_clip(frames, bits, chroma=chroma, impl="ref", **params)
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), frames=np.stack(frames),
                            out=np.stack(out), bits=bits, chroma=int(chroma),
                            params=json.dumps(params))
    x = np.arange(8).astype(np.complex64)
    kat = oracle.fft1d(x, impl="ref")
    np.savez_compressed(os.path.join(HERE, "fft8_kat.npz"), x=x, y=kat)
    print(f"wrote {len(CASES)} cases to {HERE}")


if __name__ == "__main__":
    main()
