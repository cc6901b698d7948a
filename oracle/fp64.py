"""FP64 restatement of the forward block transform (test infrastructure only).

The spectra every arithmetic form computes, evaluated in double precision:
the mode-1 block grid (src/cpu/reference.cpp:19-58), block gather with D3D
mirror addressing (src/cpu/reference.cpp:10-17, :140-170), sample conversion
(src/cpu/reference.cpp:82-105), the chroma offset (:70-79), the separable
analysis window (src/cpu/tables.cpp:21-105) formed in double, and the
unnormalised 2D real DFT (src/cpu/fft.cpp:68-86) evaluated by numpy's float64
FFT. The forms' spectral error is measured against it; only tests import it.
"""
from __future__ import annotations

import numpy as np

from . import script_params, validate


def window_axes(bw: int, bh: int, ow: int, oh: int, wintype: int) -> tuple[np.ndarray, np.ndarray]:
    """x and y factors of the mode-1 analysis window, in double."""

    def ramp(o: int) -> np.ndarray:
        i = np.arange(o)
        hc = np.cos(np.pi * (i - o + 0.5) / (o * 2.0))
        if wintype == 1:
            return np.sqrt(hc)
        if wintype == 2:
            return np.ones(o)
        return hc

    def axis(n: int, o: int) -> np.ndarray:
        r = ramp(o)
        w = np.ones(n)
        w[:o] = r
        w[n - o:] = r[::-1]
        return w

    return axis(bw, ow), axis(bh, oh)


def mirror(x: np.ndarray, w: int) -> np.ndarray:
    p = np.mod(x, 2 * w)
    return np.where(p >= w, 2 * w - 1 - p, p)


def spectra_fp64(plane: np.ndarray, bits: int, chroma: bool = False, **params) -> np.ndarray:
    """Half spectra [nblocks, bh, bw/2+1] (complex128) of a mode-1 plane."""
    h, w = plane.shape
    ip = validate(script_params(**params), w, h, bits)
    if ip.mode != 1:
        raise ValueError("the FP64 restatement covers mode 1")
    bw, bh, ow, oh = ip.bw, ip.bh, ip.ow, ip.oh
    if plane.dtype == np.uint8:
        v = plane.astype(np.float64) / 255.0
    elif plane.dtype == np.uint16:
        v = plane.astype(np.float64) * (2.0 ** (16 - bits)) / 65535.0
    else:
        v = plane.astype(np.float64)
    c = 0.0
    if chroma and plane.dtype != np.float32:
        c = 128.0 / 255.0 if bits <= 8 else 32768.0 / 65535.0
    wx, wy = window_axes(bw, bh, ow, oh, ip.wintype)
    win = wy[:, None] * wx[None, :]
    ncols, nrows = 2 * ip.nx, 2 * ip.ny
    n = np.arange(ncols)
    m = np.arange(nrows)
    bx = -ow + n * (bw - ow)
    by = -oh + m * (bh - oh)
    xs = mirror(bx[:, None] + np.arange(bw)[None, :], w)  # [ncols, bw]
    ys = mirror(by[:, None] + np.arange(bh)[None, :], h)  # [nrows, bh]
    out = np.empty((nrows * ncols, bh, bw // 2 + 1), np.complex128)
    for r in range(nrows):
        blocks = (v[ys[r]][:, xs] - c).transpose(1, 0, 2) * win  # [ncols, bh, bw]
        out[r * ncols:(r + 1) * ncols] = np.fft.rfft2(blocks)
    return out


def spectral_error(spec: np.ndarray, ref: np.ndarray) -> dict:
    """Relative RMS error over all bins and the largest bin error relative to
    the largest reference magnitude."""
    d = spec.astype(np.complex128) - ref
    return {"rel_rms": float(np.sqrt(np.sum(np.abs(d) ** 2) / np.sum(np.abs(ref) ** 2))),
            "max_rel": float(np.abs(d).max() / np.abs(ref).max())}
