"""Seeded synthetic clips: the stand-in for real video in tests and benchmarks.

No public dataset is named for this path, so every workload is generated from a
seed: a horizontal luma ramp, axis-aligned rectangles at uniform levels that
translate by a few pixels per frame (wrapping at the borders), optional hard
scene cuts that redraw the layout, and i.i.d. Gaussian noise, rounded and
clipped to the sample format. 4:2:0 chroma planes are generated the same way
at half resolution around mid-grey. Frames are plain numpy arrays.
"""
from __future__ import annotations

import numpy as np


def _layout(rng, w, h, n_rects, lo, hi):
    rects = []
    for _ in range(n_rects):
        rw = int(rng.integers(max(1, w // 16), max(2, w // 4) + 1))
        rh = int(rng.integers(max(1, h // 16), max(2, h // 4) + 1))
        x0 = int(rng.integers(0, w))
        y0 = int(rng.integers(0, h))
        level = float(rng.uniform(lo, hi))
        vel = [(-2, -2), (-2, 0), (-2, 2), (0, -2), (0, 2), (2, -2), (2, 0), (2, 2)]
        vx, vy = vel[int(rng.integers(0, len(vel)))]
        rects.append((rw, rh, x0, y0, level, vx, vy))
    return rects


def moving_rects(width: int, height: int, frames: int, seed: int, *, lo: float, hi: float,
                 noise: float, dtype=np.uint8, maxval: float | None = None, n_rects: int = 12,
                 ramp: bool = True, cuts: tuple[int, ...] = (), scale: float = 1.0) -> list[np.ndarray]:
    """One plane of a seeded moving-rectangle clip.

    lo/hi: level range of the ramp and the rectangles (sample units).
    noise: Gaussian noise standard deviation (sample units).
    dtype: uint8, uint16 (values clipped to [0, maxval]) or float32 (divided by
    `scale`, not clipped).
    cuts: frame indices at which a new random layout starts (scene cuts).
    """
    rng = np.random.default_rng(seed)
    if maxval is None:
        maxval = 255.0 if dtype == np.uint8 else 65535.0
    xs = np.arange(width, dtype=np.float64)
    base = lo + (hi - lo) * xs / max(1, width - 1) if ramp else np.full(width, 0.5 * (lo + hi))
    base = np.broadcast_to(base, (height, width))
    rects = _layout(rng, width, height, n_rects, lo, hi)
    out = []
    t0 = 0
    for f in range(frames):
        if f in cuts:
            rects = _layout(rng, width, height, n_rects, lo, hi)
            t0 = f
        img = np.array(base, dtype=np.float64)
        t = f - t0
        for (rw, rh, x0, y0, level, vx, vy) in rects:
            xa = (x0 + vx * t) % width
            ya = (y0 + vy * t) % height
            cols = (xa + np.arange(rw)) % width
            rows = (ya + np.arange(rh)) % height
            img[np.ix_(rows, cols)] = level
        img = img + rng.normal(0.0, noise, size=img.shape)
        if dtype == np.float32:
            out.append((img / scale).astype(np.float32))
        else:
            out.append(np.clip(np.rint(img), 0, maxval).astype(dtype))
    return out


def clip_gray8(width=640, height=360, frames=16, seed=0xF3D0 + 0, noise=2.0):
    """640x360 GRAY8 plain-method clip: ramp 16..235, 12 rectangles, noise 2 LSB."""
    return moving_rects(width, height, frames, seed, lo=16, hi=235, noise=noise, dtype=np.uint8)


def clip_yuv420p8(width=1920, height=1080, frames=32, seed=0xF3D0 + 1):
    """YUV420P8: luma ramp + rectangles 16..235 with noise 2.5, chroma at half
    resolution 16..240 around 128 with noise 1.5. Returns (Y, U, V) lists."""
    y = moving_rects(width, height, frames, seed, lo=16, hi=235, noise=2.5, dtype=np.uint8)
    u = moving_rects(width // 2, height // 2, frames, seed + 101, lo=16, hi=240, noise=1.5,
                     dtype=np.uint8, ramp=False)
    v = moving_rects(width // 2, height // 2, frames, seed + 202, lo=16, hi=240, noise=1.5,
                     dtype=np.uint8, ramp=False)
    return y, u, v


def clip_yuv420p10_luma(width=3840, height=2160, frames=48, seed=0xF3D0 + 2):
    """3840x2160 10-bit luma: ramp + rectangles in 64..940, noise 12 LSB."""
    return moving_rects(width, height, frames, seed, lo=64, hi=940, noise=12.0, dtype=np.uint16,
                        maxval=1023)


def clip_grays(width=1280, height=720, frames=64, seed=0xF3D0 + 3, cuts=(20, 45)):
    """GRAYS float clip in [0,1]: rectangles with scene cuts, noise 2/255."""
    return moving_rects(width, height, frames, seed, lo=0.0625, hi=0.92, noise=2.0 / 255.0,
                        dtype=np.float32, cuts=cuts)
