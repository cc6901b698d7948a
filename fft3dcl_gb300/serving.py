"""Serving workload: streams of mixed resolution, depth and parameters whose
frames arrive at their own rates, driven through a Server.

``mixed_streams`` draws the stream set (resolutions 640x360 .. 3840x2160,
8- or 10-bit luma planes, bt in {1, 3, 4}, bw in {16, 32}, 24-60 frames/s),
``run`` opens the streams, submits every stream's frames at Poisson arrival
times, collects the outputs as they finish and returns them with the
server's latency figures.
"""
from __future__ import annotations

import time

import numpy as np

from . import Server, synth

RESOLUTIONS = [(640, 360), (1280, 720), (1920, 1080), (3840, 2160)]


def mixed_streams(n: int = 16, frames: int = 120, seed: int = 0xF3D0 + 4) -> list[dict]:
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        w, h = RESOLUTIONS[int(rng.integers(len(RESOLUTIONS)))]
        bits = int(rng.choice([8, 10]))
        bw = int(rng.choice([16, 32]))
        out.append(dict(width=w, height=h, bits=bits, frames=frames, fps=float(rng.uniform(24.0, 60.0)),
                        seed=seed + 1 + i, params=dict(sigma=2.5, bt=int(rng.choice([1, 3, 4])), bw=bw, bh=bw)))
    return out


def stream_frames(spec: dict, distinct: int = 8) -> list[np.ndarray]:
    """`distinct` seeded frames of the stream; frame n is frames[n % distinct]."""
    w, h, bits = spec["width"], spec["height"], spec["bits"]
    k = min(distinct, spec["frames"])
    if bits <= 8:
        return synth.moving_rects(w, h, k, spec["seed"], lo=16, hi=235, noise=2.5)
    return synth.moving_rects(w, h, k, spec["seed"], lo=64, hi=940, noise=10.0, dtype=np.uint16, maxval=1023)


def run(server: Server, specs: list[dict], frames: list[list[np.ndarray]], realtime: bool = True,
        timeout_s: float = 120.0, seed: int = 1) -> tuple[list[list[np.ndarray]], dict]:
    """Opens every stream (retrying while the server is full), submits frame
    n of stream i at its Poisson arrival time (or as fast as the server takes
    them when not realtime), polls outputs, closes finished streams. Returns
    each stream's outputs in frame order and the server statistics."""
    rng = np.random.default_rng(seed)
    due = []
    for s in specs:
        gaps = rng.exponential(1.0 / s["fps"], s["frames"]) if realtime else np.zeros(s["frames"])
        due.append(np.cumsum(gaps))
    sid = [None] * len(specs)
    # Clients connect first: every stream the server admits now is opened
    # before the arrival clock starts; the others open as slots free up.
    for i, s in enumerate(specs):
        sid[i] = server.open(s["width"], s["height"], s["bits"], s["frames"], **s["params"])
    t0 = time.perf_counter()
    nxt = [0] * len(specs)
    outs: list[list[np.ndarray]] = [[] for _ in specs]
    done = [False] * len(specs)
    while not all(done):
        if time.perf_counter() - t0 > timeout_s:
            raise TimeoutError("serving run did not finish")
        busy = True
        for i, s in enumerate(specs):
            if done[i]:
                continue
            if sid[i] is None:
                sid[i] = server.open(s["width"], s["height"], s["bits"], s["frames"], **s["params"])
                if sid[i] is None:
                    continue
            now = time.perf_counter() - t0
            while nxt[i] < s["frames"] and due[i][nxt[i]] <= now:
                if not server.submit(sid[i], nxt[i], frames[i][nxt[i] % len(frames[i])]):
                    break
                nxt[i] += 1
                busy = False
            while True:
                r = server.poll(sid[i], 0)
                if r is None:
                    break
                outs[i].append(r[1])
                busy = False
            if len(outs[i]) == s["frames"]:
                server.close_stream(sid[i])
                done[i] = True
        if busy:
            time.sleep(0.0002)
    return outs, server.stats()
