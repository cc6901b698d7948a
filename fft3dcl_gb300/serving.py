"""Serving workload: video streams of mixed resolution, format and parameters
whose frames arrive at their own rates, driven through a Server.

``mixed_streams`` draws the stream set: resolutions 640x360 .. 3840x2160,
YUV420P8 or YUV420P10 with every plane filtered, bt in {1, 3, 4}, bw in
{16, 32}, 24-60 frames/s. A video stream is one server stream per plane (Y,
then U and V at half resolution with the chroma offset). ``run`` gives each
video stream a client that opens its planes' streams, submits frame n of
every plane at its Poisson arrival time (scaled by ``rate``) from one thread,
collects the outputs as they finish from another and closes the streams; it
returns the outputs and the latency figures:

* per video frame, from the scheduled arrival of the last frame its temporal
  window needs to the last of its planes' outputs in host memory
  (``p50_ms``, ``p99_ms``: includes any wait for a free input slot when the
  server is saturated);
* per video frame, from the arrival of the last input plane its windows need
  at the server to its last output (``server_p50_ms``, ``server_p99_ms``);
* delivered and offered video frames per second, each the sum over the
  streams of their frames over the span until their last output, and over
  the span of their scheduled arrivals.

The server and the clients use the same monotonic clock.
"""
from __future__ import annotations

import sys
import threading
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
        out.append(dict(width=w, height=h, fmt="yuv420", bits=bits, frames=frames,
                        fps=float(rng.uniform(24.0, 60.0)), seed=seed + 1 + i,
                        params=dict(sigma=2.5, bt=int(rng.choice([1, 3, 4])), bw=bw, bh=bw)))
    return out


def plane_shapes(spec: dict) -> list[tuple[int, int, bool]]:
    """(width, height, chroma) of each plane of the stream's format."""
    w, h = spec["width"], spec["height"]
    if spec.get("fmt", "gray") == "yuv420":
        return [(w, h, False), (w // 2, h // 2, True), (w // 2, h // 2, True)]
    return [(w, h, False)]


def stream_frames(spec: dict, distinct: int = 8) -> list[list[np.ndarray]]:
    """`distinct` seeded frames of each plane of the stream; frame n of plane
    p is planes[p][n % distinct]."""
    bits = spec["bits"]
    k = min(distinct, spec["frames"])
    out = []
    for p, (w, h, chroma) in enumerate(plane_shapes(spec)):
        seed = spec["seed"] + 101 * p
        if bits <= 8:
            lo, hi = (16, 240) if chroma else (16, 235)
            out.append(synth.moving_rects(w, h, k, seed, lo=lo, hi=hi, noise=1.5 if chroma else 2.5,
                                          ramp=not chroma))
        else:
            lo, hi = (64, 960) if chroma else (64, 940)
            out.append(synth.moving_rects(w, h, k, seed, lo=lo, hi=hi, noise=6.0 if chroma else 10.0,
                                          dtype=np.uint16, maxval=(1 << bits) - 1, ramp=not chroma))
    return out


def _client(server: Server, spec: dict, planes: list[list[np.ndarray]], due_ms: np.ndarray, res: dict,
            timeout_s: float, start: threading.Event, keep: bool):
    """One video stream: opens its planes' streams, then a submitter (this
    thread) and a poller thread, so that copying an output out never delays
    the next frame's submission."""
    shapes = plane_shapes(spec)
    nf = spec["frames"]
    sids: list[int | None] = [None] * len(shapes)
    deadline = time.monotonic() + timeout_s
    # Connect before the arrival clock starts; retry while the server is full.
    while any(s is None for s in sids):
        for p, (w, h, chroma) in enumerate(shapes):
            if sids[p] is None:
                sids[p] = server.open(w, h, spec["bits"], nf, chroma=chroma, **spec["params"])
        if any(s is None for s in sids):
            if time.monotonic() > deadline:
                raise TimeoutError("stream not admitted")
            time.sleep(0.001)
    outs = [[None] * nf for _ in shapes]
    ready = np.zeros((len(shapes), nf))
    done = np.zeros((len(shapes), nf))
    submitted = np.zeros(nf)
    scratch = [np.empty((h, w), planes[p][0].dtype) for p, (w, h, _) in enumerate(shapes)]
    perr = []

    def poller():
        try:
            for n in range(nf):
                for p in range(len(shapes)):
                    while True:
                        if time.monotonic() > deadline:
                            raise TimeoutError("serving run did not finish")
                        r = server.poll_timed(sids[p], 20, None if keep else scratch[p])
                        if r is not None:
                            break
                    k, img, t_ready, t_done = r
                    if keep:
                        outs[p][k] = img
                    ready[p, k], done[p, k] = t_ready, t_done
        except BaseException as e:
            perr.append(e)

    res["opened"] = True
    start.wait()
    t0 = res["t0"]
    pt = threading.Thread(target=poller, daemon=True)
    pt.start()
    for n in range(nf):
        wait = t0 + due_ms[n] / 1000.0 - time.monotonic()
        if wait > 0:
            time.sleep(wait)
        for p in range(len(shapes)):
            while not server.submit(sids[p], n, planes[p][n % len(planes[p])]):
                if time.monotonic() > deadline or perr:
                    raise perr[0] if perr else TimeoutError("serving run did not finish")
                time.sleep(0.0001)
        submitted[n] = time.monotonic() * 1000.0
    pt.join(max(0.0, deadline - time.monotonic()))
    if perr:
        raise perr[0]
    if pt.is_alive():
        raise TimeoutError("serving run did not finish")
    for s in sids:
        server.close_stream(s)
    res.update(outs=outs, ready=ready, done=done, submitted=submitted)


def run(server: Server, specs: list[dict], frames: list[list[list[np.ndarray]]], realtime: bool = True,
        rate: float = 1.0, timeout_s: float = 120.0, seed: int = 1,
        keep_outputs: bool = True) -> tuple[list[list[list[np.ndarray]]], dict]:
    """Runs every video stream through the server, two client threads each.
    frames[i] are stream i's planes (stream_frames). Frame arrivals are
    Poisson at the stream's fps times `rate` (all at once when not
    realtime). Returns outs[i][p][n] (stream i, plane p, frame n; None when
    keep_outputs is False) and the statistics."""
    rng = np.random.default_rng(seed)
    due = []
    for s in specs:
        gaps = rng.exponential(1000.0 / (s["fps"] * rate), s["frames"]) if realtime else np.zeros(s["frames"])
        due.append(np.cumsum(gaps))
    start = threading.Event()
    res = [dict() for _ in specs]
    errors = []

    def target(i):
        try:
            _client(server, specs[i], frames[i], due[i], res[i], timeout_s, start, keep_outputs)
        except BaseException as e:  # reported after the join
            errors.append(e)

    threads = [threading.Thread(target=target, args=(i,), daemon=True) for i in range(len(specs))]
    # The client threads share the interpreter lock; a short switch interval
    # keeps one thread's Python work from delaying another's submit by the
    # default 5 ms.
    switch = sys.getswitchinterval()
    sys.setswitchinterval(1e-4)
    for t in threads:
        t.start()
    t_wait = time.monotonic() + timeout_s
    while not all(r.get("opened") for r in res) and not errors and time.monotonic() < t_wait:
        time.sleep(0.001)
    t0 = time.monotonic()
    for r in res:
        r["t0"] = t0
    start.set()
    for t in threads:
        t.join(timeout_s)
    sys.setswitchinterval(switch)
    if errors:
        raise errors[0]
    if any(t.is_alive() for t in threads):
        raise TimeoutError("serving clients did not finish")
    # Per video frame: from the scheduled arrival of the last frame its
    # temporal window needs (frame n + bt - 1 - current, clamped to the clip;
    # src/fft3dcl.cpp:319-330), and from that frame's arrival at the server,
    # to its last plane's output.
    lat, lat_srv, lag, last_done = [], [], [], 0.0
    offered, delivered = 0.0, 0.0
    for i, r in enumerate(res):
        fin = r["done"].max(axis=0)
        # Per stream: frames over the span of their scheduled arrivals, and
        # over the span until the last output (all frames at once: 0).
        span_due, span_done = float(due[i][-1]), float(fin.max()) - t0 * 1000.0
        if span_due > 0:
            offered += specs[i]["frames"] / (span_due / 1000.0)
        if span_done > 0:
            delivered += specs[i]["frames"] / (span_done / 1000.0)
        nf = specs[i]["frames"]
        bm = specs[i]["params"].get("bt", 3)
        need = bm if bm >= 2 else 1
        cur = 0 if bm == 1 else (2 if bm == 4 else (1 if bm >= 2 else 0))
        last = np.minimum(np.arange(nf) - cur + need - 1, nf - 1)
        lat.append(fin - (t0 * 1000.0 + due[i][last]))
        lat_srv.append(fin - r["ready"].max(axis=0))
        lag.append(r["submitted"] - (t0 * 1000.0 + due[i]))
        last_done = max(last_done, float(fin.max()))
    lat = np.concatenate(lat)
    lat_srv = np.concatenate(lat_srv)
    lag = np.concatenate(lag)
    nframes = sum(s["frames"] for s in specs)
    seconds = (last_done - t0 * 1000.0) / 1000.0
    st = server.stats()
    st.update(
        video_frames=nframes, seconds=seconds, frames_per_s=delivered,
        offered_frames_per_s=offered if realtime else None,
        p50_ms=float(np.percentile(lat, 50)), p99_ms=float(np.percentile(lat, 99)), max_ms=float(lat.max()),
        server_p50_ms=float(np.percentile(lat_srv, 50)), server_p99_ms=float(np.percentile(lat_srv, 99)),
        submit_lag_p99_ms=float(np.percentile(lag, 99)) if realtime else None,
        plane_p50_ms=st["p50_ms"], plane_p99_ms=st["p99_ms"],
        scheduler_busy=st["busy_ms"] / 1000.0 / seconds if seconds > 0 else None)
    return [r["outs"] for r in res], st
