"""The serving loop: streams of different sizes, depths, formats and
parameters run concurrently, tensor-core streams in shared steps, each result
is the same as the stream run alone (bit for bit: the same kernels on the same
inputs), admission follows the HBM budget and slots, and latency figures are
reported."""
import numpy as np
import pytest

import fft3dcl_gb300 as F
from fft3dcl_gb300 import serving, synth

pytestmark = pytest.mark.gpu

SPECS = [
    dict(width=640, height=360, bits=8, frames=9, fps=60.0, seed=11, params=dict(bt=3)),
    dict(width=1280, height=720, bits=10, frames=7, fps=40.0, seed=12, params=dict(bt=4, sharpen=0.3)),
    dict(width=333, height=177, bits=8, frames=6, fps=50.0, seed=13, params=dict(bt=1, bw=16, bh=16)),
    dict(width=960, height=540, bits=10, frames=8, fps=30.0, seed=14, params=dict(bt=2, bw=32, bh=32)),
    dict(width=320, height=240, bits=8, frames=10, fps=45.0, seed=15, params=dict(bt=0, sigma=2.0)),
    # YUV 4:2:0 video streams: one server stream per plane.
    dict(width=480, height=272, fmt="yuv420", bits=8, frames=8, fps=55.0, seed=16, params=dict(bt=3)),
    dict(width=704, height=400, fmt="yuv420", bits=10, frames=7, fps=35.0, seed=17,
         params=dict(bt=4, sharpen=0.2)),
    dict(width=352, height=208, fmt="yuv420", bits=8, frames=6, fps=48.0, seed=18, params=dict(bt=3)),
]


def alone(spec, planes, form):
    """Each plane of the stream through its own Filter, as the plugin would."""
    bits = spec["bits"]
    outs = []
    for p, (w, h, chroma) in enumerate(serving.plane_shapes(spec)):
        seq = [planes[p][n % len(planes[p])] for n in range(spec["frames"])]
        if chroma:
            clip = [[np.zeros((spec["height"], spec["width"]), f.dtype), f, f] for f in seq]
            flt = F.Filter(clip, F.VideoFormat("yuv", bits, 0), form=form, plane=1, **spec["params"])
            k = 1
        else:
            flt = F.Filter([[f] for f in seq], F.VideoFormat("gray", bits, 0), form=form, **spec["params"])
            k = 0
        try:
            outs.append([flt.get_frame(n)[k] for n in range(spec["frames"])])
        finally:
            flt.close()
    return outs


@pytest.mark.parametrize("form", ["tc", "fast"])
def test_mixed_streams_equal_alone(form):
    # Tensor-core streams share steps (one launch per kernel for several
    # streams' planes); the others run on their own CUDA streams. Every output
    # equals the stream run alone, bit for bit.
    frames = [serving.stream_frames(s, distinct=4) for s in SPECS]
    with F.Server(form=form, max_streams=32) as sv:
        outs, st = serving.run(sv, SPECS, frames, realtime=True, timeout_s=120)
    nplanes = sum(len(serving.plane_shapes(s)) * s["frames"] for s in SPECS)
    assert st["frames"] == nplanes
    assert st["video_frames"] == sum(s["frames"] for s in SPECS)
    assert st["p99_ms"] >= st["p50_ms"] > 0.0 and st["server_p99_ms"] > 0.0
    if form == "tc":
        # At this load most steps hold one stream's output; the all-at-once
        # test below fills them.
        assert st["shared_steps"] > 0, st
    else:
        assert st["shared_steps"] == 0
    for spec, fr, got in zip(SPECS, frames, outs):
        ref = alone(spec, fr, form)
        for p, (gp, rp) in enumerate(zip(got, ref)):
            assert len(gp) == len(rp)
            for n, (g, r) in enumerate(zip(gp, rp)):
                np.testing.assert_array_equal(g, r, err_msg=f"{spec['width']}x{spec['height']} plane {p} frame {n}")


def test_shared_steps_all_at_once():
    # Every frame submitted at once (no arrival clock): tensor-core streams
    # of different sizes and depths land in the same steps; results equal
    # the streams run alone.
    specs = [s for s in SPECS if s["params"].get("bt", 3) >= 1 and s["params"].get("bw", 32) == 32]
    frames = [serving.stream_frames(s, distinct=3) for s in specs]
    with F.Server(form="tc", max_streams=32) as sv:
        outs, st = serving.run(sv, specs, frames, realtime=False, timeout_s=120)
    assert st["max_shared"] >= 2, st
    assert st["shared_outputs"] == st["frames"]
    # The scheduler's launching passes are part of the run.
    assert 0.0 < st["scheduler_busy"] <= 1.0, st
    for spec, fr, got in zip(specs, frames, outs):
        for gp, rp in zip(got, alone(spec, fr, "tc")):
            for g, r in zip(gp, rp):
                np.testing.assert_array_equal(g, r)


def test_admission_by_budget_and_slots():
    w, h = 640, 360
    frame = synth.moving_rects(w, h, 1, 3, lo=16, hi=235, noise=2.0)[0]
    with F.Server(form="fast", max_streams=2, hbm_budget=1 << 40) as sv:
        a = sv.open(w, h, 8, 4, bt=3)
        b = sv.open(w, h, 8, 4, bt=3)
        assert a is not None and b is not None
        assert sv.open(w, h, 8, 4, bt=3) is None  # no slot
        sv.close_stream(a)
        c = sv.open(w, h, 8, 4, bt=3)
        assert c is not None
        used = sv.stats()["used_bytes"]
        sv.close_stream(b)
        sv.close_stream(c)
    # A budget that holds one such stream but not two.
    with F.Server(form="fast", max_streams=8, hbm_budget=int(used * 0.75)) as sv:
        a = sv.open(w, h, 8, 4, bt=3)
        assert a is not None
        assert sv.open(w, h, 8, 4, bt=3) is None  # over budget
        for n in range(4):
            assert sv.submit(a, n, frame)
        got = [sv.poll(a, 5000) for _ in range(4)]
        assert [g[0] for g in got] == [0, 1, 2, 3]
        sv.close_stream(a)
        assert sv.open(w, h, 8, 4, bt=3) is not None  # budget freed
