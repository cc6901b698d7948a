"""Host side of the serving workload and of the batch and server wrappers:
the stream mix is seeded and within the specified ranges, and without a
GPU the server and batch refuse to start (no CPU fallback)."""
import pytest
import torch

import fft3dcl_gb300 as F
from fft3dcl_gb300 import serving


def test_mixed_streams_follow_the_serving_spec():
    a = serving.mixed_streams(16, 120)
    assert a == serving.mixed_streams(16, 120)  # seeded
    assert len(a) == 16
    for s in a:
        assert (s["width"], s["height"]) in serving.RESOLUTIONS
        assert s["fmt"] == "yuv420" and s["bits"] in (8, 10)
        assert s["params"]["bt"] in (1, 3, 4)
        assert s["params"]["bw"] in (16, 32) and s["params"]["bh"] == s["params"]["bw"]
        assert 24.0 <= s["fps"] <= 60.0
        assert s["frames"] == 120
        w, h = s["width"], s["height"]
        assert serving.plane_shapes(s) == [(w, h, False), (w // 2, h // 2, True), (w // 2, h // 2, True)]
    assert len({(s["width"], s["bits"]) for s in a}) > 3  # a real mix


def test_stream_frames_are_seeded_and_cycle():
    s = dict(width=64, height=48, fmt="yuv420", bits=10, frames=9, fps=30.0, seed=3, params={})
    f1 = serving.stream_frames(s, distinct=4)
    f2 = serving.stream_frames(s, distinct=4)
    assert len(f1) == 3 and all(len(p) == 4 for p in f1)
    assert all((a == b).all() for p1, p2 in zip(f1, f2) for a, b in zip(p1, p2))
    assert f1[0][0].shape == (48, 64) and f1[1][0].shape == (24, 32)
    assert f1[0][0].dtype.name == "uint16" and int(max(p[0].max() for p in f1)) <= 1023
    g = serving.stream_frames(dict(s, fmt="gray", bits=8), distinct=2)
    assert len(g) == 1 and g[0][0].dtype.name == "uint8"


@pytest.mark.skipif(torch.cuda.is_available(), reason="checks the behaviour without a GPU")
def test_server_needs_a_gpu():
    with pytest.raises(F.F3DError, match="CUDA"):
        F.Server()
