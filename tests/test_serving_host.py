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
        assert s["bits"] in (8, 10)
        assert s["params"]["bt"] in (1, 3, 4)
        assert s["params"]["bw"] in (16, 32) and s["params"]["bh"] == s["params"]["bw"]
        assert 24.0 <= s["fps"] <= 60.0
        assert s["frames"] == 120
    assert len({(s["width"], s["bits"]) for s in a}) > 3  # a real mix


def test_stream_frames_are_seeded_and_cycle():
    s = dict(width=64, height=48, bits=10, frames=9, fps=30.0, seed=3, params={})
    f1 = serving.stream_frames(s, distinct=4)
    f2 = serving.stream_frames(s, distinct=4)
    assert len(f1) == 4 and all((a == b).all() for a, b in zip(f1, f2))
    assert f1[0].dtype.name == "uint16" and int(f1[0].max()) <= 1023


@pytest.mark.skipif(torch.cuda.is_available(), reason="checks the behaviour without a GPU")
def test_server_needs_a_gpu():
    with pytest.raises(F.F3DError, match="CUDA"):
        F.Server()
