"""The command-line driver on a .y4m clip gives the frames the Python filter
gives for the same clip and parameters."""
import numpy as np
import pytest

import fft3dcl_gb300 as F
from fft3dcl_gb300 import __main__ as cli
from fft3dcl_gb300.y4m import Y4MClip, Y4MWriter
from test_y4m import clip420

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("bits,form", [(8, "tc"), (10, "fast")])
def test_cli_matches_filter(tmp_path, bits, form):
    frames = clip420(160, 96, 6, bits, seed=17)
    src, dst = tmp_path / "in.y4m", tmp_path / "out.y4m"
    with Y4MWriter(str(src), width=160, height=96, bits=bits) as w:
        for f in frames:
            w.write(f)
    assert cli.main([str(src), str(dst), "--form", form, "--plane", "4", "--bt", "3", "--sigma", "2.5"]) == 0
    flt = F.Filter(frames, F.VideoFormat("yuv", bits, 0, 1, 1), form=form, plane=4, bt=3, sigma=2.5)
    try:
        ref = [flt.get_frame(n) for n in range(len(frames))]
    finally:
        flt.close()
    with Y4MClip(str(dst)) as out:
        assert len(out) == len(frames)
        for n in range(len(frames)):
            for a, b in zip(out[n], ref[n]):
                np.testing.assert_array_equal(a, b)


def test_cli_half_spectra_matches_filter(tmp_path):
    frames = clip420(160, 96, 5, 8, seed=19)
    src, dst = tmp_path / "in.y4m", tmp_path / "out.y4m"
    with Y4MWriter(str(src), width=160, height=96, bits=8) as w:
        for f in frames:
            w.write(f)
    assert cli.main([str(src), str(dst), "--form", "tc", "--plane", "4", "--bt", "3", "--precision", "0",
                     "--half-spectra"]) == 0
    flt = F.Filter(frames, F.VideoFormat("yuv", 8, 0, 1, 1), form="tc", plane=4, bt=3, precision=0,
                   flags=F.FLAG_HALF_SPECTRA)
    try:
        assert all(e.info().half_spectra for e in flt.engines)
        ref = [flt.get_frame(n) for n in range(len(frames))]
    finally:
        flt.close()
    with Y4MClip(str(dst)) as out:
        for n in range(len(frames)):
            for a, b in zip(out[n], ref[n]):
                np.testing.assert_array_equal(a, b)
