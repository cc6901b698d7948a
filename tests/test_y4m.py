"""Y4M reader/writer (host-only): round trips for 4:2:0 8/10-bit, 4:4:4 and
mono, random access, header handling and malformed files."""
import numpy as np
import pytest

from fft3dcl_gb300 import synth
from fft3dcl_gb300.y4m import Y4MClip, Y4MWriter


def clip420(w, h, n, bits, seed=5):
    if bits == 8:
        y = synth.moving_rects(w, h, n, seed, lo=16, hi=235, noise=2.0)
        c = [synth.moving_rects(w // 2, h // 2, n, seed + k, lo=16, hi=240, noise=1.0, ramp=False) for k in (1, 2)]
    else:
        kw = dict(dtype=np.uint16, maxval=(1 << bits) - 1)
        y = synth.moving_rects(w, h, n, seed, lo=64, hi=900, noise=4.0, **kw)
        c = [synth.moving_rects(w // 2, h // 2, n, seed + k, lo=64, hi=900, noise=2.0, ramp=False, **kw) for k in (1, 2)]
    return [[y[i], c[0][i], c[1][i]] for i in range(n)]


@pytest.mark.parametrize("bits", [8, 10])
def test_roundtrip_420(tmp_path, bits):
    frames = clip420(64, 48, 5, bits)
    p = tmp_path / "a.y4m"
    with Y4MWriter(str(p), width=64, height=48, bits=bits) as w:
        for f in frames:
            w.write(f)
    with Y4MClip(str(p)) as c:
        assert (c.width, c.height, c.bits, c.sub_w, c.sub_h, c.mono) == (64, 48, bits, 1, 1, False)
        assert len(c) == 5
        for n in (3, 0, 4, 3):  # random access, cached and not
            for a, b in zip(c[n], frames[n]):
                np.testing.assert_array_equal(a, b)


def test_roundtrip_mono_and_444(tmp_path):
    y = synth.moving_rects(40, 30, 3, 9, lo=16, hi=235, noise=2.0)
    p = tmp_path / "m.y4m"
    with Y4MWriter(str(p), width=40, height=30, bits=8, mono=True) as w:
        for f in y:
            w.write([f])
    with Y4MClip(str(p)) as c:
        assert c.mono and len(c) == 3 and len(c[0]) == 1
        np.testing.assert_array_equal(c[2][0], y[2])
    q = tmp_path / "f.y4m"
    planes = [[f, f[::-1].copy(), f[:, ::-1].copy()] for f in y]
    with Y4MWriter(str(q), width=40, height=30, bits=8, sub_w=0, sub_h=0) as w:
        for f in planes:
            w.write(f)
    with Y4MClip(str(q)) as c:
        assert (c.sub_w, c.sub_h) == (0, 0)
        for a, b in zip(c[1], planes[1]):
            np.testing.assert_array_equal(a, b)


def test_header_kept_and_frame_parameters(tmp_path):
    p = tmp_path / "h.y4m"
    frame = np.arange(16 * 8, dtype=np.uint8).reshape(8, 16)
    with open(p, "wb") as f:
        f.write(b"YUV4MPEG2 W16 H8 F30000:1001 It A1:1 Cmono XYSCSS=MONO\n")
        f.write(b"FRAME Ixyz\n" + frame.tobytes())
    with Y4MClip(str(p)) as c:
        assert c.header.endswith("XYSCSS=MONO") and len(c) == 1
        np.testing.assert_array_equal(c[0][0], frame)


def test_malformed_files_rejected(tmp_path):
    p = tmp_path / "bad.y4m"
    p.write_bytes(b"NOTY4M W4 H4\n")
    with pytest.raises(ValueError):
        Y4MClip(str(p))
    q = tmp_path / "trunc.y4m"
    q.write_bytes(b"YUV4MPEG2 W4 H4 Cmono\nFRAME\n" + b"\0" * 10)
    with pytest.raises(ValueError):
        Y4MClip(str(q))
