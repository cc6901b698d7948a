"""The render comparator (fft3dcl_gb300/compare.py): identical share,
difference histogram and the first place of the largest difference, on
integer and float planes, and its Y4M command line."""
import numpy as np

from fft3dcl_gb300 import compare, y4m


def test_integer_histogram_and_worst_place():
    a = [[np.zeros((4, 5), np.uint16), np.zeros((2, 3), np.uint16)] for _ in range(3)]
    b = [[p.copy() for p in f] for f in a]
    b[0][0][0, 0] = 1
    b[1][1][1, 2] = 4
    b[2][0][3, 4] = 4
    st = compare.diff_stats(a, b)
    assert st["samples"] == 3 * (20 + 6)
    assert st["hist"] == {0: 75, 1: 1, 4: 2}
    assert st["identical"] == 75 and abs(st["identical_pct"] - 100 * 75 / 78) < 1e-9
    assert st["max_diff"] == 4 and st["max_at"] == {"frame": 1, "plane": "U"}
    text = compare.report(st)
    assert "identical samples: 75/78" in text and "diff 4: 2 px" in text and "frame 1, plane U" in text


def test_float_bounds():
    a = [[np.zeros((2, 2), np.float32)]]
    b = [[np.array([[0.0, 5e-7], [2e-5, 3e-4]], np.float32)]]
    st = compare.diff_stats(a, b)
    assert st["identical"] == 1
    assert st["within_pct"] == {"1e-06": 50.0, "1e-05": 50.0, "0.0001": 75.0}
    assert abs(st["max_diff"] - 3e-4) < 1e-9 and "hist" not in st


def test_y4m_command_line(tmp_path, capsys):
    frames = [[np.full((8, 16), v, np.uint8), np.full((4, 8), 128, np.uint8), np.full((4, 8), 128, np.uint8)]
              for v in (16, 17)]
    pa, pb = str(tmp_path / "a.y4m"), str(tmp_path / "b.y4m")
    for path, fr in ((pa, frames), (pb, [[f[0] + 1, f[1], f[2]] for f in frames])):
        with y4m.Y4MWriter(path, width=16, height=8, bits=8) as w:
            for f in fr:
                w.write(f)
    assert compare.main([pa, pb]) == 0
    out = capsys.readouterr().out
    assert "frames=2 16x8" in out and "diff 1: 256 px" in out and "max diff: 1 at frame 0, plane Y" in out
