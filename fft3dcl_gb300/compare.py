"""Sample-by-sample comparison of two renders of the same clip.

The portable counterpart of the reference's A/B tool (tools/compare.py of
HumbleUser33/FFT3dCL, which decodes two lossless renders with ffmpeg): the
share of identical samples, a histogram of the absolute differences, and the
largest difference with the frame and plane where it first occurs. Integer
samples are compared in LSB; float samples report the largest absolute
difference and the share within given bounds instead of a histogram.

    python -m fft3dcl_gb300.compare a.y4m b.y4m
"""
from __future__ import annotations

import sys
from collections.abc import Sequence

import numpy as np

PLANE_NAMES = ("Y", "U", "V")


def diff_stats(a: Sequence[Sequence[np.ndarray]], b: Sequence[Sequence[np.ndarray]],
               float_bounds: Sequence[float] = (1e-6, 1e-5, 1e-4)) -> dict:
    """a[n][p], b[n][p]: plane p of frame n of the two renders (same shapes
    and dtypes). Returns samples, identical (count and percent), max_diff and
    where it first occurs, and for integer samples hist: {diff: count} for
    every difference that occurs; for float samples within: {bound: percent
    of samples with |diff| <= bound} and rms."""
    total = identical = 0
    worst, where = 0.0, None
    hist: dict[int, int] = {}
    within = {float(t): 0 for t in float_bounds}
    sq = 0.0
    is_float = None
    for n, (fa, fb) in enumerate(zip(a, b)):
        for p, (x, y) in enumerate(zip(fa, fb)):
            if x.shape != y.shape or x.dtype != y.dtype:
                raise ValueError(f"frame {n} plane {p}: shapes or sample types differ")
            is_float = x.dtype.kind == "f"
            d = np.abs(x.astype(np.float64) - y.astype(np.float64))
            total += d.size
            identical += int(np.count_nonzero(x == y))
            m = float(d.max()) if d.size else 0.0
            if m > worst:
                worst, where = m, (n, p)
            if is_float:
                sq += float((d * d).sum())
                for t in within:
                    within[t] += int(np.count_nonzero(d <= t))
            else:
                vals, cnts = np.unique(d.astype(np.int64), return_counts=True)
                for v, c in zip(vals.tolist(), cnts.tolist()):
                    hist[v] = hist.get(v, 0) + c
    out = {"samples": total, "identical": identical,
           "identical_pct": 100.0 * identical / total if total else 100.0,
           "max_diff": worst if is_float else int(worst),
           "max_at": None if where is None else {"frame": where[0], "plane": PLANE_NAMES[where[1]]
                                                 if where[1] < 3 else where[1]}}
    if is_float:
        out["rms"] = float(np.sqrt(sq / total)) if total else 0.0
        out["within_pct"] = {str(t): 100.0 * c / total for t, c in within.items()}
    else:
        out["hist"] = {int(k): int(v) for k, v in sorted(hist.items())}
    return out


def report(st: dict) -> str:
    """The statistics as the reference tool prints them."""
    lines = [f"identical samples: {st['identical']}/{st['samples']} ({st['identical_pct']:.2f}%)"]
    for d, c in st.get("hist", {}).items():
        if d > 0:
            lines.append(f"  diff {d}: {c} px ({100.0 * c / st['samples']:.4f}%)")
    for t, pct in st.get("within_pct", {}).items():
        lines.append(f"  |diff| <= {t}: {pct:.4f}%")
    at = st["max_at"]
    lines.append(f"max diff: {st['max_diff']}" + (f" at frame {at['frame']}, plane {at['plane']}" if at else ""))
    return "\n".join(lines)


def main(argv: list[str]) -> int:
    if len(argv) != 2:
        print("usage: python -m fft3dcl_gb300.compare a.y4m b.y4m", file=sys.stderr)
        return 2
    from .y4m import Y4MClip
    with Y4MClip(argv[0]) as ca, Y4MClip(argv[1]) as cb:
        if (ca.width, ca.height, ca.shapes, ca.bits) != (cb.width, cb.height, cb.shapes, cb.bits):
            print("the two clips differ in geometry or format", file=sys.stderr)
            return 1
        n = min(len(ca), len(cb))
        print(f"frames={n} {ca.width}x{ca.height} {ca.bits}-bit")
        print(report(diff_stats([ca[i] for i in range(n)], [cb[i] for i in range(n)])))
    return 0


if __name__ == "__main__":
    sys.exit(main(sys.argv[1:]))
