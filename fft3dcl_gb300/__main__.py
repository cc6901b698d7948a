"""Command-line driver: denoise a .y4m clip with the GB300 engine.

    python -m fft3dcl_gb300 IN.y4m OUT.y4m [--form exact|fast|tc] [--gpu N] [--half-spectra]
        [--sigma S --bt N --bw N --bh N --ow N --oh N --sharpen X --plane P ...]

Every FFT3DCL argument of the plugin (src/fft3dcl.cpp:540-546) is accepted as
--name value, with the plugin's defaults. Frames are read on demand, so the
clip is never held in memory whole; the output keeps the input's header.
"""
from __future__ import annotations

import argparse
import sys
import time

from . import FLAG_HALF_SPECTRA, Filter, VideoFormat, ScriptParams
from .y4m import Y4MClip, Y4MWriter

_INT = {"bw", "bh", "bt", "plane", "mode", "bordersize", "precision", "ow", "oh", "wintype", "interlaced", "oldfft"}


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(prog="python -m fft3dcl_gb300", description="FFT3D denoise of a .y4m clip on the GPU")
    ap.add_argument("input")
    ap.add_argument("output")
    ap.add_argument("--form", default="tc", choices=["exact", "fast", "tc"])
    ap.add_argument("--gpu", type=int, default=0)
    ap.add_argument("--frames", type=int, default=0, help="process only the first N frames")
    ap.add_argument("--half-spectra", action="store_true",
                    help="cache the spectra as fp16 (8-bit clips at precision 0/1, tensor-core form)")
    for name, _ in ScriptParams._fields_:
        ap.add_argument(f"--{name}", type=int if name in _INT else float, default=None)
    args = ap.parse_args(argv)
    params = {k: getattr(args, k) for k, _ in ScriptParams._fields_ if getattr(args, k) is not None}
    with Y4MClip(args.input) as clip:
        n = len(clip) if args.frames <= 0 else min(args.frames, len(clip))
        fmt = VideoFormat("gray" if clip.mono else "yuv", clip.bits, 0, clip.sub_w, clip.sub_h)
        view = _Prefix(clip, n)
        flt = Filter(view, fmt, form=args.form, gpu=args.gpu,
                     flags=FLAG_HALF_SPECTRA if args.half_spectra else 0, **params)
        t0 = time.perf_counter()
        try:
            with Y4MWriter(args.output, header=clip.header) as out:
                for i in range(n):
                    out.write(flt.get_frame(i))
        finally:
            flt.close()
        dt = time.perf_counter() - t0
    print(f"{n} frames {clip.width}x{clip.height} {clip.bits}-bit in {dt:.2f} s ({n / dt:.1f} frames/s)",
          file=sys.stderr)
    return 0


class _Prefix:
    """The first n frames of a clip."""

    def __init__(self, clip, n):
        self.clip, self.n = clip, n

    def __len__(self):
        return self.n

    def __getitem__(self, i):
        if not 0 <= i < self.n:
            raise IndexError(i)
        return self.clip[i]


if __name__ == "__main__":
    sys.exit(main())
