"""Builds and runs the mock VapourSynth API-4 host (tests/vsmock/mock_host.cpp)
against the plugin library (test infrastructure)."""
from __future__ import annotations

import json
import os
import subprocess

import numpy as np

from fft3dcl_gb300 import build

HERE = os.path.dirname(os.path.abspath(__file__))


def plugin_available() -> bool:
    return bool(build.vs_include_dir()) and os.path.exists(build.PLUGIN)


def compile_host(out_dir: str) -> str:
    exe = os.path.join(out_dir, "mock_host")
    subprocess.run(["g++", "-std=c++17", "-O1", "-I", build.vs_include_dir(),
                    os.path.join(HERE, "vsmock", "mock_host.cpp"), "-o", exe, "-ldl"], check=True)
    return exe


def run_cases(exe: str) -> dict:
    """Registration and the argument-error cases, keyed by case name."""
    out = subprocess.run([exe, build.PLUGIN], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stderr
    return {d["case"]: d for d in (json.loads(line) for line in out.stdout.splitlines() if line.strip())}


def plane_shapes(family: str, width: int, height: int) -> list[tuple[int, int]]:
    if family == "gray":
        return [(height, width)]
    if family == "yuv":  # 4:2:0
        return [(height, width), (height // 2, width // 2), (height // 2, width // 2)]
    return [(height, width)] * 3


def run_clip(exe: str, workdir: str, planes: list[list[np.ndarray]], family: str, bits: int,
             order: str = "forward", form: str | None = None, extra_env: dict | None = None, **args):
    """Filters a clip through the plugin under the mock host.

    planes[p][n] is plane p of frame n (uint8, uint16 or float32). Returns
    (out_planes, report): out_planes[p][n] the filtered plane, report the
    host's JSON line (created, error, frame_error, filter_mode, unrequested
    frame fetches, source frames the filter did not free, engines alive after
    the filter was freed)."""
    nframes = len(planes[0])
    h, w = planes[0][0].shape
    dtype = planes[0][0].dtype
    sample = "float" if dtype == np.float32 else "int"
    raw_in = os.path.join(workdir, "in.raw")
    raw_out = os.path.join(workdir, "out.raw")
    with open(raw_in, "wb") as f:
        for n in range(nframes):
            for p in range(len(planes)):
                f.write(np.ascontiguousarray(planes[p][n]).tobytes())
    cmd = [exe, build.PLUGIN, "clip", raw_in, raw_out, family, sample, str(bits), str(w), str(h),
           str(nframes), order] + [f"{k}={v}" for k, v in args.items()]
    env = dict(os.environ)
    env.pop("FFT3DCL_FORM", None)
    if form:
        env["FFT3DCL_FORM"] = form
    env.update(extra_env or {})
    out = subprocess.run(cmd, capture_output=True, text=True, timeout=600, env=env)
    assert out.returncode == 0, (out.returncode, out.stdout, out.stderr)
    report = json.loads(out.stdout.strip().splitlines()[-1])
    result = None
    if report.get("created"):
        data = np.fromfile(raw_out, dtype=dtype)
        shapes = plane_shapes(family, w, h)
        result = [[None] * nframes for _ in shapes]
        off = 0
        for n in range(nframes):
            for p, (ph, pw) in enumerate(shapes):
                result[p][n] = data[off:off + ph * pw].reshape(ph, pw)
                off += ph * pw
    return result, report
