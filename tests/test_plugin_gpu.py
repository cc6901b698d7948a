"""The VapourSynth plugin's frame path on the GPU, frame by frame against the
oracle.

Each case loads the plugin into the mock API-4 host (tests/vsmock), creates
FFT3DCL over a seeded clip with VapourSynth's call sequence
(VapourSynthPluginInit2 -> create -> getFrame(arInitial) ->
getFrame(arAllFramesReady) -> free) and compares every returned plane with
the oracle's run over the same clip (oracle.run_clip: the reference's window
clamping, src/fft3dcl.cpp:303-331). Planes the filter does not process must
come back byte-identical to the input (src/fft3dcl.cpp:200-225, 395-410).

The host also checks the protocol: every fetched input frame was requested
first (the window requests, src/fft3dcl.cpp:319-331), every source frame is
freed, the filter is fmFrameState for Kalman and fmParallelRequests otherwise
(:286-292), and no engine is left alive once the filter is freed.

Tolerances: the exact form is bit-equal to the oracle; fast and tc (tc is
the plugin's default) within +-1 LSB at 8 bits, +-4 LSB at 10 bits, 1e-4
absolute on float samples in [0, 1] (Kalman runs the exact form in every
form)."""
import numpy as np
import pytest

import oracle
import plugin_host
from fft3dcl_gb300 import synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def host(tmp_path_factory):
    if not plugin_host.plugin_available():
        pytest.skip("plugin not built here (no VapourSynth API-4 headers found at build time)")
    return plugin_host.compile_host(str(tmp_path_factory.mktemp("vsmock")))


def tol(frames, bits, form):
    if form == "exact":
        return 0
    if frames[0].dtype == np.float32:
        return 1e-4
    return 1 if bits <= 8 else 4


def worst(got, ref):
    return max(float(np.abs(g.astype(np.float64) - r.astype(np.float64)).max()) for g, r in zip(got, ref))


def check_protocol(rep, nframes, kalman=False):
    assert rep["created"], rep["error"]
    assert rep["frame_error"] == "", rep["frame_error"]
    assert rep["frames_done"] == nframes
    assert rep["unrequested"] == [], "frames fetched without a request"
    assert rep["source_frames_not_freed"] == 0
    assert rep["frames_alive"] == 0
    assert rep["nodes_freed"] == 1
    assert rep["live_engines_after_free"] == 0
    assert rep["filter_mode"] == ("fmFrameState" if kalman else "fmParallelRequests")
    assert rep["dependency"] == "rpGeneral" and rep["deps"] == 1


def run_and_compare(host, tmp_path, planes, family, bits, processed, form=None, order="forward",
                    chroma_planes=(), **args):
    """Runs the plugin and checks every plane: processed ones against the
    oracle within the form's tolerance, the others byte-identical to the input."""
    out, rep = plugin_host.run_clip(host, str(tmp_path), planes, family, bits, order=order, form=form, **args)
    check_protocol(rep, len(planes[0]), kalman=args.get("bt", 3) == 0)
    oracle_args = {k: v for k, v in args.items() if k != "plane"}
    diffs = {}
    for p, frames in enumerate(planes):
        if p in processed:
            ref = oracle.run_clip(frames, bits, chroma=p in chroma_planes, threads=4, **oracle_args)
            d = worst(out[p], ref)
            assert d <= tol(frames, bits, form), f"plane {p}: max |diff| {d} (form {form})"
            diffs[p] = d
        else:
            for n, (g, s) in enumerate(zip(out[p], frames)):
                assert np.array_equal(g, s), f"untouched plane {p} of frame {n} changed"
    return diffs


def test_gray8_plain_method_every_form(host, tmp_path):
    # 640x360 GRAY8, the plain method: sigma=2 beta=1 bt=3 bw=bh=32 ow=oh=16 degrid=1.
    y = synth.clip_gray8(frames=8)
    for form in ("exact", "fast", "tc"):
        run_and_compare(host, tmp_path, [y], "gray", 8, {0}, form=form, sigma=2.0, beta=1.0, bt=3)


def test_gray8_default_form_is_tc(host, tmp_path):
    # FFT3DCL_FORM unset: the tensor-core form, within +-1 LSB at 8 bits,
    # frames requested out of order.
    y = synth.clip_gray8(width=200, height=136, frames=7)
    run_and_compare(host, tmp_path, [y], "gray", 8, {0}, form=None, order="shuffle", bt=3, sharpen=0.3)


@pytest.mark.parametrize("form", ["exact", "fast", "tc"])
def test_yuv420p8_all_planes(host, tmp_path, form):
    # plane=4 with the 1080p YUV parameters on a smaller frame; requested in reverse.
    y, u, v = synth.clip_yuv420p8(width=352, height=208, frames=7)
    run_and_compare(host, tmp_path, [y, u, v], "yuv", 8, {0, 1, 2}, form=form, order="reverse",
                    chroma_planes=(1, 2), plane=4, sigma=2.5, bt=4, sharpen=0.4, scutoff=0.3, svr=1.0,
                    smin=4.0, smax=20.0, degrid=1.0)


def test_yuv420p8_chroma_only_leaves_luma(host, tmp_path):
    y, u, v = synth.clip_yuv420p8(width=256, height=160, frames=6, seed=11)
    run_and_compare(host, tmp_path, [y, u, v], "yuv", 8, {1, 2}, chroma_planes=(1, 2), plane=1, bt=2)
    # plane=2 and 3 mean chroma too (src/fft3dcl.cpp:212-213).
    run_and_compare(host, tmp_path, [y, u, v], "yuv", 8, {1, 2}, chroma_planes=(1, 2), plane=3, bt=2)


def test_yuv420p8_luma_only_leaves_chroma(host, tmp_path):
    y, u, v = synth.clip_yuv420p8(width=256, height=160, frames=6, seed=12)
    run_and_compare(host, tmp_path, [y, u, v], "yuv", 8, {0}, plane=0, bt=4, sharpen=0.2)


@pytest.mark.parametrize("form", ["exact", "tc"])
def test_yuv420p10_luma(host, tmp_path, form):
    # The 4K 10-bit parameters (sigma=3 bt=4 sharpen=0.4 precision=2) on a
    # 480x272 P10 clip; chroma untouched.
    y = synth.moving_rects(480, 272, 8, 0xF3D2, lo=64, hi=940, noise=12.0, dtype=np.uint16, maxval=1023)
    u = synth.moving_rects(240, 136, 8, 77, lo=64, hi=960, noise=6.0, dtype=np.uint16, maxval=1023, ramp=False)
    v = synth.moving_rects(240, 136, 8, 78, lo=64, hi=960, noise=6.0, dtype=np.uint16, maxval=1023, ramp=False)
    run_and_compare(host, tmp_path, [y, u, v], "yuv", 10, {0}, form=form, order="shuffle", plane=0,
                    sigma=3.0, bt=4, sharpen=0.4, precision=2)


@pytest.mark.parametrize("form", ["exact", "tc"])
def test_grays_kalman_scene_cuts_in_frame_order(host, tmp_path, form):
    # GRAYS Kalman (bt=0, kratio=2, bw=bh=64, ow=oh=32, sigma pattern) with
    # scene cuts: fmFrameState, frames in order even when asked shuffled;
    # Kalman runs the exact form whatever the form asked.
    y = synth.clip_grays(width=320, height=200, frames=14, cuts=(5, 10))
    run_and_compare(host, tmp_path, [y], "gray", 32, {0}, form=form, order="shuffle", bt=0, kratio=2.0,
                    bw=64, bh=64, ow=32, oh=32, sigma=2.0, sigma2=1.5, sigma3=2.5, sigma4=3.0)


def test_rgb_processes_every_plane(host, tmp_path):
    # RGB: plane is forced to 4 (src/fft3dcl.cpp:204); no chroma offset.
    planes = [synth.moving_rects(160, 96, 5, 40 + p, lo=16, hi=235, noise=3.0) for p in range(3)]
    run_and_compare(host, tmp_path, planes, "rgb", 8, {0, 1, 2}, plane=0, bt=3)


@pytest.mark.parametrize("nframes", [1, 2, 3])
def test_short_clips_clamp_the_window(host, tmp_path, nframes):
    # Clips shorter than the bt=4 window: every request clamps to the clip.
    y = synth.moving_rects(96, 64, nframes, 90 + nframes, lo=16, hi=235, noise=3.0)
    run_and_compare(host, tmp_path, [y], "gray", 8, {0}, order="reverse", bt=4, sharpen=0.3)


def test_float_yuv_and_mode0(host, tmp_path):
    # 32-bit float YUV (no chroma offset for float) and mode 0.
    y = synth.moving_rects(192, 128, 5, 7, lo=0.06, hi=0.92, noise=0.01, dtype=np.float32)
    u = synth.moving_rects(96, 64, 5, 8, lo=0.1, hi=0.9, noise=0.01, dtype=np.float32, ramp=False)
    v = synth.moving_rects(96, 64, 5, 9, lo=0.1, hi=0.9, noise=0.01, dtype=np.float32, ramp=False)
    run_and_compare(host, tmp_path, [y, u, v], "yuv", 32, {0, 1, 2}, chroma_planes=(1, 2), plane=4, bt=2)
    run_and_compare(host, tmp_path, [y, u, v], "yuv", 32, {0, 1, 2}, chroma_planes=(1, 2), plane=4, bt=3,
                    mode=0, bw=16, bh=16)


def test_stage_timing_table(host, tmp_path):
    # FFT3DCL_TIME (src/timing.h:1-31, timing.cpp:45-62): the released
    # instance appends one line per stage with its calls and seconds; the
    # output is unchanged by the timing.
    y = synth.clip_gray8(width=160, height=96, frames=6)
    path = tmp_path / "stages.txt"
    out, rep = plugin_host.run_clip(host, str(tmp_path), [y], "gray", 8, form="tc", bt=3,
                                    extra_env={"FFT3DCL_TIME": str(path)})
    check_protocol(rep, 6)
    plain, _ = plugin_host.run_clip(host, str(tmp_path), [y], "gray", 8, form="tc", bt=3)
    assert all(np.array_equal(a, b) for a, b in zip(out[0], plain[0]))
    lines = path.read_text().splitlines()
    assert lines[0].startswith("== FFT3DCL")
    calls = {}
    for ln in lines[1:]:
        if "calls=" in ln:
            name, rest = ln.split("calls=")
            calls[name.strip()] = int(rest.split()[0])
    assert len(calls) == 10
    # Six outputs: one source fetch each plus one per forwarded frame (every
    # frame once), six output frames, six filter/synthesis kernel pairs.
    assert calls["allocate output frame"] == 6
    assert calls["upload + forward"] == 6
    assert calls["fetch source frames"] == 12
    assert calls["filter .. readback"] == 6
    assert calls["GPU: filter"] == calls["GPU: synthesis"] == 6
    assert 1 <= calls["GPU: forward transform"] <= 6
    assert "host stages total" in lines[-1]
