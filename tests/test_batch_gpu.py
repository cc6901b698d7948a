"""Batches of planes (f3d_batch_*): one launch per kernel for the planes of a
YUV frame, of several streams or consecutive outputs of one plane, replayed
as a CUDA graph and autotuned in the tensor-core form, launched directly in
the fast form, give the same bits as each plane's own engine."""
import numpy as np
import pytest
import torch

import fft3dcl_gb300 as F
from fft3dcl_gb300 import synth

pytestmark = pytest.mark.gpu


def run_planes(planes, params, chroma_flags, bits, batch_flags, ahead=False, shape=None, form="tc"):
    """planes[i]: list of frames of plane i. Returns outputs per plane, by
    the batch when batch_flags is not None (with the launch shape pinned to
    `shape` when given), else by separate engines."""
    dev = torch.device("cuda", 0)
    st = torch.cuda.Stream(device=dev)
    nfr = len(planes[0])
    ip = F.validate(planes[0][0].shape[1], planes[0][0].shape[0], bits, **params)
    bt, cur = ip.bt, ip.current
    engines = [F.Engine(p[0].shape[1], p[0].shape[0], bits, chroma=c, form=form, stream=st.cuda_stream, **params)
               for p, c in zip(planes, chroma_flags)]
    src = [torch.from_numpy(np.stack(p)).to(dev) for p in planes]
    dst = [torch.empty(p[0].shape, dtype=src[i].dtype, device=dev) for i, p in enumerate(planes)]
    outs = [[] for _ in planes]
    pitch = [p[0].shape[1] * p[0].itemsize for p in planes]
    b = F.Batch(engines, graph=bool(batch_flags & 1), autotune=bool(batch_flags & 2)) if batch_flags is not None else None
    if b is not None and shape is not None:
        b.set_tune(*shape)
    with torch.cuda.stream(st):
        for n in range(nfr):
            win = [min(max(n - cur + i, 0), nfr - 1) for i in range(bt)]
            missing = sorted(set(win))
            for fn in missing[:-1]:
                for i, e in enumerate(engines):
                    if not e.has(fn):
                        if b is not None:
                            b.step([fn if j == i else -1 for j in range(len(engines))],
                                   [s[fn].data_ptr() for s in src], pitch, [[] for _ in engines],
                                   [d.data_ptr() for d in dst], pitch)
                        else:
                            e.forward_device(fn, src[i][fn].data_ptr(), pitch[i])
            last = missing[-1]
            if b is not None and ahead:
                # Every window frame cached first; the step forwards the frame
                # after the window, concurrently with the outputs.
                for i, e in enumerate(engines):
                    if not e.has(last):
                        e.forward_device(last, src[i][last].data_ptr(), pitch[i])
                nxt = min(win[-1] + 1, nfr - 1)
                b.step([nxt] * len(engines), [s[nxt].data_ptr() for s in src], pitch, [win] * len(engines),
                       [d.data_ptr() for d in dst], pitch)
            elif b is not None:
                b.step([last] * len(engines), [s[last].data_ptr() for s in src], pitch, [win] * len(engines),
                       [d.data_ptr() for d in dst], pitch)
            else:
                for i, e in enumerate(engines):
                    if not e.has(last):
                        e.forward_device(last, src[i][last].data_ptr(), pitch[i])
                    e.process_device(win, dst[i].data_ptr(), pitch[i])
            st.synchronize()
            for i, e in enumerate(engines):
                outs[i].append(dst[i].cpu().numpy())
                e.prune(n - cur - 1, n - cur + bt)
    tune = b.tune() if b is not None else None
    if b is not None:
        b.close()
    for e in engines:
        e.close()
    return outs, tune


def yuv420(w, h, frames, seed, bits):
    if bits == 8:
        y = synth.moving_rects(w, h, frames, seed, lo=16, hi=235, noise=2.5)
        u = synth.moving_rects(w // 2, h // 2, frames, seed + 1, lo=16, hi=240, noise=1.5, ramp=False)
        v = synth.moving_rects(w // 2, h // 2, frames, seed + 2, lo=16, hi=240, noise=1.5, ramp=False)
    else:
        kw = dict(dtype=np.uint16, maxval=1023)
        y = synth.moving_rects(w, h, frames, seed, lo=64, hi=940, noise=10.0, **kw)
        u = synth.moving_rects(w // 2, h // 2, frames, seed + 1, lo=64, hi=960, noise=6.0, ramp=False, **kw)
        v = synth.moving_rects(w // 2, h // 2, frames, seed + 2, lo=64, hi=960, noise=6.0, ramp=False, **kw)
    return [y, u, v]


@pytest.mark.parametrize("flags", [0, 1, 3])
def test_yuv_planes_batch_equals_engines(flags):
    planes = yuv420(480, 272, 7, 21, 8)
    params = dict(sigma=2.5, bt=4, sharpen=0.4, scutoff=0.3, svr=1.0, smin=4.0, smax=20.0)
    got, tune = run_planes(planes, params, [False, True, True], 8, flags)
    ref, _ = run_planes(planes, params, [False, True, True], 8, None)
    for i in range(3):
        for n, (g, r) in enumerate(zip(got[i], ref[i])):
            np.testing.assert_array_equal(g, r, err_msg=f"plane {i} frame {n}")
    if flags & 2:
        assert tune["tuned"] and tune["fwd_ctas_per_sm"] in (1, 2, 3) and tune["filter_minb"] in (3, 4, 5)


@pytest.mark.parametrize("bt", [-1, 1, 2, 3, 4])
def test_every_launch_shape_equals_engines(bt):
    # Every filter-kernel variant (5, 4, 3 CTAs per SM) and forward grid (1
    # to 3 CTAs per SM): the same bits as the engines, in every temporal mode.
    planes = yuv420(400, 240, 6, 31 + bt, 10)[:2]
    params = dict(sigma=3.0, bt=bt, sharpen=0.3, degrid=1.0)
    ref, _ = run_planes(planes, params, [False, True], 10, None)
    for shape in [(3, 5), (2, 5), (1, 5), (2, 4), (3, 3)]:
        got, tune = run_planes(planes, params, [False, True], 10, 1, shape=shape)
        assert (tune["fwd_ctas_per_sm"], tune["filter_minb"]) == shape
        for i in range(2):
            for n, (g, r) in enumerate(zip(got[i], ref[i])):
                np.testing.assert_array_equal(g, r, err_msg=f"shape {shape} plane {i} frame {n}")


@pytest.mark.parametrize("bt", [1, 3, 4])
def test_bw16_planes_and_outputs_batch_equal_engines(bt):
    # 16x16 blocks: YUV planes in one batch (every launch shape), and
    # consecutive outputs of one plane, equal the engines' own calls.
    planes = yuv420(352, 208, 6, 91 + bt, 10)
    params = dict(sigma=3.0, bt=bt, bw=16, bh=16, sharpen=0.3)
    ref, _ = run_planes(planes, params, [False, True, True], 10, None)
    for shape in [(3, 5), (1, 4), (2, 3)]:
        got, _ = run_planes(planes, params, [False, True, True], 10, 1, shape=shape)
        for i in range(3):
            for n, (g, r) in enumerate(zip(got[i], ref[i])):
                np.testing.assert_array_equal(g, r, err_msg=f"shape {shape} plane {i} frame {n}")
    frames = planes[0]
    ref1 = F.FFT3DCL(frames, bits=10, form="tc", **params)
    got1, _ = consecutive_outputs(frames, 10, params, 3, True)
    for n in range(len(frames)):
        np.testing.assert_array_equal(got1[n], ref1[n], err_msg=f"frame {n}")


def test_batch_kernel_times():
    import torch
    frames = synth.moving_rects(320, 192, 6, 61, lo=64, hi=940, noise=10.0, dtype=np.uint16, maxval=1023)
    dev = torch.device("cuda", 0)
    st = torch.cuda.Stream(device=dev)
    src = torch.from_numpy(np.stack(frames)).to(dev)
    dst = torch.empty((192, 320), dtype=torch.uint16, device=dev)
    with F.Engine(320, 192, 10, form="tc", stream=st.cuda_stream, bt=3) as e:
        b = F.Batch([e], graph=False, autotune=False)
        try:
            with pytest.raises(F.F3DError):
                b.last_kernel_ms()  # no step yet
            with torch.cuda.stream(st):
                for fn in range(3):
                    e.forward_device(fn, src[fn].data_ptr(), 640)
                b.step([-1], [src[0].data_ptr()], [640], [[0, 1, 2]], [dst.data_ptr()], [640])
            ms = b.last_kernel_ms()
            assert len(ms) == 2 and all(0.0 < t < 1000.0 for t in ms)
        finally:
            b.close()


def test_set_tune_rejects_unknown_shapes():
    eng = F.Engine(128, 96, 8, form="tc", bt=3)
    b = F.Batch([eng])
    try:
        for shape in [(4, 5), (0, 5), (2, 2), (2, 6)]:
            with pytest.raises(F.F3DError):
                b.set_tune(*shape)
        b.set_tune(1, 3)
        assert b.tune() == {"tuned": True, "fwd_ctas_per_sm": 1, "filter_minb": 3}
    finally:
        b.close()
        eng.close()


@pytest.mark.parametrize("flags", [0, 1])
def test_lookahead_step_overlaps_and_equals_engines(flags):
    # The forward of the frame after the window runs on the side stream,
    # concurrently with the outputs (directly, or inside the captured graph).
    planes = yuv420(320, 192, 8, 41, 10)
    params = dict(sigma=3.0, bt=4, sharpen=0.3)
    got, _ = run_planes(planes, params, [False, True, True], 10, flags, ahead=True)
    ref, _ = run_planes(planes, params, [False, True, True], 10, None)
    for i in range(3):
        for n, (g, r) in enumerate(zip(got[i], ref[i])):
            np.testing.assert_array_equal(g, r, err_msg=f"plane {i} frame {n}")


@pytest.mark.parametrize("graph", [False, True])
@pytest.mark.parametrize("order,nf", [("by_plane", 2), ("by_frame", 2), ("by_plane", 4), ("by_plane", 5)])
def test_yuv_frames_per_step_equal_engines(order, nf, graph):
    # nf consecutive YUV frames per step, 3 nf outputs of three engines. By
    # plane ([Y, Y, U, U, V, V] for two) the filter runs two runs of one
    # geometry (luma; both chroma planes), each interleaving its outputs'
    # CTAs; by frame ([Y, U, V, Y, U, V]) the chroma pairs form the runs.
    planes = yuv420(480, 272, 11, 27, 8)
    params = dict(sigma=2.5, bt=4, sharpen=0.4, scutoff=0.3, svr=1.0, smin=4.0, smax=20.0)
    ref, _ = run_planes(planes, params, [False, True, True], 8, None)
    dev = torch.device("cuda", 0)
    st = torch.cuda.Stream(device=dev)
    nfr = len(planes[0])
    ip = F.validate(480, 272, 8, **params)
    bt, cur = ip.bt, ip.current
    engines = [F.Engine(p[0].shape[1], p[0].shape[0], 8, chroma=i > 0, form="tc", stream=st.cuda_stream,
                        **params) for i, p in enumerate(planes)]
    src = [torch.from_numpy(np.stack(p)).to(dev) for p in planes]
    slots = [(i, r) for i in range(3) for r in range(nf)] if order == "by_plane" else \
            [(i, r) for r in range(nf) for i in range(3)]
    dst = [torch.empty(planes[i][0].shape, dtype=torch.uint8, device=dev) for i, _ in slots]
    pitch = [planes[i][0].shape[1] for i, _ in slots]
    b = F.Batch([engines[i] for i, _ in slots], graph=graph, autotune=True)
    got = [[None] * nfr for _ in range(3)]
    with torch.cuda.stream(st):
        for n in range(0, nfr, nf):
            wins = [[min(max(n + r - cur + k, 0), nfr - 1) for k in range(bt)] for _, r in slots]
            for (i, _), win in zip(slots, wins):
                for fn in win:
                    if not engines[i].has(fn):
                        engines[i].forward_device(fn, src[i][fn].data_ptr(), planes[i][0].shape[1])
            b.step([-1] * len(slots), [src[i][0].data_ptr() for i, _ in slots], pitch, wins,
                   [d.data_ptr() for d in dst], pitch)
            st.synchronize()
            for (i, r), d in zip(slots, dst):
                if n + r < nfr:
                    got[i][n + r] = d.cpu().numpy()
            for e in engines:
                e.prune(n - cur - 1, n + nf - cur + bt)
    b.close()
    for e in engines:
        e.close()
    for i in range(3):
        for n in range(nfr):
            np.testing.assert_array_equal(got[i][n], ref[i][n], err_msg=f"plane {i} frame {n}")


def test_mixed_sizes_batch_equals_engines():
    a = synth.moving_rects(640, 360, 6, 31, lo=64, hi=940, noise=10.0, dtype=np.uint16, maxval=1023)
    b = synth.moving_rects(1000, 200, 6, 32, lo=64, hi=940, noise=10.0, dtype=np.uint16, maxval=1023)
    params = dict(sigma=3.0, bt=3)
    got, _ = run_planes([a, b], params, [False, False], 10, 3)
    ref, _ = run_planes([a, b], params, [False, False], 10, None)
    for i in range(2):
        for g, r in zip(got[i], ref[i]):
            np.testing.assert_array_equal(g, r)


def test_batch_holds_at_most_sixteen_entries():
    with F.Engine(96, 64, 8, form="tc", bt=3) as e:
        F.Batch([e] * 16).close()
        with pytest.raises(F.F3DError):
            F.Batch([e] * 17)


def test_batch_rejects_mixed_forms():
    with F.Engine(96, 64, 8, form="tc", bt=3) as e1, F.Engine(96, 64, 8, form="fast", bt=3) as e2:
        with pytest.raises(F.F3DError):
            F.Batch([e1, e2])


def consecutive_outputs(frames, bits, params, k, graph, shape=None, flags=0, form="tc"):
    """The same engine k times in a batch: k consecutive outputs per step, the
    forwards of the next k frames concurrent with them. Returns the outputs
    and the batch's launch shape."""
    h, w = frames[0].shape
    ip = F.validate(w, h, bits, **params)
    bt, cur = max(ip.bt, 1), ip.current
    dev = torch.device("cuda", 0)
    st = torch.cuda.Stream(device=dev)
    e = F.Engine(w, h, bits, form=form, stream=st.cuda_stream, flags=flags, **params)
    assert e.info().form == ["exact", "fast", "tc"].index(form)
    src = torch.from_numpy(np.stack(frames)).to(dev)
    dst = [torch.empty((h, w), dtype=src.dtype, device=dev) for _ in range(k)]
    b = F.Batch([e] * k, graph=graph, autotune=shape is None)
    if shape is not None:
        b.set_tune(*shape)
    nfr, pitch = len(frames), w * frames[0].itemsize
    got = []
    with torch.cuda.stream(st):
        for n in range(0, nfr, k):
            wins = [[min(max(m - cur + i, 0), nfr - 1) for i in range(bt)] for m in range(n, n + k)]
            for win in wins:
                for fn in win:
                    if not e.has(fn):
                        e.forward_device(fn, src[fn].data_ptr(), pitch)
            # The frames after the last window, unless a clamped window holds them.
            ahead = [n + k - 1 - cur + bt + i for i in range(k)]
            ahead = [a if a < nfr else -1 for a in ahead]
            b.step(ahead, [src[min(a, nfr - 1)].data_ptr() for a in ahead], [pitch] * k, wins,
                   [d.data_ptr() for d in dst], [pitch] * k)
            st.synchronize()
            got += [d.cpu().numpy() for d in dst]
            e.prune(n - cur - 1, n + k - 1 - cur + bt + k)
    tune = b.tune()
    b.close()
    e.close()
    return got[:nfr], tune


@pytest.mark.parametrize("graph", [False, True])
@pytest.mark.parametrize("k", [2, 4, 8, 16])
def test_several_outputs_per_step_equal_engine(k, graph):
    frames = synth.moving_rects(320, 192, 13, 51, lo=64, hi=940, noise=10.0, dtype=np.uint16, maxval=1023)
    params = dict(sigma=3.0, bt=4, sharpen=0.3)
    ref = F.FFT3DCL(frames, bits=10, form="tc", **params)
    got, _ = consecutive_outputs(frames, 10, params, k, graph)
    for n in range(len(frames)):
        np.testing.assert_array_equal(got[n], ref[n], err_msg=f"frame {n}")


@pytest.mark.parametrize("bits,bt,k,graph,flags,extra", [
    (10, 4, 2, False, 0, dict(degrid=0.0)),
    (10, 3, 4, True, 0, dict(sigma2=1.0, sigma3=3.0, sigma4=4.0)),
    (10, 2, 6, False, 0, dict(beta=1.5, sharpen=0.5)),
    (8, 4, 8, True, F.FLAG_HALF_SPECTRA, dict(precision=0, sharpen=0.4)),
    (8, 2, 4, False, F.FLAG_HALF_SPECTRA, dict(precision=1)),
])
def test_consecutive_outputs_each_temporal_mode(bits, bt, k, graph, flags, extra):
    # Batches of consecutive outputs (shifted windows: the filter pulls only
    # each later output's newest frame into L2) in temporal modes 2-4, with
    # degrid off, a sigma pattern and half storage: the per-output engine
    # path's values bit for bit.
    if bits == 8:
        frames = synth.moving_rects(352, 208, 15, 61 + bt, lo=16, hi=235, noise=4.0)
    else:
        frames = synth.moving_rects(352, 208, 15, 61 + bt, lo=64, hi=940, noise=10.0, dtype=np.uint16,
                                    maxval=1023)
    params = dict(sigma=3.0, bt=bt, **extra)
    ref = F.FFT3DCL(frames, bits=bits, form="tc", flags=flags, **params)
    got, _ = consecutive_outputs(frames, bits, params, k, graph, flags=flags)
    for n in range(len(frames)):
        np.testing.assert_array_equal(got[n], ref[n], err_msg=f"frame {n}")


@pytest.mark.parametrize("k,graph", [(2, False), (4, True), (10, False)])
def test_fast_batch_consecutive_outputs_equal_engine(k, graph):
    # The fast form's batch: one forward launch per entering frame, the fused
    # sweeps of the k outputs in one launch with their CTAs interleaved (the
    # graph flag does not apply to it): the engine's own values bit for bit.
    frames = synth.moving_rects(320, 192, 13, 71, lo=64, hi=940, noise=10.0, dtype=np.uint16, maxval=1023)
    params = dict(sigma=3.0, bt=4, sharpen=0.3)
    ref = F.FFT3DCL(frames, bits=10, form="fast", **params)
    got, tune = consecutive_outputs(frames, 10, params, k, graph, form="fast")
    assert not tune["tuned"]
    for n in range(len(frames)):
        np.testing.assert_array_equal(got[n], ref[n], err_msg=f"frame {n}")


@pytest.mark.parametrize("bw,bt", [(8, 3), (16, 3), (32, 3), (32, 1), (16, 4), (8, 2), (32, -1)])
def test_fast_batch_yuv_planes_equal_engines(bw, bt):
    y, u, v = yuv420(256, 160, 6, 81 + bw + bt, 8)
    params = dict(sigma=2.5, bt=bt, bw=bw, bh=bw, sharpen=0.3)
    ref, _ = run_planes([y, u, v], params, [False, True, True], 8, None, form="fast")
    got, _ = run_planes([y, u, v], params, [False, True, True], 8, 0, ahead=True, form="fast")
    for p in range(3):
        for n in range(len(y)):
            np.testing.assert_array_equal(got[p][n], ref[p][n], err_msg=f"plane {p} frame {n}")

