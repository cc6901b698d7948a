"""f3d_denoise_noalloc: the entry point for callers that cannot call
cudaMalloc (hosts that hand out a fixed device-memory budget up front,
real-time threads that must not take cudaMalloc's device-wide
synchronisation). Its spectra, windowed blocks and tables live in one static
device array shared by every call.

Checked through the C ABI against the engine's own entry points
(f3d_forward_raw + f3d_process_raw) with the exact form's tolerance -- bit
equality -- on calls in a row with different planes, formats and parameters,
so that contents left in the shared array by one call cannot leak into the
next. Collected last so that a run stopping at the first failure has run
everything else first."""
import ctypes as C

import numpy as np
import pytest

import fft3dcl_gb300 as F
from fft3dcl_gb300 import synth

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def noalloc_lib():
    L = F.lib()
    L.f3d_denoise_noalloc.argtypes = [C.POINTER(F.ScriptParams), C.POINTER(F.PlaneGeom),
                                      C.POINTER(C.c_void_p), C.c_int, C.c_size_t, C.c_void_p,
                                      C.c_size_t, C.c_void_p]
    return L


def call_noalloc(frames, bits, chroma=False, **params):
    """Run the window `frames` (temporal order) through f3d_denoise_noalloc on
    torch's current stream; returns the output plane on the host."""
    h, w = frames[0].shape
    st = 1 if frames[0].dtype == np.float32 else 0
    dev = [torch.from_numpy(np.ascontiguousarray(f)).cuda() for f in frames]
    out = torch.empty_like(dev[0])
    ptrs = (C.c_void_p * len(dev))(*[d.data_ptr() for d in dev])
    pitch = w * frames[0].itemsize
    sp = F.script_params(**params)
    g = F.PlaneGeom(w, h, bits, st, int(chroma))
    stream = torch.cuda.current_stream().cuda_stream
    rc = noalloc_lib().f3d_denoise_noalloc(C.byref(sp), C.byref(g), ptrs, len(dev), pitch,
                                          C.c_void_p(out.data_ptr()), pitch, C.c_void_p(stream))
    torch.cuda.synchronize()
    return rc, out.cpu().numpy()


def engine_output(frames, bits, chroma=False, **params):
    h, w = frames[0].shape
    st = 1 if frames[0].dtype == np.float32 else 0
    with F.Engine(w, h, bits, st, chroma=chroma, **params) as e:
        for i, f in enumerate(frames):
            e.forward_raw(i, f)
        return e.process_raw(list(range(len(frames))))


CALLS = [
    # (frames, bits, chroma, params): planes, formats and temporal modes differ
    # from one call to the next.
    (synth.clip_gray8(frames=3), 8, False, dict(bt=3, sharpen=0.4)),
    (synth.moving_rects(320, 200, 4, 77, lo=64, hi=940, noise=12.0, dtype=np.uint16, maxval=1023),
     10, True, dict(bt=4, sigma=3.0, sigma2=1.5, sigma3=2.5, sigma4=3.5)),
    (synth.moving_rects(200, 120, 1, 5, lo=0.06, hi=0.92, noise=0.01, dtype=np.float32),
     32, False, dict(bt=1, bw=64, bh=64, degrid=0.5)),
    (synth.moving_rects(150, 90, 2, 6, lo=16, hi=235, noise=4.0), 8, False,
     dict(bt=2, mode=0, bw=16, bh=16)),
]


def test_noalloc_equals_engine_on_calls_in_a_row():
    results = []
    for frames, bits, chroma, params in CALLS:
        rc, got = call_noalloc(frames, bits, chroma, **params)
        assert rc == F.F3D_OK, F.lib().f3d_last_error().decode()
        ref = engine_output(frames, bits, chroma, **params)
        np.testing.assert_array_equal(got, ref)
        results.append(got)
    # The first call again, after the others have left their data in the
    # shared array: same bits, and no device memory taken by the repeat.
    frames, bits, chroma, params = CALLS[0]
    free0 = torch.cuda.mem_get_info()[0]
    rc, again = call_noalloc(frames, bits, chroma, **params)
    free1 = torch.cuda.mem_get_info()[0]
    assert rc == F.F3D_OK
    np.testing.assert_array_equal(again, results[0])
    assert free1 >= free0 - (4 << 20)  # torch's own small input buffers at most


def test_noalloc_size_limit():
    # 1024x576 at bt=4 with 32x32 blocks needs 53,953,024 bytes of the
    # 64 MiB array; 1280x720 needs 81,134,080 and is refused.
    frames = synth.moving_rects(1024, 576, 4, 31, lo=16, hi=235, noise=3.0)
    rc, got = call_noalloc(frames, 8, bt=4)
    assert rc == F.F3D_OK, F.lib().f3d_last_error().decode()
    np.testing.assert_array_equal(got, engine_output(frames, 8, bt=4))
    over = [np.zeros((720, 1280), np.uint8) for _ in range(4)]
    rc, _ = call_noalloc(over, 8, bt=4)
    assert rc == -5  # F3D_E_UNSUPPORTED
    msg = F.lib().f3d_last_error().decode()
    assert "81134080 bytes" in msg and "no-alloc limit" in msg


def test_noalloc_rejects_what_it_cannot_hold():
    big = [np.zeros((2160, 3840), np.uint16) for _ in range(4)]
    rc, _ = call_noalloc(big, 10, bt=4)
    assert rc == -5  # F3D_E_UNSUPPORTED
    msg = F.lib().f3d_last_error().decode()
    assert "no-alloc limit" in msg and "bytes" in msg
    rc, _ = call_noalloc(synth.clip_gray8(frames=1), 8, bt=1, bw=128, bh=128)
    assert rc == -5 and "4..64" in F.lib().f3d_last_error().decode()
    rc, _ = call_noalloc(synth.clip_gray8(frames=1), 8, bt=0)
    assert rc == -5 and "Kalman" in F.lib().f3d_last_error().decode()
    rc, _ = call_noalloc(synth.clip_gray8(frames=2), 8, bt=3)
    assert rc == -1 and "window frame" in F.lib().f3d_last_error().decode()
