"""fft3dcl_gb300 -- GB300-native FFT3D block-FFT video denoiser.

Python bindings of the engine's C ABI (include/fft3d_gb300.h, implemented in
lib/libfft3d_gb300.so) and a clip-level driver with the reference plugin's
semantics, for hosts that hold frames as numpy arrays.

* :class:`Engine` -- one plane of one filter instance; the methods mirror the
  reference backend class GpuRef (src/cl/gpu.h:16-88): forward / forward_raw,
  has, process / process_raw, prune, live counters.
* :class:`Filter` / :func:`FFT3DCL` -- the frame callback of the reference's
  VapourSynth plugin (src/fft3dcl.cpp:123-526): plane selection, temporal
  window clamped to the clip, spectra cache pruning, untouched planes copied.

There is no CPU fallback: if the CUDA library is missing or no GPU is
present, constructing an engine raises.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass, field

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "lib", "libfft3d_gb300.so")

F3D_OK = 0
FORMS = {"exact": 0, "fast": 1, "tc": 2}

TAB_WIN_ANA, TAB_WIN_SYN_A, TAB_WIN_SYN_B, TAB_PATTERN, TAB_SHARPEN, TAB_GS_RE, TAB_GS_IM, \
    TAB_TWIDDLE_ROW, TAB_TWIDDLE_COL = range(9)


class ScriptParams(C.Structure):
    """f3d_script_params (the reference's ScriptParams, src/params.h:8-27)."""

    _fields_ = [
        ("sigma", C.c_float), ("beta", C.c_float),
        ("bw", C.c_int), ("bh", C.c_int), ("bt", C.c_int),
        ("sharpen", C.c_float),
        ("plane", C.c_int), ("mode", C.c_int), ("bordersize", C.c_int), ("precision", C.c_int),
        ("degrid", C.c_float), ("scutoff", C.c_float), ("svr", C.c_float),
        ("smin", C.c_float), ("smax", C.c_float), ("kratio", C.c_float),
        ("ow", C.c_int), ("oh", C.c_int), ("wintype", C.c_int), ("interlaced", C.c_int),
        ("sigma2", C.c_float), ("sigma3", C.c_float), ("sigma4", C.c_float),
        ("oldfft", C.c_int),
    ]


class InternalParams(C.Structure):
    """f3d_internal_params (InternalParams, src/params.h:30-59)."""

    _fields_ = [
        ("sigma", C.c_float), ("beta", C.c_float),
        ("bw", C.c_int), ("bh", C.c_int), ("bm", C.c_int), ("bt", C.c_int),
        ("sharpen", C.c_float),
        ("sharpen_on", C.c_int), ("mode", C.c_int), ("bordersize", C.c_int),
        ("precision", C.c_int),
        ("degrid", C.c_float), ("degrid_on", C.c_int),
        ("scutoff", C.c_float), ("svr", C.c_float), ("smin", C.c_float),
        ("smax", C.c_float), ("kratio", C.c_float),
        ("ow", C.c_int), ("oh", C.c_int), ("wintype", C.c_int), ("interlaced", C.c_int),
        ("sigma2", C.c_float), ("sigma3", C.c_float), ("sigma4", C.c_float),
        ("use_pattern", C.c_int), ("current", C.c_int), ("nx", C.c_int), ("ny", C.c_int),
        ("totw", C.c_int), ("toth", C.c_int), ("oldfft", C.c_int),
        ("wiener_s", C.c_float), ("beta_x", C.c_float), ("kalman_cn", C.c_float),
        ("ssmin", C.c_float), ("ssmax", C.c_float),
    ]


class PlaneGeom(C.Structure):
    _fields_ = [("width", C.c_int), ("height", C.c_int), ("bits", C.c_int),
                ("sample_type", C.c_int), ("chroma", C.c_int)]


class Options(C.Structure):
    _fields_ = [("device", C.c_int), ("form", C.c_int), ("stream", C.c_void_p), ("flags", C.c_int)]


FLAG_UNFUSED, FLAG_PREFETCH_EARLY, FLAG_PREFETCH_LATE, FLAG_HALF_SPECTRA = 1, 2, 4, 8
FLAG_TEST_WAIT_TIMEOUT = 1 << 20  # tests of the error path only (include/fft3d_gb300.h)


class EngineInfo(C.Structure):
    _fields_ = [("nblocks", C.c_int), ("fbw", C.c_int), ("ncols", C.c_int), ("nrows", C.c_int),
                ("bytes_per_sample", C.c_int), ("raw_path", C.c_int),
                ("spectrum_bytes", C.c_size_t), ("device_bytes", C.c_size_t),
                ("cached_frames", C.c_int), ("chroma_norm", C.c_float), ("form", C.c_int),
                ("fused", C.c_int), ("half_spectra", C.c_int)]


# Every symbol the C ABI declares (include/fft3d_gb300.h).
EXPORTS = (
    "f3d_default_params", "f3d_validate_params", "f3d_last_error", "f3d_engine_create",
    "f3d_engine_destroy", "f3d_engine_error", "f3d_engine_get_info", "f3d_engine_get_table",
    "f3d_compute_table",
    "f3d_forward", "f3d_forward_raw", "f3d_forward_device", "f3d_get_spectra", "f3d_has", "f3d_raw_path",
    "f3d_bytes_per_sample", "f3d_upload_degrid_sample", "f3d_process", "f3d_process_raw",
    "f3d_process_device", "f3d_prune", "f3d_synchronize", "f3d_last_kernel_ms",
    "f3d_live_instances", "f3d_live_bytes", "f3d_kernel_launches", "f3d_denoise_noalloc",
    "f3d_server_create", "f3d_server_destroy", "f3d_server_open", "f3d_server_submit", "f3d_server_poll",
    "f3d_server_poll_timed", "f3d_server_close", "f3d_server_get_stats",
    "f3d_batch_create", "f3d_batch_destroy", "f3d_batch_error", "f3d_batch_step", "f3d_batch_tune",
    "f3d_batch_set_tune", "f3d_batch_last_kernel_ms",
)

_lib = None


def lib():
    """The engine library. Raises if it has not been built: the product path
    has no fallback."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"fft3dcl_gb300: CUDA engine library missing ({LIB_PATH}); "
                               "run `python -m fft3dcl_gb300.build`")
        L = C.CDLL(LIB_PATH)
        P, vp, i, sz = C.POINTER, C.c_void_p, C.c_int, C.c_size_t
        L.f3d_default_params.argtypes = [P(ScriptParams)]
        L.f3d_default_params.restype = None
        L.f3d_validate_params.argtypes = [P(ScriptParams), i, i, i, P(InternalParams)]
        L.f3d_last_error.restype = C.c_char_p
        L.f3d_engine_create.argtypes = [P(ScriptParams), P(PlaneGeom), P(Options), P(vp)]
        L.f3d_engine_destroy.argtypes = [vp]
        L.f3d_engine_destroy.restype = None
        L.f3d_engine_error.argtypes = [vp]
        L.f3d_engine_error.restype = C.c_char_p
        L.f3d_engine_get_info.argtypes = [vp, P(EngineInfo)]
        L.f3d_engine_get_table.argtypes = [vp, i, vp]
        L.f3d_compute_table.argtypes = [P(ScriptParams), P(PlaneGeom), i, vp]
        L.f3d_forward.argtypes = [vp, i, vp]
        L.f3d_forward_raw.argtypes = [vp, i, vp, sz]
        L.f3d_forward_device.argtypes = [vp, i, vp, sz]
        L.f3d_get_spectra.argtypes = [vp, i, vp]
        L.f3d_has.argtypes = [vp, i]
        L.f3d_raw_path.argtypes = [vp]
        L.f3d_bytes_per_sample.argtypes = [vp]
        L.f3d_upload_degrid_sample.argtypes = [vp]
        L.f3d_process.argtypes = [vp, P(i), i, vp]
        L.f3d_process_raw.argtypes = [vp, P(i), i, vp, sz]
        L.f3d_process_device.argtypes = [vp, P(i), i, vp, sz]
        L.f3d_batch_create.argtypes = [P(vp), i, i, P(vp)]
        L.f3d_batch_destroy.argtypes = [vp]
        L.f3d_batch_destroy.restype = None
        L.f3d_batch_error.argtypes = [vp]
        L.f3d_batch_error.restype = C.c_char_p
        L.f3d_batch_step.argtypes = [vp, P(i), P(vp), P(sz), P(P(i)), P(i), P(vp), P(sz)]
        L.f3d_batch_tune.argtypes = [vp, P(i), P(i)]
        L.f3d_batch_set_tune.argtypes = [vp, i, i]
        L.f3d_batch_last_kernel_ms.argtypes = [vp, P(C.c_float)]
        L.f3d_server_create.argtypes = [P(ServerConfig), P(vp)]
        L.f3d_server_destroy.argtypes = [vp]
        L.f3d_server_destroy.restype = None
        L.f3d_server_open.argtypes = [vp, P(ScriptParams), P(PlaneGeom), i, P(i)]
        L.f3d_server_submit.argtypes = [vp, i, i, vp, C.c_longlong]
        L.f3d_server_poll.argtypes = [vp, i, P(i), vp, C.c_longlong, i]
        L.f3d_server_poll_timed.argtypes = [vp, i, P(i), vp, C.c_longlong, i, P(C.c_double), P(C.c_double)]
        L.f3d_server_close.argtypes = [vp, i]
        L.f3d_server_get_stats.argtypes = [vp, P(ServerStats)]
        L.f3d_prune.argtypes = [vp, i, i]
        L.f3d_synchronize.argtypes = [vp]
        L.f3d_last_kernel_ms.argtypes = [vp, P(C.c_float)]
        L.f3d_live_instances.restype = i
        L.f3d_live_bytes.restype = sz
        L.f3d_kernel_launches.restype = C.c_uint64
        _lib = L
    return _lib


class ServerConfig(C.Structure):
    _fields_ = [("device", C.c_int), ("form", C.c_int), ("max_streams", C.c_int), ("hbm_budget", C.c_size_t)]


class ServerStats(C.Structure):
    _fields_ = [("frames", C.c_longlong), ("p50_ms", C.c_double), ("p99_ms", C.c_double),
                ("max_ms", C.c_double), ("mean_ms", C.c_double), ("seconds", C.c_double),
                ("open_streams", C.c_int), ("used_bytes", C.c_size_t), ("shared_steps", C.c_longlong),
                ("shared_outputs", C.c_longlong), ("max_shared", C.c_int), ("busy_ms", C.c_double)]


F3D_E_BUSY = -6


class F3DError(RuntimeError):
    pass


def script_params(**kw) -> ScriptParams:
    """Script parameters with the plugin's defaults (src/fft3dcl.cpp:171-195),
    including the dependent ones: degrid = 1 if mode == 1 else 0, ow/oh =
    bw/2, bh/2 of the script values, sigma2/3/4 = sigma."""
    unknown = set(kw) - {f for f, _ in ScriptParams._fields_}
    if unknown:
        raise TypeError(f"FFT3DCL: unknown parameter(s) {sorted(unknown)}")
    sp = ScriptParams()
    sp.sigma = kw.get("sigma", 2.0)
    sp.beta = kw.get("beta", 1.0)
    sp.bw = kw.get("bw", 32)
    sp.bh = kw.get("bh", 32)
    sp.bt = kw.get("bt", 3)
    sp.sharpen = kw.get("sharpen", 0.0)
    sp.plane = kw.get("plane", 0)
    sp.mode = kw.get("mode", 1)
    sp.bordersize = kw.get("bordersize", 1)
    sp.precision = kw.get("precision", 0)
    sp.degrid = kw.get("degrid", 1.0 if sp.mode == 1 else 0.0)
    sp.scutoff = kw.get("scutoff", 0.3)
    sp.svr = kw.get("svr", 1.0)
    sp.smin = kw.get("smin", 4.0)
    sp.smax = kw.get("smax", 20.0)
    sp.kratio = kw.get("kratio", 2.0)
    sp.ow = kw.get("ow", sp.bw // 2)
    sp.oh = kw.get("oh", sp.bh // 2)
    sp.wintype = kw.get("wintype", 0)
    sp.interlaced = kw.get("interlaced", 0)
    sp.sigma2 = kw.get("sigma2", sp.sigma)
    sp.sigma3 = kw.get("sigma3", sp.sigma)
    sp.sigma4 = kw.get("sigma4", sp.sigma)
    sp.oldfft = kw.get("oldfft", -1)
    return sp


def validate(width: int, height: int, bits: int, **params) -> InternalParams:
    """validateParams (src/params.h:76-148); raises ValueError with the
    reference's message."""
    ip = InternalParams()
    if lib().f3d_validate_params(C.byref(script_params(**params)), width, height, bits,
                                 C.byref(ip)) != F3D_OK:
        raise ValueError(lib().f3d_last_error().decode())
    return ip


def compute_table(which: int, width: int, height: int, bits: int = 8, sample_type: int = 0,
                  chroma: bool = False, **params) -> np.ndarray:
    """A plane table (TAB_*) computed on the host, without a device."""
    sp = script_params(**params)
    g = PlaneGeom(width, height, bits, sample_type, int(chroma))
    n = lib().f3d_compute_table(C.byref(sp), C.byref(g), which, None)
    if n < 0:
        raise ValueError(lib().f3d_last_error().decode())
    out = np.zeros(n, np.float32)
    if n:
        lib().f3d_compute_table(C.byref(sp), C.byref(g), which, out.ctypes.data_as(C.c_void_p))
    return out


def live_instances() -> int:
    return lib().f3d_live_instances()


def live_bytes() -> int:
    return lib().f3d_live_bytes()


def kernel_launches() -> int:
    return lib().f3d_kernel_launches()


def _sample_info(dtype):
    dt = np.dtype(dtype)
    if dt == np.uint8:
        return 0, 1
    if dt == np.uint16:
        return 0, 2
    if dt == np.float32:
        return 1, 4
    raise ValueError(f"FFT3DCL: unsupported sample type {dt}")


class Engine:
    """One plane of a filter instance on the GPU (GpuRef, src/cl/gpu.h:16-88)."""

    def __init__(self, width: int, height: int, bits: int = 8, sample_type: int = 0,
                 chroma: bool = False, form: str = "exact", device: int = 0, stream: int | None = None,
                 fused: bool = True, flags: int = 0, **params):
        self.sp = script_params(**params)
        self.geom = PlaneGeom(width, height, bits, sample_type, int(chroma))
        self.width, self.height, self.bits, self.sample_type = width, height, bits, sample_type
        opts = Options(device, FORMS[form], stream or None, flags | (0 if fused else FLAG_UNFUSED))
        h = C.c_void_p()
        if lib().f3d_engine_create(C.byref(self.sp), C.byref(self.geom), C.byref(opts),
                                   C.byref(h)) != F3D_OK:
            raise F3DError(lib().f3d_last_error().decode())
        self._h = h
        info = self.info()
        self.nblocks, self.fbw = info.nblocks, info.fbw
        self.bps = info.bytes_per_sample
        self.sp_bh = validate(width, height, bits, **params).bh
        self.dtype = np.float32 if sample_type == 1 else (np.uint8 if bits <= 8 else np.uint16)

    def _check(self, rc):
        if rc != F3D_OK:
            raise F3DError(lib().f3d_engine_error(self._h).decode() or lib().f3d_last_error().decode())

    def close(self):
        if getattr(self, "_h", None):
            lib().f3d_engine_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def info(self) -> EngineInfo:
        info = EngineInfo()
        self._check(lib().f3d_engine_get_info(self._h, C.byref(info)))
        return info

    def table(self, which: int) -> np.ndarray:
        n = lib().f3d_engine_get_table(self._h, which, None)
        out = np.zeros(max(n, 0), np.float32)
        if n > 0:
            lib().f3d_engine_get_table(self._h, which, out.ctypes.data_as(C.c_void_p))
        return out

    def forward(self, fn: int, plane: np.ndarray):
        """GpuRef::forward: float plane (already converted) -> cached spectra."""
        plane = np.ascontiguousarray(plane, np.float32)
        assert plane.shape == (self.height, self.width)
        self._check(lib().f3d_forward(self._h, fn, plane.ctypes.data_as(C.c_void_p)))

    def forward_raw(self, fn: int, raw: np.ndarray):
        """GpuRef::forwardRaw: native samples -> cached spectra."""
        raw = np.ascontiguousarray(raw)
        self._check(lib().f3d_forward_raw(self._h, fn, raw.ctypes.data_as(C.c_void_p), raw.nbytes))

    def forward_device(self, fn: int, ptr: int, pitch: int):
        self._check(lib().f3d_forward_device(self._h, fn, C.c_void_p(ptr), pitch))

    def spectra(self, fn: int) -> np.ndarray:
        """Cached half spectra of frame fn as complex64 [nblocks, bh, fbw]."""
        out = np.empty((self.nblocks, self.sp_bh, self.fbw), np.complex64)
        self._check(lib().f3d_get_spectra(self._h, fn, out.ctypes.data_as(C.c_void_p)))
        return out

    def has(self, fn: int) -> bool:
        return bool(lib().f3d_has(self._h, fn))

    def upload_degrid_sample(self):
        self._check(lib().f3d_upload_degrid_sample(self._h))

    @staticmethod
    def _win(window):
        w = (C.c_int * len(window))(*window)
        return w, len(window)

    def process(self, window) -> np.ndarray:
        """GpuRef::process: float output plane (before packing)."""
        w, n = self._win(window)
        out = np.empty((self.height, self.width), np.float32)
        self._check(lib().f3d_process(self._h, w, n, out.ctypes.data_as(C.c_void_p)))
        return out

    def process_raw(self, window, out: np.ndarray | None = None) -> np.ndarray:
        """GpuRef::processRaw: output packed to the native sample format."""
        w, n = self._win(window)
        if out is None:
            out = np.empty((self.height, self.width), self.dtype)
        self._check(lib().f3d_process_raw(self._h, w, n, out.ctypes.data_as(C.c_void_p), out.nbytes))
        return out

    def process_device(self, window, ptr: int, pitch: int):
        w, n = self._win(window)
        self._check(lib().f3d_process_device(self._h, w, n, C.c_void_p(ptr), pitch))

    def prune(self, lo: int, hi: int):
        self._check(lib().f3d_prune(self._h, lo, hi))

    def synchronize(self):
        self._check(lib().f3d_synchronize(self._h))

    def last_kernel_ms(self):
        """(forward, filter+inverse, overlap-add) device ms of the last calls."""
        ms = (C.c_float * 3)()
        self._check(lib().f3d_last_kernel_ms(self._h, ms))
        return tuple(ms)


@dataclass
class VideoFormat:
    """Constant clip format: color family 'gray' | 'yuv' | 'rgb', sample
    type, bits per sample and chroma subsampling (log2)."""
    color_family: str = "gray"
    bits: int = 8
    sample_type: int = 0
    sub_w: int = 0
    sub_h: int = 0
    num_planes: int = field(init=False)

    def __post_init__(self):
        self.num_planes = 1 if self.color_family == "gray" else 3


def _clamp(n, num):
    return 0 if n < 0 else (num - 1 if n > num - 1 else n)


class Filter:
    """One FFT3DCL filter instance over a clip (src/fft3dcl.cpp:123-534).

    clip: a sequence of frames, each a list of 2D numpy planes. get_frame(n)
    returns the filtered frame n. Kalman (bt=0) frames must be requested in
    order, as the reference's fmFrameState mode delivers them."""

    def __init__(self, clip, fmt: VideoFormat, form: str = "exact", device: int = 2,
                 gpu: int = 0, fused: bool = True, flags: int = 0, **params):
        if fmt.sample_type == 1 and fmt.bits != 32:
            raise ValueError("FFT3DCL: only 32-bit float clips supported (16-bit float not ported yet)")
        if fmt.sample_type == 0 and not 8 <= fmt.bits <= 16:
            raise ValueError("FFT3DCL: integer bit depths 8-16 only")
        if device == 0:
            raise ValueError("FFT3DCL: device=0 (CPU backend) is not available: there is no CPU path; "
                             "use device=1 or 2")
        self.clip = clip
        self.fmt = fmt
        self.sp = script_params(**params)
        plane = self.sp.plane
        # Plane semantics, src/fft3dcl.cpp:200-225.
        if fmt.color_family == "rgb":
            plane = 4
        if fmt.color_family == "gray":
            if plane == 1:
                raise ValueError("FFT3DCL: cannot set chroma processing for a greyscale clip")
            if plane == 4:
                plane = 0
        if plane in (2, 3):
            plane = 1
        if plane not in (0, 1, 4):
            raise ValueError("FFT3DCL: plane must be 0 (luma), 1 (chroma) or 4 (all)")
        if fmt.color_family == "gray" or plane == 0:
            self.planes = [0]
        elif plane == 1:
            self.planes = [1, 2]
        else:
            self.planes = [0, 1, 2]
        first = clip[0]
        self.engines = []
        try:
            for p in self.planes:
                h, w = first[p].shape
                self.engines.append(Engine(w, h, fmt.bits, fmt.sample_type,
                                           chroma=(fmt.color_family == "yuv" and p > 0),
                                           form=form, device=gpu, fused=fused, flags=flags, **params))
        except Exception:
            self.close()
            raise
        self.ip = validate(first[0].shape[1], first[0].shape[0], fmt.bits, **params)
        self.num_frames = len(clip)

    def close(self):
        for e in self.engines:
            e.close()
        self.engines = []

    def window(self, n):
        ip = self.ip
        if ip.bm >= 2:
            return [_clamp(n - ip.current + i, self.num_frames) for i in range(ip.bt)]
        return [_clamp(n, self.num_frames)]

    def get_frame(self, n: int):
        src = self.clip[n]
        out = [np.array(p, copy=True) for p in src]  # untouched planes copied
        ip = self.ip
        for k, p in enumerate(self.planes):
            e = self.engines[k]
            win = self.window(n)
            for fn in win:
                if not e.has(fn):
                    e.forward_raw(fn, self.clip[fn][p])
            out[p] = e.process_raw(win)
            # Cache kept to what the next requests reuse (src/fft3dcl.cpp:457-466).
            if ip.bm >= 2:
                e.prune(n - ip.current - 1, n - ip.current + ip.bt)
            elif ip.bm != 0:
                e.prune(-1, -2)
            else:
                e.prune(n, n)
        return out


def FFT3DCL(clip, fmt: VideoFormat | None = None, **params):
    """Filter a whole numpy clip; returns the list of output frames. A clip of
    2D arrays is taken as a one-plane (gray) clip."""
    single = isinstance(clip[0], np.ndarray)
    frames = [[f] for f in clip] if single else clip
    if fmt is None:
        st, _ = _sample_info(frames[0][0].dtype)
        bits = params.pop("bits", 32 if st == 1 else (8 if frames[0][0].dtype == np.uint8 else 16))
        fmt = VideoFormat("gray" if len(frames[0]) == 1 else "yuv", bits, st)
    flt = Filter(frames, fmt, **params)
    try:
        res = [flt.get_frame(n) for n in range(len(frames))]
    finally:
        flt.close()
    return [r[0] for r in res] if single else res


class Server:
    """The serving loop (f3d_server_*): many plane streams of any size, depth
    and parameters on one GPU, admitted by an HBM budget, each keeping its
    window spectra resident, launched as their frames arrive: tensor-core
    streams in shared steps (one launch per kernel for many streams), the
    others concurrently on their own CUDA streams."""

    def __init__(self, form: str = "tc", device: int = 0, max_streams: int = 16,
                 hbm_budget: int = 64 << 30):
        cfg = ServerConfig(device, FORMS[form], max_streams, hbm_budget)
        h = C.c_void_p()
        if lib().f3d_server_create(C.byref(cfg), C.byref(h)) != F3D_OK:
            raise F3DError(lib().f3d_last_error().decode())
        self._h = h
        self._geom = {}

    @staticmethod
    def _rc(rc):
        if rc == F3D_E_BUSY:
            return False
        if rc != F3D_OK:
            raise F3DError(lib().f3d_last_error().decode())
        return True

    def open(self, width: int, height: int, bits: int, nframes: int, sample_type: int = 0,
             chroma: bool = False, **params):
        """Stream id, or None when the server has no slot or budget for it now."""
        sp = script_params(**params)
        geom = PlaneGeom(width, height, bits, sample_type, int(chroma))
        sid = C.c_int(-1)
        if not self._rc(lib().f3d_server_open(self._h, C.byref(sp), C.byref(geom), nframes, C.byref(sid))):
            return None
        dtype = np.float32 if sample_type == 1 else (np.uint8 if bits <= 8 else np.uint16)
        self._geom[sid.value] = (width, height, dtype)
        return sid.value

    def submit(self, sid: int, n: int, frame: np.ndarray) -> bool:
        """Queues frame n; False when the stream's input slots are full."""
        f = np.ascontiguousarray(frame)
        return self._rc(lib().f3d_server_submit(self._h, sid, n, f.ctypes.data_as(C.c_void_p), f.strides[0]))

    def poll(self, sid: int, timeout_ms: int = 0):
        """(frame number, output plane) of the stream's next finished output,
        or None."""
        w, h, dtype = self._geom[sid]
        out = np.empty((h, w), dtype)
        n = C.c_int(-1)
        if not self._rc(lib().f3d_server_poll(self._h, sid, C.byref(n), out.ctypes.data_as(C.c_void_p),
                                              out.strides[0], timeout_ms)):
            return None
        return n.value, out

    def poll_timed(self, sid: int, timeout_ms: int = 0, out: np.ndarray | None = None):
        """(frame number, output plane, ready ms, done ms) of the stream's next
        finished output, or None: ready is when the last input frame its
        window needs arrived, done when its copy to host memory finished (one
        clock for all streams of the server). `out` (optional) receives the
        plane instead of a new array."""
        w, h, dtype = self._geom[sid]
        if out is None:
            out = np.empty((h, w), dtype)
        elif out.shape != (h, w) or out.dtype != dtype or not out.flags.c_contiguous:
            raise ValueError("FFT3DCL: output buffer does not match the stream's plane")
        n = C.c_int(-1)
        t0, t1 = C.c_double(0.0), C.c_double(0.0)
        if not self._rc(lib().f3d_server_poll_timed(self._h, sid, C.byref(n), out.ctypes.data_as(C.c_void_p),
                                                    out.strides[0], timeout_ms, C.byref(t0), C.byref(t1))):
            return None
        return n.value, out, t0.value, t1.value

    def close_stream(self, sid: int):
        self._rc(lib().f3d_server_close(self._h, sid))
        self._geom.pop(sid, None)

    def stats(self) -> dict:
        st = ServerStats()
        self._rc(lib().f3d_server_get_stats(self._h, C.byref(st)))
        return {k: getattr(st, k) for k, _ in ServerStats._fields_}

    def close(self):
        if self._h:
            lib().f3d_server_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


BATCH_GRAPH = 1
BATCH_AUTOTUNE = 2


class Batch:
    """One temporal step of up to sixteen tensor-core engines, or fast-form
    engines (the planes of a frame, planes of several streams, or one engine
    several times for consecutive outputs) with one launch per kernel
    (f3d_batch_*; the fast form: one forward launch per entering frame);
    tensor-core batches optionally replayed as a CUDA graph and autotuned."""

    def __init__(self, engines: list, graph: bool = True, autotune: bool = True):
        self.engines = list(engines)
        arr = (C.c_void_p * len(engines))(*[e._h.value for e in engines])
        h = C.c_void_p()
        flags = (BATCH_GRAPH if graph else 0) | (BATCH_AUTOTUNE if autotune else 0)
        if lib().f3d_batch_create(arr, len(engines), flags, C.byref(h)) != F3D_OK:
            raise F3DError(lib().f3d_last_error().decode())
        self._h = h

    def step(self, fns, srcs, src_pitches, windows, dsts, dst_pitches):
        """fns[i]: frame entering plane i (-1: none) from device pointer
        srcs[i]; windows[i]: the output window of plane i, written to device
        pointer dsts[i]."""
        n = len(self.engines)
        wins = [(C.c_int * len(w))(*w) for w in windows]
        wptr = (C.POINTER(C.c_int) * n)(*[C.cast(w, C.POINTER(C.c_int)) for w in wins])
        rc = lib().f3d_batch_step(self._h, (C.c_int * n)(*fns), (C.c_void_p * n)(*srcs),
                                  (C.c_size_t * n)(*src_pitches), wptr, (C.c_int * n)(*[len(w) for w in windows]),
                                  (C.c_void_p * n)(*dsts), (C.c_size_t * n)(*dst_pitches))
        if rc != F3D_OK:
            raise F3DError(lib().f3d_batch_error(self._h).decode() or lib().f3d_last_error().decode())

    def tune(self):
        a, b = C.c_int(), C.c_int()
        tuned = lib().f3d_batch_tune(self._h, C.byref(a), C.byref(b))
        return {"tuned": bool(tuned), "fwd_ctas_per_sm": a.value, "filter_minb": b.value}

    def last_kernel_ms(self) -> list[float]:
        """[filter, inverse + overlap-add + seam merge] device ms of the last
        step with outputs that ran outside a CUDA graph."""
        ms = (C.c_float * 2)()
        if lib().f3d_batch_last_kernel_ms(self._h, ms) != F3D_OK:
            raise F3DError(lib().f3d_batch_error(self._h).decode())
        return [ms[0], ms[1]]

    def set_tune(self, fwd_ctas_per_sm: int, filter_minb: int):
        """Pins the launch shape (every shape gives the same results)."""
        if lib().f3d_batch_set_tune(self._h, fwd_ctas_per_sm, filter_minb) != F3D_OK:
            raise F3DError(lib().f3d_batch_error(self._h).decode())

    def close(self):
        if self._h:
            lib().f3d_batch_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

