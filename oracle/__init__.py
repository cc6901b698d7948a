"""ctypes bindings for the CPU oracle (test infrastructure only).

Only the tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this package, and only as the oracle the CUDA path is
compared with (or, for the CPU baseline, timed beside). The product (the
``fft3dcl_gb300`` package and its CUDA library) never imports it.

Two libraries are bound here:

* ``liboracle.so``: the C restatement of the reference's fp32 CPU backend
  (``fft3d_oracle.c``; built by ``make -C oracle`` or ``__graft_entry__.build``).
* ``_ref/libfft3dref.so``: the reference's own CPU backend (src/cpu/*.cpp,
  src/params.h) compiled where it lies by ``make -C oracle ref``. It only exists
  where the reference sources are available and is used to pin the restatement.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_PATH = os.path.join(HERE, "_ref", "libfft3dref.so")


class ScriptParams(C.Structure):
    """Script-level parameters, src/params.h:8-27 (same defaults)."""

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
    """Validated parameters, src/params.h:30-59."""

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


def script_params(**kw) -> ScriptParams:
    """ScriptParams with the plugin's defaults, including the parameter-
    dependent ones (src/fft3dcl.cpp:171-195): degrid = 1 if mode == 1 else 0,
    ow/oh = bw/2, bh/2 of the script values, sigma2/3/4 = sigma."""
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


_lib = None
_ref = None


def build(ref: bool = False) -> None:
    """Compile the restatement (and the pinned reference when asked and when
    its sources are present)."""
    subprocess.run(["make", "-s", "-C", HERE, "liboracle.so"], check=True)
    if ref and os.path.isdir("/root/reference/src/cpu"):
        subprocess.run(["make", "-s", "-C", HERE, "ref"], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        P = C.POINTER
        L.orc_validate_params.argtypes = [P(ScriptParams), C.c_int, C.c_int, C.c_int,
                                          P(InternalParams), P(C.c_char_p)]
        L.orc_plane_new.restype = C.c_void_p
        L.orc_plane_new.argtypes = [P(InternalParams), C.c_int, C.c_int, C.c_int, C.c_int, C.c_int]
        L.orc_plane_free.argtypes = [C.c_void_p]
        for f in ("orc_nblocks", "orc_fbw", "orc_ncols"):
            getattr(L, f).argtypes = [C.c_void_p]
        L.orc_chroma_norm.argtypes = [C.c_void_p]
        L.orc_chroma_norm.restype = C.c_float
        L.orc_get_grid.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        L.orc_get_table.argtypes = [C.c_void_p, C.c_int, C.c_void_p]
        L.orc_upload.argtypes = [C.c_void_p, C.c_void_p, C.c_ssize_t, C.c_void_p]
        L.orc_download.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_ssize_t]
        L.orc_compute_spectra.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]
        L.orc_build_degrid.argtypes = [C.c_void_p]
        L.orc_filter_and_synthesize.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int,
                                                C.c_void_p, C.c_int]
        L.orc_fft1d.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_int]
        L.orc_fft2d_forward.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p]
        L.orc_fft2d_inverse_half.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p]
        L.orc_run_clip.argtypes = [P(ScriptParams), C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                   C.c_int, C.c_void_p, C.c_ssize_t, C.c_int, C.c_int, C.c_void_p,
                                   C.c_ssize_t, C.c_int, P(C.c_char_p)]
        L.orc_round_pow2_clamp.argtypes = [C.c_int]
        _lib = L
    return _lib


def ref_available() -> bool:
    return os.path.exists(REF_PATH)


def ref():
    """The reference's own CPU backend, or None when it is not built here."""
    global _ref
    if _ref is None:
        if not ref_available():
            return None
        R = C.CDLL(REF_PATH)
        P = C.POINTER
        R.ref_validate.argtypes = [P(ScriptParams), C.c_int, C.c_int, C.c_int,
                                   P(C.c_double), P(C.c_char_p)]
        R.ref_fft1d.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_int]
        R.ref_get_table.argtypes = [P(ScriptParams), C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                    C.c_int, C.c_void_p]
        R.ref_spectra.argtypes = [P(ScriptParams), C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                  C.c_void_p, C.c_void_p, C.c_void_p]
        R.ref_run_clip.argtypes = [P(ScriptParams), C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                   C.c_int, C.c_void_p, C.c_ssize_t, C.c_int, C.c_int, C.c_void_p,
                                   C.c_ssize_t, P(C.c_char_p)]
        _ref = R
    return _ref


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


def _ptr_array(frames):
    arr = (C.c_void_p * len(frames))()
    for i, f in enumerate(frames):
        arr[i] = f.ctypes.data
    return arr


def fmt_info(dtype) -> tuple[int, int]:
    """(sample_type, bytes per sample) for a numpy sample dtype."""
    dt = np.dtype(dtype)
    if dt == np.float32:
        return 1, 4
    if dt == np.uint8:
        return 0, 1
    if dt == np.uint16:
        return 0, 2
    raise ValueError(f"unsupported sample type {dt}")


def validate(sp: ScriptParams, width: int, height: int, bits: int):
    """Returns InternalParams, or raises ValueError with the reference's message."""
    ip = InternalParams()
    err = C.c_char_p()
    if not lib().orc_validate_params(C.byref(sp), width, height, bits, C.byref(ip), C.byref(err)):
        raise ValueError(err.value.decode())
    return ip


def run_clip(frames: list[np.ndarray], bits: int, first: int = 0, count: int | None = None,
             chroma: bool = False, threads: int = 1, impl: str = "oracle", **params) -> list[np.ndarray]:
    """Run one plane of a clip through the oracle (impl='oracle') or through the
    reference's compiled CPU backend (impl='ref'). Frames are 2D numpy arrays of
    uint8, uint16 or float32; output frames first..first+count-1 are returned."""
    sp = script_params(**params)
    h, w = frames[0].shape
    st, bps = fmt_info(frames[0].dtype)
    frames = [np.ascontiguousarray(f) for f in frames]
    if count is None:
        count = len(frames) - first
    outs = [np.zeros_like(frames[0]) for _ in range(count)]
    err = C.c_char_p()
    if impl == "oracle":
        rc = lib().orc_run_clip(C.byref(sp), w, h, bits, st, int(chroma), len(frames),
                                _ptr_array(frames), w * bps, first, count, _ptr_array(outs),
                                w * bps, threads, C.byref(err))
    else:
        R = ref()
        if R is None:
            raise RuntimeError("reference CPU backend is not built here")
        rc = R.ref_run_clip(C.byref(sp), w, h, bits, st, int(chroma), len(frames),
                            _ptr_array(frames), w * bps, first, count, _ptr_array(outs),
                            w * bps, C.byref(err))
    if rc != 0:
        raise ValueError(err.value.decode())
    return outs


class Plane:
    """One plane of the oracle pipeline (the reference's PlaneRef,
    src/cpu/reference.h:24-103)."""

    def __init__(self, width, height, bits=8, sample_type=0, chroma=False, **params):
        self.sp = script_params(**params)
        self.ip = validate(self.sp, width, height, bits)
        self.width, self.height, self.bits, self.sample_type = width, height, bits, sample_type
        self.h = lib().orc_plane_new(C.byref(self.ip), width, height, bits, sample_type, int(chroma))
        L = lib()
        self.nb = L.orc_nblocks(self.h)
        self.fbw = L.orc_fbw(self.h)
        self.ncols = L.orc_ncols(self.h)
        self.chroma_norm = L.orc_chroma_norm(self.h)

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_plane_free(self.h)
            self.h = None

    def grid(self):
        bx = np.zeros(self.nb, np.int32)
        by = np.zeros(self.nb, np.int32)
        par = np.zeros(self.nb, np.uint8)
        lib().orc_get_grid(self.h, _ptr(bx), _ptr(by), _ptr(par))
        return bx, by, par

    def table(self, which: int) -> np.ndarray:
        n = lib().orc_get_table(self.h, which, None)
        out = np.zeros(max(n, 0), np.float32)
        if n > 0:
            lib().orc_get_table(self.h, which, _ptr(out))
        return out

    def upload(self, frame: np.ndarray) -> np.ndarray:
        frame = np.ascontiguousarray(frame)
        out = np.zeros((self.height, self.width), np.float32)
        lib().orc_upload(self.h, _ptr(frame), frame.strides[0], _ptr(out))
        return out

    def download(self, plane: np.ndarray, dtype) -> np.ndarray:
        out = np.zeros((self.height, self.width), dtype)
        plane = np.ascontiguousarray(plane, np.float32)
        lib().orc_download(self.h, _ptr(plane), _ptr(out), out.strides[0])
        return out

    def spectra(self, plane: np.ndarray, threads: int = 1) -> np.ndarray:
        """Half spectra as complex64 [nblocks, bh, fbw]."""
        plane = np.ascontiguousarray(plane, np.float32)
        n = self.nb * self.fbw * self.ip.bh
        re = np.zeros(n, np.float32)
        im = np.zeros(n, np.float32)
        lib().orc_compute_spectra(self.h, _ptr(plane), _ptr(re), _ptr(im), threads)
        return (re + 1j * im).astype(np.complex64).reshape(self.nb, self.ip.bh, self.fbw)

    def build_degrid(self):
        lib().orc_build_degrid(self.h)

    def filter_and_synthesize(self, window: list[np.ndarray], threads: int = 1) -> np.ndarray:
        res = [np.ascontiguousarray(w.real.ravel(), np.float32) for w in window]
        ims = [np.ascontiguousarray(w.imag.ravel(), np.float32) for w in window]
        out = np.zeros((self.height, self.width), np.float32)
        lib().orc_filter_and_synthesize(self.h, _ptr_array(res), _ptr_array(ims), len(window),
                                        _ptr(out), threads)
        return out


def fft1d(x: np.ndarray, inverse: bool = False, impl: str = "oracle") -> np.ndarray:
    x = np.ascontiguousarray(x, np.complex64)
    out = np.zeros_like(x)
    f = lib().orc_fft1d if impl == "oracle" else ref().ref_fft1d
    f(len(x), _ptr(x), _ptr(out), int(inverse))
    return out
