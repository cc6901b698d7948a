"""YUV4MPEG2 (.y4m) clips: a lazy, random-access reader and a writer.

Feeds real material to the filter (the reference drives its tests through
ffmpeg/FFV1 on Windows, tools/run_test.ps1): planar 8-bit and high-bit-depth
(little-endian 16-bit words) 4:2:0, 4:2:2, 4:4:4 and monochrome. Frames are
lists of 2D numpy planes, the clip layout ``Filter`` takes.
"""
from __future__ import annotations

import os
from collections import OrderedDict

import numpy as np

# Y4M colour-space tag -> (chroma subsampling log2 w, h or None for mono, bits)
_CSP = {
    "420jpeg": (1, 1, 8), "420paldv": (1, 1, 8), "420mpeg2": (1, 1, 8), "420": (1, 1, 8),
    "422": (1, 0, 8), "444": (0, 0, 8), "mono": (None, None, 8),
    "420p10": (1, 1, 10), "422p10": (1, 0, 10), "444p10": (0, 0, 10),
    "420p12": (1, 1, 12), "422p12": (1, 0, 12), "444p12": (0, 0, 12),
    "420p16": (1, 1, 16), "422p16": (1, 0, 16), "444p16": (0, 0, 16),
    "mono10": (None, None, 10), "mono12": (None, None, 12), "mono16": (None, None, 16),
}


def _csp_tag(sub_w, sub_h, bits, mono):
    for tag, v in _CSP.items():
        if v == ((None, None, bits) if mono else (sub_w, sub_h, bits)) and tag not in ("420paldv", "420mpeg2", "420"):
            return tag
    raise ValueError("no Y4M colour space for this format")


class Y4MClip:
    """Random-access frames of a .y4m file (indexed once, read on demand,
    the last `cache` frames kept)."""

    def __init__(self, path: str, cache: int = 8):
        self.path = path
        self._f = open(path, "rb")
        line = self._f.readline()
        if not line.startswith(b"YUV4MPEG2"):
            raise ValueError(f"{path}: not a YUV4MPEG2 stream")
        self.header = line.rstrip(b"\n").decode("ascii")
        fields = {t[0]: t[1:] for t in self.header.split()[1:]}
        self.width, self.height = int(fields["W"]), int(fields["H"])
        csp = fields.get("C", "420jpeg")
        if csp not in _CSP:
            raise ValueError(f"{path}: unsupported colour space C{csp}")
        sw, sh, self.bits = _CSP[csp]
        self.mono = sw is None
        self.sub_w, self.sub_h = (0, 0) if self.mono else (sw, sh)
        self.bps = 1 if self.bits <= 8 else 2
        self.dtype = np.uint8 if self.bps == 1 else np.dtype("<u2")
        cw = (self.width + (1 << self.sub_w) - 1) >> self.sub_w
        ch = (self.height + (1 << self.sub_h) - 1) >> self.sub_h
        self.shapes = [(self.height, self.width)] + ([] if self.mono else [(ch, cw)] * 2)
        self.frame_bytes = sum(h * w for h, w in self.shapes) * self.bps
        # Index the frames: each is a FRAME line (possibly with parameters) + payload.
        self._offsets = []
        size = os.path.getsize(path)
        pos = self._f.tell()
        while pos < size:
            self._f.seek(pos)
            fl = self._f.readline()
            if not fl.startswith(b"FRAME"):
                raise ValueError(f"{path}: bad frame header at byte {pos}")
            start = pos + len(fl)
            if start + self.frame_bytes > size:
                raise ValueError(f"{path}: truncated frame {len(self._offsets)}")
            self._offsets.append(start)
            pos = start + self.frame_bytes
        self._cache: OrderedDict[int, list[np.ndarray]] = OrderedDict()
        self._cap = cache

    def __len__(self) -> int:
        return len(self._offsets)

    def __getitem__(self, n: int) -> list[np.ndarray]:
        if n < 0:
            n += len(self)
        if n in self._cache:
            self._cache.move_to_end(n)
            return self._cache[n]
        self._f.seek(self._offsets[n])
        buf = self._f.read(self.frame_bytes)
        planes, o = [], 0
        for h, w in self.shapes:
            nbytes = h * w * self.bps
            planes.append(np.frombuffer(buf, self.dtype, h * w, o).reshape(h, w).astype(
                np.uint8 if self.bps == 1 else np.uint16))
            o += nbytes
        self._cache[n] = planes
        if len(self._cache) > self._cap:
            self._cache.popitem(last=False)
        return planes

    def close(self):
        self._f.close()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


class Y4MWriter:
    """Writes frames (lists of planes) with the header of the source clip, or
    a header built from width, height, bits and subsampling."""

    def __init__(self, path: str, header: str | None = None, width: int = 0, height: int = 0, bits: int = 8,
                 sub_w: int = 1, sub_h: int = 1, mono: bool = False, fps: str = "25:1"):
        if header is None:
            header = f"YUV4MPEG2 W{width} H{height} F{fps} Ip A1:1 C{_csp_tag(sub_w, sub_h, bits, mono)}"
        self._f = open(path, "wb")
        self._f.write(header.encode("ascii") + b"\n")
        self.bits = int(_CSP[{t[0]: t[1:] for t in header.split()[1:]}.get("C", "420jpeg")][2])

    def write(self, planes: list[np.ndarray]):
        self._f.write(b"FRAME\n")
        for p in planes:
            a = np.ascontiguousarray(p, np.uint8 if self.bits <= 8 else np.dtype("<u2"))
            self._f.write(a.tobytes())

    def close(self):
        self._f.close()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()
