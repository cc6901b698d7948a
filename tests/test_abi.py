"""Host-side checks that need no GPU: the C-ABI library loads and exports
every entry point include/fft3d_gb300.h declares, the engine's parameter
contract equals the oracle's (itself pinned to the reference), defaults match
the plugin's, and without a CUDA device the engine fails loudly instead of
falling back to the CPU."""
import ctypes as C
import os
import re
import subprocess
import sys

import numpy as np
import pytest

import fft3dcl_gb300 as F
import oracle

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "fft3d_gb300.h")


def declared_symbols():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(f3d_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol():
    lib = F.lib()
    syms = declared_symbols()
    assert len(syms) >= 20
    for s in syms:
        assert hasattr(lib, s), s
    assert set(syms) == set(F.EXPORTS)


def test_default_params_match_plugin_defaults():
    sp = F.ScriptParams()
    F.lib().f3d_default_params(C.byref(sp))
    ref = F.script_params()
    for name, _ in F.ScriptParams._fields_:
        assert getattr(sp, name) == getattr(ref, name), name


def test_validate_params_matches_oracle():
    rng = np.random.default_rng(11)
    for _ in range(300):
        kw = dict(bw=int(rng.integers(1, 600)), bh=int(rng.integers(1, 600)), bt=int(rng.integers(-2, 6)),
                  mode=int(rng.integers(-1, 4)), sigma=float(rng.uniform(0.1, 9)),
                  beta=float(rng.uniform(0.5, 3)), smin=float(rng.uniform(0, 8)),
                  sigma2=float(rng.choice([2.0, 3.0])), interlaced=int(rng.integers(0, 2)) * int(rng.integers(0, 2)))
        kw["ow"] = int(rng.integers(0, kw["bw"] + 2))
        kw["oh"] = int(rng.integers(0, kw["bh"] + 2))
        w, h, bits = int(rng.integers(1, 4000)), int(rng.integers(1, 3000)), int(rng.choice([8, 10, 12, 16, 32]))
        try:
            ref = oracle.validate(oracle.script_params(**kw), w, h, bits)
        except ValueError as e:
            with pytest.raises(ValueError) as ex:
                F.validate(w, h, bits, **kw)
            assert str(ex.value) == str(e)
            continue
        mine = F.validate(w, h, bits, **kw)
        for name, _ in F.InternalParams._fields_:
            assert getattr(mine, name) == getattr(ref, name), (name, kw)


@pytest.mark.parametrize("params", [
    {}, {"bt": 4, "sharpen": 0.4}, {"wintype": 1, "bw": 16, "ow": 6}, {"wintype": 2, "bh": 64, "bw": 8},
    {"mode": 0, "sharpen": -0.5, "svr": 0.3}, {"sigma2": 3.0, "sigma3": 1.0, "sigma4": 0.5, "bt": 2},
    {"bw": 64, "bh": 64, "bt": 0, "sigma2": 1.5, "sigma3": 2.5, "sigma4": 3.0, "degrid": 0.6},
    {"bw": 4, "bh": 4, "scutoff": 0.1, "sharpen": 2.0},
])
def test_engine_tables_equal_oracle_tables(params):
    # The kernels read these tables; built on the host with no fused
    # multiply-add they must equal the oracle's (and so the reference's) bits
    # on either host architecture.
    pl = oracle.Plane(200, 120, 8, **params)
    pl.build_degrid()
    for which in range(9):
        mine = F.compute_table(which, 200, 120, 8, **params)
        ref = pl.table(which)
        if which in (F.TAB_GS_RE, F.TAB_GS_IM) and not F.validate(200, 120, 8, **params).degrid_on:
            assert mine.size == 0
            continue
        np.testing.assert_array_equal(mine, ref, err_msg=f"table {which}")


def test_bad_bt_message_is_the_reference_one():
    with pytest.raises(ValueError, match="valid modes for bt are -1,0,1,2,3,4"):
        F.validate(640, 360, 8, bt=5)
    with pytest.raises(ValueError, match="mode 2 is not implemented"):
        F.validate(640, 360, 8, mode=2)


def test_unknown_parameter_rejected():
    with pytest.raises(TypeError):
        F.script_params(sigmaa=3.0)


def test_product_does_not_import_the_oracle():
    code = ("import sys; import fft3dcl_gb300, fft3dcl_gb300.synth; "
            "assert 'oracle' not in sys.modules, 'oracle imported'")
    subprocess.run([sys.executable, "-c", code], cwd=ROOT, check=True)
    pkg = os.path.join(ROOT, "fft3dcl_gb300")
    for dirpath, _, files in os.walk(pkg):
        for f in files:
            if f.endswith((".py", ".cpp", ".cu", ".cuh", ".hpp")):
                txt = open(os.path.join(dirpath, f)).read()
                assert "import oracle" not in txt and "liboracle" not in txt, f


def _has_gpu():
    try:
        out = subprocess.run(["nvidia-smi", "-L"], capture_output=True, text=True, timeout=20)
        return out.returncode == 0 and "GPU" in out.stdout
    except Exception:
        return False


@pytest.mark.skipif(_has_gpu(), reason="checks the no-GPU error path")
def test_engine_fails_loudly_without_gpu():
    with pytest.raises(F.F3DError, match="CUDA"):
        F.Engine(64, 48, 8)
    assert F.live_instances() == 0
    assert F.live_bytes() == 0


def test_large_blocks_validate_like_the_reference():
    # Block sizes round up to powers of two and clamp to 512, as the
    # reference CPU backend does (src/params.h:62-72); the engine takes them
    # all (its OpenCL backend stopped at 64, src/cl/gpu.cpp:82-89).
    for bw, want in ((100, 128), (256, 256), (300, 512), (1000, 512)):
        ip = F.validate(1280, 720, 8, bw=bw, bh=bw)
        ref = oracle.validate(oracle.script_params(bw=bw, bh=bw), 1280, 720, 8)
        assert ip.bw == ip.bh == want == ref.bw == ref.bh
        assert (ip.nx, ip.ny, ip.ow, ip.oh) == (ref.nx, ref.ny, ref.ow, ref.oh)


def test_plane_selection_errors():
    frames = [[np.zeros((16, 16), np.uint8)]]
    with pytest.raises(ValueError, match="greyscale"):
        F.Filter(frames, F.VideoFormat("gray", 8), plane=1)
    with pytest.raises(ValueError, match="device=0"):
        F.Filter(frames, F.VideoFormat("gray", 8), device=0)
    with pytest.raises(ValueError, match="bit depths"):
        F.Filter(frames, F.VideoFormat("gray", 20))
