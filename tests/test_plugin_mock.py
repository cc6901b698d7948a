"""The VapourSynth plugin under a mock API-4 host (tests/vsmock): the same
identifier, namespace, function name and argument string as the reference
(src/fft3dcl.cpp:540-552), and its argument errors. Runs where the plugin
was built, i.e. where the VapourSynth headers were found."""
import pytest

import fft3dcl_gb300 as F
import oracle
import plugin_host

REF_ARGS = ("clip:vnode;sigma:float:opt;beta:float:opt;bw:int:opt;bh:int:opt;bt:int:opt;sharpen:float:opt;"
            "plane:int:opt;mode:int:opt;bordersize:int:opt;precision:int:opt;degrid:float:opt;scutoff:float:opt;"
            "svr:float:opt;smin:float:opt;smax:float:opt;kratio:float:opt;ow:int:opt;oh:int:opt;wintype:int:opt;"
            "interlaced:int:opt;sigma2:float:opt;sigma3:float:opt;sigma4:float:opt;oldfft:int:opt;device:int:opt")


@pytest.fixture(scope="module")
def results(tmp_path_factory):
    if not plugin_host.plugin_available():
        pytest.skip("plugin not built here (no VapourSynth headers)")
    return plugin_host.run_cases(plugin_host.compile_host(str(tmp_path_factory.mktemp("vsmock"))))


def test_registration_matches_reference(results):
    r = results["register"]
    assert r["id"] == "com.github.humbleuser33.fft3dcl"
    assert r["namespace"] == "fft3dcl"
    assert r["function"] == "FFT3DCL"
    assert r["args"] == REF_ARGS
    assert r["returns"] == "clip:vnode;"


def test_argument_errors(results):
    assert "clip" in results["no_clip"]["error"]
    ref_msg = None
    try:
        oracle.validate(oracle.script_params(bt=7), 96, 64, 8)
    except ValueError as e:
        ref_msg = str(e)
    assert ref_msg and results["bad_bt"]["error"] == ref_msg
    assert results["bad_bw"]["error"].startswith("FFT3DCL:")
    assert "device=0" in results["device0"]["error"]
    assert "greyscale" in results["gray_chroma"]["error"]
    assert "plane" in results["bad_plane"]["error"]
    assert "bit depths" in results["bad_bits"]["error"]
    for c in ("bad_bt", "bad_bw", "device0", "gray_chroma", "bad_plane", "bad_bits"):
        assert not results[c]["created"]


def test_valid_arguments_reach_the_gpu_setup(results):
    # With a GPU the filter is created and its frames come back; without one
    # the engine reports the missing device: there is no CPU fallback.
    for c in ("valid_gray", "valid_yuv_all"):
        r = results[c]
        if r["created"]:
            assert r["frame_error"] == ""
        else:
            assert r["error"].startswith("FFT3DCL: GPU setup failed") and "CUDA" in r["error"]
    assert F.live_instances() == 0
