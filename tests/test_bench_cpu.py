"""Host-side figures of bench.py that the JSON line is built from: the
algorithmic bytes per output frame of the 4K workload and the DRAM-traffic
table of the filter launch at the default batch step."""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import bench  # noqa: E402


def test_algorithmic_bytes_of_the_4k_workload():
    # 3840x2160 with 32x32 blocks at half overlap: 121 x 68 cells, 32912
    # blocks of 32 x 17 bins; per output frame the 10-bit plane in and out
    # (16,588,800 B each), the new spectrum written once and the four window
    # spectra read once.
    ab = bench.algorithmic_bytes(32912, 17, 32, 4)
    assert ab["plane"] == 3840 * 2160 * 2 == 16588800
    assert ab["spectrum"] == 32912 * 17 * 32 * 8 == 143233024
    assert ab["frame"] == 749342720
    assert ab["filter_inverse"] == 4 * 143233024


def test_default_batch_step_has_measured_filter_traffic():
    k = bench.DEFAULT_OUTPUTS_PER_STEP
    assert 1 <= k <= 16
    traffic = bench.NCU_TRAFFIC_BATCH[k]
    # The launch reads the k + 3 distinct window spectra once and writes the
    # k outputs' operand tiles: below the k x 4 spectra of algorithmic reads.
    spec = 143233024
    assert (k + 3) * spec * 0.95 < traffic < k * 4 * spec


def test_algorithmic_bytes_of_the_other_workloads():
    # Block counts and spectrum sizes from the oracle's own geometry.
    import oracle
    g = oracle.Plane(640, 360, 8, **bench.GRAY8_PARAMS)
    spec = g.nb * g.fbw * g.ip.bh * 8
    assert bench.AB_GRAY8 == 2 * 640 * 360 + spec * (1 + 3) == 18008064
    k = oracle.Plane(1280, 720, 32, 1, **bench.KALMAN_PARAMS)
    bins = k.nb * k.fbw * k.ip.bh
    assert bench.AB_KALMAN == 2 * 1280 * 720 * 4 + 2 * 16 * bins == 75497472
    y = oracle.Plane(1920, 1080, 8, **bench.YUV_PARAMS)
    u = oracle.Plane(960, 540, 8, chroma=True, **bench.YUV_PARAMS)
    sy, su = (p.nb * p.fbw * p.ip.bh * 8 for p in (y, u))
    assert bench.AB_YUV1080 == 2 * 1920 * 1080 + sy * 5 + 2 * (2 * 960 * 540 + su * 5) == 289187840


def test_sections_are_the_extra_workloads():
    # `--section NAME` runs one extra workload alone; the names are the keys
    # the full line carries.
    import inspect
    src = inspect.getsource(bench.extra_section)
    for name in bench.SECTIONS:
        assert f'"{name}"' in src
    assert set(bench.SECTIONS) == {"yuv1080p_all_planes", "gray8_640x360_bt3", "grays_1280x720_kalman_bw64"}
