"""The tensor-core kernels' bounded waits, made to run out.

Every mbarrier wait of the tensor-core kernels gives up after one second: the
CTA agrees on it, sets its bit in the engine's error word, frees its tensor
memory and leaves, and f3d_synchronize reports the wait. The test flag
F3D_FLAG_TEST_WAIT_TIMEOUT makes the inverse kernel's first CTA leave out its
first operand-tile copy, so that the wait for it runs out with no copy and
no tensor-core product in flight. The GPU stays usable: the next output of
the same engine and a fresh engine are both correct."""
import numpy as np
import pytest

import fft3dcl_gb300 as F
import oracle
from fft3dcl_gb300 import synth

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def test_operand_copy_wait_gives_up_and_is_reported():
    frames = synth.moving_rects(200, 136, 4, 5, lo=16, hi=235, noise=3.0)
    params = dict(bt=3, sharpen=0.2)
    ref = oracle.run_clip(frames, 8, **params)
    with F.Engine(200, 136, 8, form="tc", flags=F.FLAG_TEST_WAIT_TIMEOUT, **params) as e:
        info = e.info()
        assert info.form == F.FORMS["tc"] and info.fused
        for fn in range(3):
            e.forward_raw(fn, frames[fn])
        # Queued; inside the kernel the wait gives up after one second.
        dst = torch.empty((136, 200), dtype=torch.uint8, device="cuda")
        e.process_device([0, 1, 2], dst.data_ptr(), 200)
        with pytest.raises(F.F3DError, match="tensor-core wait timed out: inverse kernel \\(operand tile copy\\)"):
            e.synchronize()
        # Reported once; the next output of the same engine is correct.
        e.synchronize()
        out = e.process_raw([0, 1, 2])
        assert int(np.abs(out.astype(int) - ref[1].astype(int)).max()) <= 1
    assert F.live_instances() == 0
    # A fresh engine on the same GPU: bit-equal to the oracle in the exact form.
    got = F.FFT3DCL(frames, **params)
    for g, r in zip(got, ref):
        np.testing.assert_array_equal(g, r)
