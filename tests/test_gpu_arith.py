"""The arithmetic the kernels are built on, checked on the GPU: the refined
reciprocal that replaces IEEE division, and the FP64 pipe behaviour the
kernel design assumes (documented in the package's design notes)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_refined_reciprocal(cuda_lib):
    """rcp.approx seed + one cubic Newton-Raphson step is within one ulp of the
    correctly rounded 1/x (the reference divides), over 26 decades."""
    import torch
    from dadi_gb300 import _lib
    x = np.exp(np.random.default_rng(0).uniform(-30, 30, 1 << 18))
    d_x = torch.from_numpy(x).cuda()
    d_o = torch.empty_like(d_x)
    _lib.check(cuda_lib.dgb_probe_rcp(_lib.dptr(d_x), _lib.dptr(d_o), len(x),
                                      _lib.stream_handle(torch)), "rcp")
    r = d_o.cpu().numpy()
    exact = 1.0 / x
    ulps = np.abs(r.view(np.int64) - exact.view(np.int64))
    assert ulps.max() <= 1
    assert (ulps == 0).mean() > 0.99


def test_fp64_rate_and_idle_lanes(cuda_lib):
    """The FP64 FMA rate is positive and a warp instruction with a quarter of
    its lanes active takes as long as a full one (idle lanes are not free),
    which is why the kernels pack lines into full warps."""
    import torch
    from dadi_gb300 import _lib
    full = _lib.fp64_fma_peak_tflops(torch, active_lanes=32, target_s=0.01, repeats=2)
    quarter = _lib.fp64_fma_peak_tflops(torch, active_lanes=8, target_s=0.01, repeats=2)
    assert full > 0.1
    assert quarter < 0.5 * full
