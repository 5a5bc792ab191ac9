"""The reference's own known-answer tests (tests/test_Results.py:5-41) run
through the GPU integrator: the standard neutral spectrum theta/i, a
two-epoch model relaxed to its new equilibrium, and the IM spectrum against
the ms coalescent simulation dadi ships (tests/IM.fs, stored in
tests/golden/known.npz), with log-extrapolation as the reference tests use."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_snm_is_one_over_i(cuda_lib):
    from dadi_gb300 import models, numerics
    fs = numerics.make_extrap_log_func(models.snm_1d)([], (17,), [100, 120, 140])
    with np.errstate(divide="ignore"):
        answer = np.ma.masked_array(1. / np.arange(18), mask=np.ma.getmaskarray(fs))
    assert np.ma.allclose(fs, answer, atol=1e-3)


def test_two_epoch_relaxes_to_new_equilibrium(cuda_lib):
    """After tau = 10 at half the size, the spectrum is the new equilibrium's
    0.5 / i (the one_pop GPU path over 1e4 steps)."""
    from dadi_gb300 import models, numerics
    fs = numerics.make_extrap_log_func(models.two_epoch)((0.5, 10), (17,), [40, 50, 60])
    with np.errstate(divide="ignore"):
        answer = np.ma.masked_array(0.5 / np.arange(18), mask=np.ma.getmaskarray(fs))
    assert np.ma.allclose(fs, answer, atol=1e-2)


def test_im_matches_coalescent_simulation(cuda_lib, golden):
    from dadi_gb300 import inference, models, numerics, spectrum
    k = golden["known"]
    msfs = spectrum.Spectrum(k["im_ms_data"], mask=k["im_ms_mask"])
    fs = 1000. * numerics.make_extrap_log_func(models.IM)(
        (0.8, 2.0, 0.6, 0.45, 5.0, 0.3), (7, 13), [40, 50, 60])
    resid = inference.Anscombe_Poisson_residual(fs, msfs)
    assert abs(resid).max() < 0.2
