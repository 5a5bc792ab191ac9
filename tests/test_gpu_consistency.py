"""The reference's consistency tests of its multi-population integrators
(tests/test_4D.py:4-83, tests/test_Freezing.py:10-60) run through the GPU
integrators: marginal spectra of split and integrated 4-D densities against
1-D and 2-D results, and frozen populations leaving their marginals
unchanged, with the reference's tolerances."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _split4(xx):
    from dadi_gb300 import phimanip as pm
    phi = pm.phi_1D_to_2D(xx, pm.phi_1D(xx))
    phi = pm.phi_2D_to_3D(phi, 0, xx, xx, xx)
    return pm.phi_3D_to_4D(phi, 0, 0, xx, xx, xx, xx)


def test_4d_snm_marginals(cuda_lib):
    from dadi_gb300 import integration as gi, numerics, phimanip as pm, spectrum
    xx = numerics.default_grid(30)
    fs1 = spectrum.from_phi(pm.phi_1D(xx), [5], (xx,))
    phi = gi.four_pops(_split4(xx), xx, T=0.1)
    fs4 = spectrum.from_phi(phi, [5, 5, 5, 5], (xx,) * 4)
    for ii in range(4):
        fsm = fs4.marginalize([k for k in range(4) if k != ii])
        assert np.allclose(fs1, fsm, rtol=1e-2, atol=1e-2)


def test_4d_against_2d(cuda_lib):
    """A 2-D model embedded in each pair (k, 4) of a 4-D model."""
    from dadi_gb300 import integration as gi, numerics, phimanip as pm, spectrum
    nu1 = lambda t: 0.5 + 5 * t  # noqa: E731
    nu2 = lambda t: 10 - 50 * t  # noqa: E731
    m12 = lambda t: 2 - t  # noqa: E731
    m21 = lambda t: 0.5 + 3 * t  # noqa: E731
    g1 = lambda t: -2 * t  # noqa: E731
    g2 = lambda t: 3 * t  # noqa: E731
    h1 = lambda t: 0.2 + t  # noqa: E731
    h2 = lambda t: 0.9 - t  # noqa: E731
    xx = numerics.default_grid(20)
    phi = gi.two_pops(pm.phi_1D_to_2D(xx, pm.phi_1D(xx)), xx, T=0.1, nu1=nu1, nu2=nu2,
                      m12=m12, m21=m21, gamma1=g1, gamma2=g2, h1=h1, h2=h2)
    fs2 = spectrum.from_phi(phi, [5, 5], (xx, xx))
    for k, keep in ((1, (1, 2)), (2, (0, 2)), (3, (0, 1))):
        kw = {"nu%d" % k: nu1, "nu4": nu2, "m%d4" % k: m12, "m4%d" % k: m21,
              "gamma%d" % k: g1, "gamma4": g2, "h%d" % k: h1, "h4": h2}
        phi4 = gi.four_pops(_split4(xx), xx, T=0.1, **kw)
        fs4 = spectrum.from_phi(phi4, [5, 5, 5, 5], (xx,) * 4)
        assert np.allclose(fs2, fs4.marginalize(keep), rtol=1e-2, atol=1e-2)


def test_freezing(cuda_lib):
    from dadi_gb300 import integration as gi, numerics, phimanip as pm
    xx = numerics.default_grid(30)
    phi1 = pm.phi_1D(xx)
    assert np.allclose(gi.one_pop(phi1, xx, T=0.1, nu=0.1, gamma=0.2, frozen=True), phi1,
                       rtol=1e-6)
    phi = pm.phi_1D_to_2D(xx, gi.one_pop(phi1, xx, T=0.2, nu=0.1))
    f1 = gi.two_pops(phi, xx, T=0.1, nu2=0.3, gamma2=0.5, frozen1=True)
    f2 = gi.two_pops(phi, xx, T=0.1, nu1=0.2, gamma1=0.3, frozen2=True)
    dec = gi.two_pops(phi, xx, T=0.1, nu1=0.2, gamma1=0.3, nu2=0.3, gamma2=0.5)
    rp = pm.remove_pop
    # a frozen population's marginal does not change
    assert np.allclose(rp(phi, xx, 2)[1:-1], rp(f1, xx, 2)[1:-1], rtol=1e-4)
    assert np.allclose(rp(phi, xx, 1)[1:-1], rp(f2, xx, 1)[1:-1], rtol=1e-4)
    # the other evolves as if decoupled
    assert np.allclose(rp(f2, xx, 2)[1:-1], rp(dec, xx, 2)[1:-1], rtol=5e-2)
    assert np.allclose(rp(f1, xx, 1)[1:-1], rp(dec, xx, 1)[1:-1], rtol=5e-2)
