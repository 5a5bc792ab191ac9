"""Maximum-likelihood fitting with adjoint gradients
(inference.optimize_log_lbfgsb, dadi/Inference.py:337-455): the multinomial
log-likelihood's adjoint gradient against finite differences, and fits of a
synthetic IM data set with adjoint and with finite-difference gradients
reaching the same optimum."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

P_TRUE = np.array([0.5, 2.0, 0.6, 0.15, 1.5, 0.8])
PTS = [20, 25, 30]
NS = (10, 10)


def _data():
    from dadi_gb300 import batch, spectrum
    eng = batch.Batch2D(PTS, NS)
    fs, _, _ = eng.run(P_TRUE[None, :])
    d = np.random.default_rng(11).poisson(1e4 * fs.cpu().numpy()[0]).astype(float)
    return spectrum.Spectrum(d)


def test_multinomial_gradient_matches_fd(cuda_lib):
    from dadi_gb300 import batch, inference
    eng = batch.Batch2D(PTS, NS)
    data = _data()
    d = np.ma.getdata(data)
    # T / dt must not be an integer: there the likelihood has a kink in the
    # parameters that set dt (here m12 does: dt = 1e-3 / m12) and finite
    # differences straddle it; T * m12 / 1e-3 = 199.8
    p = P_TRUE * np.array([1.1, 0.9, 1.2, 1.07, 0.83, 1.3])
    ll, g, _ = eng.loglik_and_grad(p[None, :], d, mask=np.ma.getmaskarray(data),
                                   multinom=True)

    def llm(q):
        fs, _, _ = eng.run(q[None, :])
        return float(inference.ll_multinom(fs.cpu().numpy()[0], data))
    assert abs(float(ll.cpu().numpy()[0]) - llm(p)) < 1e-9 * abs(llm(p))

    def fd(eps):
        out = np.zeros(6)
        for k in range(6):
            h = eps * p[k]
            a, b = p.copy(), p.copy()
            a[k] += h
            b[k] -= h
            out[k] = (llm(a) - llm(b)) / (2 * h)
        return out
    d1, d2 = fd(1e-4), fd(5e-5)
    rich = (4 * d2 - d1) / 3
    g = g.cpu().numpy()[0]
    assert np.max(np.abs(g - rich)) / np.max(np.abs(rich)) < 1e-6, (g, rich)


def test_adjoint_fit_matches_fd_fit(cuda_lib):
    from dadi_gb300 import inference, models, numerics
    data = _data()
    func = numerics.make_extrap_func(models.IM)
    p0 = P_TRUE * np.array([1.2, 0.8, 1.3, 0.9, 1.1, 0.85])
    lb = [0.01, 0.01, 0.01, 0.001, 0, 0]
    ub = [0.99, 100, 100, 5, 20, 20]
    xa, fa, ia = inference.optimize_log_lbfgsb(p0, data, models.IM, PTS, lb, ub,
                                               full_output=True, gradient="adjoint")
    xf, ff, inf = inference.optimize_log_lbfgsb(p0, data, func, PTS, lb, ub,
                                                full_output=True, gradient="fd")
    lla = float(inference.ll_multinom(func(xa, NS, PTS), data))
    llf = float(inference.ll_multinom(func(xf, NS, PTS), data))
    # both reach the optimum; the exact gradient is at least as good
    assert lla >= llf - 1e-3 * abs(llf), (lla, llf, xa, xf)
    assert np.max(np.abs(np.log(xa[:4] / xf[:4]))) < 0.05, (xa, xf)
    # and needs far fewer model evaluations than finite differences
    assert ia["model_evaluations"] * 3 < inf["model_evaluations"], (ia, inf)
