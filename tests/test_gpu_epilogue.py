"""The device spectrum epilogue (dgb_from_phi2d, dgb_extrap_ll) against the
oracle's from_phi, extrapolation and Poisson log-likelihood (the reference's
arithmetic, pinned to dadi's golden vectors in test_oracle.py).

Tolerance: the contraction sums the same terms as numpy's matrix products in
another order, and terms of both signs cancel, so entries agree to a few ulps
of the larger terms: 1e-11 relative on entries >= 1e-12 of the maximum,
1e-24 of the maximum absolute below that.  A spectrum is bitwise the same
whatever else shares the launch.
"""
import numpy as np
import pytest

from util import max_rel

pytestmark = pytest.mark.gpu

REL = 1e-11


def _close(a, b):
    a, b = np.asarray(a), np.asarray(b)
    mx = np.max(np.abs(b))
    big = np.abs(b) >= 1e-12 * mx
    assert max_rel(a[big], b[big]) <= REL, max_rel(a[big], b[big])
    assert np.max(np.abs(a[~big] - b[~big]), initial=0.0) <= 1e-24 * mx


def _phis(pts_l, params=(0.4, 0.3, 2.0, 0.2, 1.5, 0.7)):
    """(density, grid) of a real IM integration on each grid, from the
    oracle (its two_pops loop over the C sweeps)."""
    from oracle import integration as oint, numerics as onum
    s, nu1, nu2, T, m12, m21 = params
    out = []
    for L in pts_l:
        xx = onum.default_grid(L)
        phi = onum.phi_1D_to_2D(xx, onum.phi_1D(xx))
        phi = oint.two_pops(phi, xx, T, lambda t: s * (nu1 / s) ** (t / T),
                            lambda t: (1 - s) * (nu2 / (1 - s)) ** (t / T), m12=m12, m21=m21)
        out.append((phi, xx))
    return out


@pytest.mark.parametrize("pts_l,ns", [((30,), (10, 10)), ((40, 50, 60), (20, 20)),
                                      ((40, 50), (12, 17)), ((80, 90, 100), (40, 40))])
def test_from_phi_extrap_ll_match_oracle(cuda_lib, pts_l, ns):
    """Raw per-grid spectra to REL; the extrapolation and likelihood
    arithmetic to REL on the same raw spectra (extrapolation weights of
    order 1e2 with cancellation amplify ulp-level differences of the raw
    spectra, so end to end the extrapolated spectrum is held to the 1e-9
    spectrum bar)."""
    import torch
    from dadi_gb300 import epilogue
    from oracle import numerics as onum
    from util import assert_fs_parity
    pairs = _phis(pts_l)
    xxs = [xx for _, xx in pairs]
    x_l = [xx[1] for xx in xxs]
    d_phis = [torch.from_numpy(phi).cuda() for phi, _ in pairs]
    raw_ref = [onum.from_phi(phi, ns, xx) for phi, xx in pairs]
    raw_dev = []
    for d, xx, ref in zip(d_phis, xxs, raw_ref):
        f1, l1, _ = epilogue.spectra_2d(torch, [([d], [xx], ns, None, 1.0)])
        raw_dev.append(f1[0].cpu().numpy())
        _close(raw_dev[-1], ref)
        assert np.isnan(float(l1[0]))

    ex_ref = onum.extrapolate(raw_ref, x_l)
    mask = onum.corner_mask(ex_ref.shape)
    data = np.random.default_rng(1).poisson(1e3 * np.abs(ex_ref)).astype(np.float64)
    fs, ll, _ = epilogue.spectra_2d(torch, [(d_phis, xxs, ns, torch.from_numpy(data).cuda(),
                                             1e3)])
    fs = fs[0].cpu().numpy()
    _close(fs, onum.extrapolate(raw_dev, x_l))
    assert_fs_parity(fs, ex_ref)
    ok = ~mask & (fs > 0)
    m = 1e3 * fs[ok]
    scale = np.sum(np.abs(m)) + np.sum(np.abs(data[ok] * np.log(m)))
    assert abs(float(ll[0]) - onum.ll(1e3 * fs, data, mask)) <= 1e-12 * scale


def test_fail_mag_guard(cuda_lib):
    """Entries whose extrapolation lands more than fail_mag orders of
    magnitude from the finest grid's value take that value
    (dadi/Numerics.py:449-464); with fail_mag = 1e-3 most entries trip it.
    Compared with the oracle's extrapolation of the same raw spectra."""
    import torch
    from dadi_gb300 import epilogue
    from oracle import numerics as onum
    ns = (10, 10)
    pairs = _phis((30, 40, 50))
    xxs = [xx for _, xx in pairs]
    x_l = [xx[1] for xx in xxs]
    d_phis = [torch.from_numpy(phi).cuda() for phi, _ in pairs]
    raws = [epilogue.spectra_2d(torch, [([d], [xx], ns, None, 1.0)])[0][0].cpu().numpy()
            for d, xx in zip(d_phis, xxs)]
    for fail_mag in (10.0, 1e-3):
        ref = onum.extrapolate(raws, x_l, fail_mag=fail_mag)
        fs, _, _ = epilogue.spectra_2d(torch, [(d_phis, xxs, ns, None, 1.0)],
                                       fail_mag=fail_mag)
        _close(fs[0].cpu().numpy(), ref)
    best = raws[int(np.argmin(x_l))]
    assert np.mean(ref == best) > 0.5


def test_batch_and_list_forms_agree_bitwise(cuda_lib):
    """spectra_2d_batch (one grid set, many densities) and spectra_2d (a
    list of jobs) produce identical bits, alone or together."""
    import torch
    from dadi_gb300 import batch, epilogue
    import cases
    eng = batch.Batch2D((30, 40, 50), (12, 12))
    draws = cases.im_draws(6)
    phis, _ = eng.integrate(batch.im_instances(draws))
    data = torch.ones(13, 13, dtype=torch.float64, device="cuda")
    fs_b, ll_b = epilogue.spectra_2d_batch(torch, phis, eng.xxs, (12, 12), data, 10.0)
    jobs = [([p[i] for p in phis], eng.xxs, (12, 12), data, 10.0) for i in range(6)]
    fs_l, ll_l, _ = epilogue.spectra_2d(torch, jobs)
    for i in range(6):
        assert np.array_equal(fs_b[i].cpu().numpy(), fs_l[i].cpu().numpy())
        alone, ll1, _ = epilogue.spectra_2d(torch, [jobs[i]])
        assert np.array_equal(alone[0].cpu().numpy(), fs_b[i].cpu().numpy())
        assert float(ll1[0]) == float(ll_b[i]) == float(ll_l[i])


def test_multinomial_ll_in_epilogue(cuda_lib):
    """The multinomial log-likelihood (optimal scaling over the unmasked
    entries, dadi/Inference.py:559-575, 668-685) from the same epilogue
    launch: against the oracle on the device spectra and against the torch
    form Batch2D.loglik(multinom=True); the Poisson ll of that launch is
    bitwise the one without it."""
    import torch
    from dadi_gb300 import batch, epilogue
    from oracle import numerics as onum
    import cases
    ns = (12, 12)
    eng = batch.Batch2D((30, 40, 50), ns)
    draws = cases.im_draws(5)
    phis, _ = eng.integrate(batch.im_instances(draws))
    fs0 = epilogue.spectra_2d_batch(torch, phis, eng.xxs, ns)[0].cpu().numpy()
    data = np.random.default_rng(3).poisson(2e3 * np.abs(fs0[0])).astype(np.float64)
    d_data = torch.from_numpy(data).cuda()
    fs_p, ll_p = epilogue.spectra_2d_batch(torch, phis, eng.xxs, ns, d_data, 2e3)
    fs_m, ll_m, llm = epilogue.spectra_2d_batch(torch, phis, eng.xxs, ns, d_data, 2e3,
                                                multinom=True)
    assert np.array_equal(fs_p.cpu().numpy(), fs_m.cpu().numpy())
    assert np.array_equal(ll_p.cpu().numpy(), ll_m.cpu().numpy())
    fs = fs_m.cpu().numpy()
    mask = onum.corner_mask(fs[0].shape)
    torch_llm = eng.loglik(fs_m, d_data, multinom=True).cpu().numpy()
    for i in range(len(draws)):
        ref = onum.ll_multinom(fs[i], data, mask)
        theta = np.sum(data[~mask]) / np.sum(fs[i][~mask])
        m = theta * fs[i][~mask & (fs[i] > 0)]
        d = data[~mask & (fs[i] > 0)]
        scale = np.sum(np.abs(m)) + np.sum(np.abs(d * np.log(m)))
        assert abs(float(llm[i]) - ref) <= 1e-12 * scale, (float(llm[i]), ref)
        assert abs(float(torch_llm[i]) - ref) <= 1e-12 * scale
    _, ll2, llm2 = eng.spectra_ll(phis, d_data, 2e3, multinom=True)
    assert np.array_equal(llm2.cpu().numpy(), llm.cpu().numpy())


@pytest.mark.parametrize("P,L,ns", [(1, 30, (12,)), (2, 25, (8, 11)), (3, 20, (6, 7, 9)),
                                    (3, 90, (20, 20, 20)), (4, 12, (4, 5, 3, 6)),
                                    (4, 40, (10, 10, 10, 10)), (5, 8, (3, 2, 4, 3, 2))])
def test_from_phi_nd_matches_reference_contraction(cuda_lib, P, L, ns):
    """The N-dimensional contraction kernel (dgb_from_phi_nd) on a batch of
    densities against the oracle's from_phi (1-4 populations) and the host
    5-D path (pinned to dadi's golden vectors), to REL."""
    import torch
    import cases
    from dadi_gb300 import spectrum
    from oracle import numerics as onum
    xx = cases.grid("default", L)
    phis = np.stack([cases.initial_phi(70 + b, (L,) * P) for b in range(3)])
    out = spectrum.from_phi_nd_batch(torch, torch.from_numpy(phis).cuda(), ns, xx)
    out = out.cpu().numpy()
    for b in range(3):
        if P <= 4:
            ref = onum.from_phi(phis[b], ns, xx)
        else:
            ref = spectrum._from_phi_5D(*ns, *(xx,) * 5, phis[b])
        _close(out[b], ref)
