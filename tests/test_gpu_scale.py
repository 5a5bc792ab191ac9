"""Parity at the scale of the batched workload (4096 seed-0 IM draws at pts
[80,90,100], ns (40,40), extrapolated, Poisson likelihood against
Poisson(5e4 * model(set 0))).

The batched engine, in the launch configuration the benchmark uses, runs a
stratified 64-instance sample of the workload (tests/golden/cases.py
im_parity_sample: draws 0-5, the longest schedule of 19,546 steps and the
shortest, the smallest and largest value of every parameter -- nu near 0.01
and 100, T near 2, m near 10 -- and step-count quantiles).  Every spectrum is
held to the spectrum bar and every likelihood to 1e-9 relative against:

* dadi itself for the 16 longest schedules (golden vectors made by
  tests/golden/make_golden.py --only im_scale), and
* the oracle for the other 48 (bit-identical to dadi on every golden
  vector, tests/test_oracle.py), computed here in a spawn pool.

The adjoint is also checked at config 4's grids (pts [100,110,120], ns
(40,40)) against Richardson central differences of the same forward.
"""
import multiprocessing as mp
import os

import numpy as np
import pytest

import cases
from util import FS_REL, TINY_FRAC, fs_parity

pytestmark = pytest.mark.gpu

PTS_L = (80, 90, 100)
NS = (40, 40)


def _oracle_fs(p):
    from oracle import numerics as onum
    return np.asarray(onum.extrap_model(onum.IM, p, NS, list(PTS_L)))


@pytest.fixture(scope="module")
def scale_golden():
    d = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "im_scale.npz")
    return np.load(d)


@pytest.fixture(scope="module")
def oracle_spectra(scale_golden):
    """The oracle's spectra of the sample instances without a dadi golden,
    by instance index (a spawn pool: the test process already uses CUDA)."""
    draws = cases.im_draws()
    gold = set(int(i) for i in scale_golden["golden_idx"])
    rest = [int(i) for i in scale_golden["sample_idx"] if int(i) not in gold]
    with mp.get_context("spawn").Pool(os.cpu_count() or 1) as pool:
        fs = pool.map(_oracle_fs, [draws[i] for i in rest], chunksize=1)
    return dict(zip(rest, fs))


def test_batched_workload_sample_matches_dadi_and_oracle(cuda_lib, golden, scale_golden,
                                                         oracle_spectra):
    from oracle import numerics as onum
    from dadi_gb300 import batch
    draws = cases.im_draws()
    idx = [int(i) for i in scale_golden["sample_idx"]]
    obs = golden["models"]["im_obs"]
    eng = batch.Batch2D(PTS_L, NS)
    eng.launch_mode = "per_grid"  # the benchmark's tuned configuration
    fs, ll, status = eng.run(draws[idx], data=obs, scale=5e4)
    assert int(status.abs().sum()) == 0
    fs = fs.cpu().numpy()
    ll = ll.cpu().numpy()
    ref = dict(oracle_spectra)
    for k, i in enumerate(scale_golden["golden_idx"]):
        ref[int(i)] = scale_golden["golden_fs"][k]
    worst = 0.0
    mask = onum.corner_mask(fs.shape[1:])
    bad = []
    for k, i in enumerate(idx):
        rel, ab, _ = fs_parity(fs[k], ref[i])
        worst = max(worst, rel)
        if rel > FS_REL or ab > FS_REL * TINY_FRAC:
            bad.append((i, rel, ab))
        ll_ref = onum.ll(5e4 * ref[i], obs, mask)
        assert abs(ll[k] - ll_ref) <= 1e-9 * abs(ll_ref), (i, ll[k], ll_ref)
    assert not bad, bad
    print("max rel over %d instances: %.3g" % (len(idx), worst))


def test_batched_default_launch_equals_tuned(cuda_lib, scale_golden):
    """The persistent single-launch configuration gives the tuned per-grid
    launch's spectra bit for bit on the sample's longest instances."""
    from dadi_gb300 import batch
    draws = cases.im_draws()
    sel = [int(i) for i in scale_golden["golden_idx"][:6]]
    a = batch.Batch2D(PTS_L, NS)
    a.launch_mode = "per_grid"
    b = batch.Batch2D(PTS_L, NS)
    b.launch_mode = "persistent"
    fa = a.run(draws[sel])[0].cpu().numpy()
    fb = b.run(draws[sel])[0].cpu().numpy()
    assert np.array_equal(fa, fb)


#: Relative step of the config-4 finite differences (and half of it for the
#: Richardson combination).  At these grids both ends of the usual range
#: fail: the extrapolated likelihood carries rounding noise of about 1e-12
#: of itself that varies from one parameter set to the next, so steps below
#: ~3e-6 measure noise (oracle central differences in T on draw 14: D(1e-5)
#: = 318006.32, D(3e-6) = .29, D(1e-6) = .56, D(3e-7) = .03, D(1e-7) =
#: 318003.37), while steps of 1e-4 reach into the structure the likelihood has
#: on the scale of 1e-5 in T (draw 15: D(1e-4) = -460208, D(1e-5) = -460301,
#: D(1e-6) = -460282.6).  1e-5 and 5e-6 sit between the two.
FD_EPS = 1e-5


def _stencil(p, eps=FD_EPS):
    """The parameter sets of central differences at eps and eps/2 (relative
    steps), in the order _fd_rich reads them."""
    rows = []
    for e in (eps, eps / 2):
        for k in range(6):
            for sgn in (1, -1):
                q = p.copy()
                q[k] += sgn * e * p[k]
                rows.append(q)
    return np.array(rows)


def _fd_rich(eng, p, data, scale, eps=FD_EPS):
    """Central differences at eps and eps/2 in one batch, and their
    Richardson combination."""
    _, ll, st = eng.run(_stencil(p, eps), data=data, scale=scale)
    assert int(st.abs().sum()) == 0
    ll = ll.cpu().numpy().reshape(2, 6, 2)
    d = [(ll[j, :, 0] - ll[j, :, 1]) / (2 * e * p) for j, e in enumerate((eps, eps / 2))]
    return d[0], (4 * d[1] - d[0]) / 3


def _branches(p, tsf=1e-3):
    """Which term binds the timestep at each step of an IM schedule
    (dadi/Integration.py:147-176, 346-386): population (the min over the
    two) and 0.25/nu or the migration rate (the max), and whether the step
    was cut to T - t."""
    s, nu1, nu2, T, m12, m21 = p
    f = [lambda t: s * (nu1 / s) ** (t / T), lambda t: (1 - s) * (nu2 / (1 - s)) ** (t / T)]
    m = [m12, m21]
    t, out = 0.0, []
    nu = [f[0](t), f[1](t)]
    while t < T:
        d = [tsf / max(0.25 / nu[k], m[k]) for k in range(2)]
        k = 1 if d[1] < d[0] else 0
        term = 0 if 0.25 / nu[k] >= m[k] else 1
        dt = d[k]
        cut = T - t < dt
        out.append((k, term, cut))
        t = t + min(dt, T - t)
        nu = [f[0](t), f[1](t)]
    return out


def _smooth_candidates(draws, want=2, lo=150, hi=900):
    """Draws among the first 256 whose finite-difference stencil stays on one
    smooth piece of the discrete likelihood.  The schedule is built from
    max/min choices (dt = 1e-3 / max(0.25 / nu, m), the smaller of the two
    populations' dt, the last step cut to T - t): where a stencil point takes
    another number of steps or another branch at some step, the likelihood
    has a kink between the points and a central difference measures the
    kink, not the derivative the adjoint gives.  With m12 near 5 and T near
    0.5 such kinks are only 4e-4 apart in relative m12.  (The stencil is
    checked at 1e-4 so that it is safely inside one piece.)"""
    from dadi_gb300 import batch
    steps = batch.count_steps(batch.im_instances(draws[:256]))
    out = []
    for i in range(256):
        if not lo <= steps[i] <= hi:
            continue
        base = _branches(draws[i])
        if all(_branches(q) == base for q in _stencil(draws[i].copy(), 1e-4)):
            out.append(i)
            if len(out) == want:
                break
    return out


@pytest.mark.parametrize("which", [0, 1])
def test_adjoint_at_config4_grids_matches_fd(cuda_lib, golden, which):
    """Config 4: gradients of the Poisson likelihood at pts [100,110,120],
    ns (40,40) for seed-0 draws among the first 256, against Richardson
    central differences on a smooth piece, 1e-6 max-norm relative."""
    from dadi_gb300 import batch
    draws = cases.im_draws()
    i = _smooth_candidates(draws)[which]
    obs = golden["models"]["im_obs"]
    eng = batch.Batch2D((100, 110, 120), NS)
    ll, grad, st = eng.loglik_and_grad(draws[i][None, :], obs, scale=5e4)
    assert int(st.abs().sum()) == 0
    adj = grad.cpu().numpy()[0]
    fd, rich = _fd_rich(eng, draws[i].copy(), obs, 5e4)
    err = float(np.max(np.abs(adj - rich)) / np.max(np.abs(rich)))
    assert err < 1e-6, (i, adj, rich, err)
