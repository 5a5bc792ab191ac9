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
from util import assert_fs_parity, fs_parity

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
    for k, i in enumerate(idx):
        assert_fs_parity(fs[k], ref[i])
        worst = max(worst, fs_parity(fs[k], ref[i])[0])
        ll_ref = onum.ll(5e4 * ref[i], obs, mask)
        assert abs(ll[k] - ll_ref) <= 1e-9 * abs(ll_ref), (i, ll[k], ll_ref)
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


def _fd_rich(eng, p, data, scale, eps=1e-4):
    """Central differences at eps and eps/2 (relative steps) in one batch,
    and their Richardson combination."""
    rows = []
    for e in (eps, eps / 2):
        for k in range(6):
            for sgn in (1, -1):
                q = p.copy()
                q[k] += sgn * e * p[k]
                rows.append(q)
    _, ll, st = eng.run(np.array(rows), data=data, scale=scale)
    assert int(st.abs().sum()) == 0
    ll = ll.cpu().numpy().reshape(2, 6, 2)
    d = [(ll[j, :, 0] - ll[j, :, 1]) / (2 * e * p) for j, e in enumerate((eps, eps / 2))]
    return d[0], (4 * d[1] - d[0]) / 3


@pytest.mark.parametrize("which", [0, 1])
def test_adjoint_at_config4_grids_matches_fd(cuda_lib, golden, which):
    """Config 4: gradients of the Poisson likelihood at pts [100,110,120],
    ns (40,40) for seed-0 draws among the first 256, against Richardson
    central differences, 1e-6 max-norm relative."""
    from dadi_gb300 import batch
    draws = cases.im_draws()
    steps = batch.count_steps(batch.im_instances(draws[:256]))
    cand = [i for i in range(256) if 150 <= steps[i] <= 900]
    i = cand[which * 3]
    obs = golden["models"]["im_obs"]
    eng = batch.Batch2D((100, 110, 120), NS)
    ll, grad, st = eng.loglik_and_grad(draws[i][None, :], obs, scale=5e4)
    assert int(st.abs().sum()) == 0
    adj = grad.cpu().numpy()[0]
    fd, rich = _fd_rich(eng, draws[i].copy(), obs, 5e4)
    err = float(np.max(np.abs(adj - rich)) / np.max(np.abs(rich)))
    assert err < 1e-6, (i, adj, rich, err)
