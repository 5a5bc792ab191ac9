"""The serving loop: a mixed request stream (2-D IM at assorted grid and
sample sizes, DFE-style IM with selection, 3-D growth, four populations,
gradient requests) arriving over time is served with continuous batching;
every result equals the same request served alone -- bitwise for 3-D / 4-D
spectra and gradients (the same kernels on the same data, only the
neighbours differ), to 1e-10 relative for 2-D spectra (a small wave runs
each work item on a cluster of CTAs, a large one on one CTA: the same
equations solved in another order, whose last-bit differences accumulate
over up to 19,546 steps and grow through the extrapolation: measured up to
2.2e-11) -- the 2-D results match the oracle
(the reference's algorithm on the CPU) and the 3-D / 4-D ones the
one-at-a-time drop-in, within the spectrum bar."""
import copy
import multiprocessing as mp
import os

import numpy as np
import pytest

from util import assert_fs_parity

pytestmark = pytest.mark.gpu


def _obs():
    from dadi_gb300 import batch
    import cases
    eng = batch.Batch2D((80, 90, 100), (40, 40))
    fs0, _, _ = eng.run(cases.im_draws(1))
    return np.random.default_rng(0).poisson(5e4 * fs0.cpu().numpy()[0]).astype(np.float64)


def _oracle_fs(args):
    kind, params, ns, pts_l = args
    from oracle import numerics as onum
    model = {"im": onum.IM, "im_sel": onum.IM_sel}[kind]
    return np.asarray(onum.extrap_model(model, params, ns, list(pts_l)))


def test_serving_mix_equals_alone_and_reference(cuda_lib):
    from dadi_gb300 import models, numerics, serving
    obs = _obs()
    reqs = serving.config5_stream(40, seed=3, rate=2000.0, grad_frac=0.3, obs=obs)
    kinds = {r.kind for r in reqs}
    assert {"im", "im_sel"} <= kinds
    srv = serving.Server(hbm_budget=8 << 30, max_wave=16)
    mix = srv.run([copy.copy(r) for r in reqs])
    assert all(r.error is None and r.status == 0 and r.t_done is not None for r in mix), \
        [(r.rid, r.error) for r in mix if r.error]
    summ = serving.latency_summary(mix)
    assert summ["completed"] == len(reqs) and summ["p99_s"] >= summ["p50_s"] > 0
    by_id = {r.rid: r for r in mix}
    # each request alone, through a fresh server
    for r in reqs[:12]:
        alone = serving.Server(hbm_budget=8 << 30).run([copy.copy(r)])[0]
        if r.kind in ("im", "im_sel"):
            a, b = alone.fs, by_id[r.rid].fs
            rel = np.abs(a - b) / np.maximum(np.abs(b), 1e-12 * np.abs(b).max())
            assert float(rel.max()) <= 1e-10, (r.kind, float(rel.max()))
        else:
            assert np.array_equal(alone.fs, by_id[r.rid].fs), r.kind
        if r.want_grad:
            assert np.array_equal(alone.grad, by_id[r.rid].grad)
    # 2-D results against the oracle (a spawn pool: this process uses CUDA)
    two = [r for r in mix[:12] if r.kind in ("im", "im_sel")]
    assert len(two) == 12
    with mp.get_context("spawn").Pool(os.cpu_count() or 1) as pool:
        refs = pool.map(_oracle_fs, [(r.kind, r.params, r.ns, r.pts_l) for r in two],
                        chunksize=1)
    for r, ref in zip(two, refs):
        assert_fs_parity(r.fs, ref)
    # 3-D and 4-D results against the one-at-a-time drop-in
    fns = {"growth3": models.growth3, "four": models.four_split}
    for r in mix:
        if r.kind in fns:
            ref = numerics.make_extrap_func(fns[r.kind])(r.params, r.ns, list(r.pts_l))
            assert_fs_parity(r.fs, np.asarray(ref.data))


def test_serving_admits_by_footprint(cuda_lib):
    """With a budget that holds only a few requests at a time, everything is
    still served and the budget is never exceeded at admission."""
    from dadi_gb300 import serving
    reqs = [r for r in serving.config5_stream(30, seed=5) if r.kind in ("im", "im_sel")][:10]
    srv = serving.Server(hbm_budget=1, max_wave=4)  # admits one request at a time
    out = srv.run(reqs)
    assert all(r.t_done is not None and r.error is None for r in out)
    assert srv._used == 0
