"""The launch-configuration autotuner of the batched engine: every candidate
computes bitwise the same densities, the tuner picks one of them and caches
the choice."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_candidates_agree_and_tuner_picks_one(cuda_lib):
    import cases
    from dadi_gb300 import autotune, batch
    eng = batch.Batch2D((30, 40, 50), (10, 10))
    rec = batch.im_instances(cases.im_draws(64))
    ref = None
    for mode, gam, threads in autotune.CANDIDATES:
        eng.launch_mode, eng.gam_placement, eng.threads = mode, gam, threads
        phis, st = eng.integrate(rec)
        assert int(st.abs().sum()) == 0
        out = [p.cpu().numpy() for p in phis]
        if ref is None:
            ref = out
        else:
            assert all(np.array_equal(a, b) for a, b in zip(out, ref)), (mode, gam, threads)
    res = autotune.tune_batch2d(eng, rec, sample_size=48)
    assert res["choice"] in res["ms"]
    assert (eng.launch_mode, eng.gam_placement, eng.threads) == res["choice"]
    assert len(res["ms"]) == len(autotune.CANDIDATES) and all(v > 0 for v in res["ms"].values())
    again = autotune.tune_batch2d(eng, rec, sample_size=48)
    assert again is res


def test_tuner_second_stage_on_a_larger_slice(cuda_lib):
    """For a batch much larger than the sample, the best candidate and the
    best per_grid candidate are timed again on a larger slice, which
    decides."""
    import cases
    from dadi_gb300 import autotune, batch
    eng = batch.Batch2D((30, 40, 50), (10, 10))
    rec = batch.im_instances(cases.im_draws(256))
    res = autotune.tune_batch2d(eng, rec, sample_size=32, large_size=96)
    assert res["large_sample"] == 96
    assert len(res["ms_large"]) in (0, 2)  # none when the sample's best is per_grid
    if res["ms_large"]:
        assert res["choice"] == min(res["ms_large"], key=res["ms_large"].get)
    assert (eng.launch_mode, eng.gam_placement, eng.threads) == res["choice"]


def test_threads_setting_is_checked(cuda_lib):
    """dgb_settings.threads accepts 0, 64, 96 and 128 (each where that many
    threads hold every line, else the automatic choice), all bitwise the
    same; other values are an argument error."""
    import cases
    from dadi_gb300 import _lib, batch
    eng = batch.Batch2D((30, 40), (10, 10))
    rec = batch.im_instances(cases.im_draws(8))
    ref = [p.cpu().numpy() for p in eng.integrate(rec)[0]]
    for t in (64, 96, 128):
        eng.threads = t
        out = [p.cpu().numpy() for p in eng.integrate(rec)[0]]
        assert all(np.array_equal(a, b) for a, b in zip(out, ref))
    eng.threads = 80
    with pytest.raises(_lib.DgbError):
        eng.integrate(rec)
