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
    for mode, gam in autotune.CANDIDATES:
        eng.launch_mode, eng.gam_placement = mode, gam
        phis, st = eng.integrate(rec)
        assert int(st.abs().sum()) == 0
        out = [p.cpu().numpy() for p in phis]
        if ref is None:
            ref = out
        else:
            assert all(np.array_equal(a, b) for a, b in zip(out, ref)), (mode, gam)
    res = autotune.tune_batch2d(eng, rec, sample_size=48)
    assert res["choice"] in res["ms"] and (eng.launch_mode, eng.gam_placement) == res["choice"]
    assert len(res["ms"]) == len(autotune.CANDIDATES) and all(v > 0 for v in res["ms"].values())
    again = autotune.tune_batch2d(eng, rec, sample_size=48)
    assert again is res
