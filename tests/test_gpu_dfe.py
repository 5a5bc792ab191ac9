"""DFE cache generation on the batched engine (dadi.DFE.Cache2D with
DemogSelModels.IM_sel, dadi/DFE/Cache2D_mod.py:13-207) against the cache
dadi itself generated: every cached spectrum within the spectrum bar, and the
integrated spectrum over a bivariate lognormal."""
import numpy as np
import pytest

from util import assert_fs_parity

pytestmark = pytest.mark.gpu


def test_cache2d_matches_reference(cuda_lib, golden):
    import cases
    from dadi_gb300 import dfe, models
    d = cases.DFE
    g = golden["dfe"]
    c = dfe.Cache2D(d["params"], d["ns"], models.IM_sel, d["pts"], gamma_pts=d["gamma_pts"])
    assert np.array_equal(c.gammas, g["dfe_gammas"])
    G = len(c.gammas)
    for ii in range(G):
        for jj in range(G):
            assert_fs_parity(c.spectra[ii, jj], g["dfe_spectra"][ii, jj])
    fs = c.integrate(d["sel_params"], None, dfe.biv_lognormal, d["theta"], None)
    assert_fs_parity(np.asarray(fs.data), g["dfe_fs"])


def test_cache2d_split_jobs_merge(cuda_lib):
    """split_jobs / merge give the single-job cache."""
    import cases
    from dadi_gb300 import dfe, models
    d = cases.DFE
    full = dfe.Cache2D(d["params"], d["ns"], models.IM_sel, d["pts"], gamma_pts=2)
    parts = [dfe.Cache2D(d["params"], d["ns"], models.IM_sel, d["pts"], gamma_pts=2,
                         split_jobs=3, this_job_id=k) for k in range(3)]
    merged = dfe.Cache2D.merge(parts)
    assert np.array_equal(merged.spectra, full.spectra)
