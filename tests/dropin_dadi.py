"""dadi's own model code through the drop-in boundary, on the CPU.

Run by tests/test_dropin_dadi.py in a subprocess (it imports dadi, built from
the reference tree as tests/golden/make_golden.py builds it):

    python tests/dropin_dadi.py <reference tree> <scratch build dir>

`dadi_gb300.install()` registers the package as `dadi.cuda`, and
`dadi.cuda_enabled(True)` then sends dadi's Integration.one_pop .. five_pops
(and the constant-parameter paths with enable_cuda_cached=True) through the
drop-in drivers of dadi_gb300.cuda.Integration: argument order, the host
table build (parameters at the next time, dt from the current ones), masks,
Demes records.  Only the two calls that launch kernels --
integration.run_table and integration.run_precalc -- are replaced by shims
that execute the same table (or step lengths and a/b/c arrays) with the
oracle's C sweeps, so the comparison runs without a GPU: each model's result
must equal dadi with CUDA disabled bit for bit where both take the same
loop (temporal parameters, and enable_cuda_cached), and within 1e-9 where
dadi itself switches loops (constant parameters: dadi's CPU precalc path
against the temporal path dadi uses under CUDA).  Prints one JSON object.
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(HERE, "golden"))


def shims():
    """run_table / run_precalc executed on the CPU by the oracle."""
    from dadi_gb300 import integration as gi
    from oracle import clib, integration as oint

    def run_table(phi, xx, table, frozen_mask=0, nomut_mask=0):
        phi = np.array(phi, dtype=np.float64, copy=True)
        P = phi.ndim
        delj = gi.current_settings()[3]
        for row in table:
            dt, theta0 = row[0], row[1]
            active = [not (frozen_mask >> k & 1) and not (nomut_mask >> k & 1)
                      for k in range(P)]
            oint.inject_mutations(phi, dt, xx, theta0, active)
            for k in range(P):
                if frozen_mask >> k & 1:
                    continue
                mig = [0.0 if j == k else row[3 + 3 * P + k * (P - 1) + (j if j < k else j - 1)]
                       for j in range(P)]
                clib.sweep(phi, xx, k, row[2 + k], mig, row[2 + P + k], row[2 + 2 * P + k], dt,
                           beta=row[2 + 3 * P], use_delj_trick=delj)
        return phi

    def run_precalc(phi, xx, abc, dts, theta0, frozen_mask=0, nomut_mask=0):
        phi = np.array(phi, dtype=np.float64, copy=True)
        P = phi.ndim
        for dt in dts:
            active = [not (frozen_mask >> k & 1) and not (nomut_mask >> k & 1)
                      for k in range(P)]
            oint.inject_mutations(phi, dt, xx, theta0, active)
            for k in range(P):
                if not frozen_mask >> k & 1:
                    clib.sweep_precalc(phi, k, abc[3 * k], abc[3 * k + 1], abc[3 * k + 2], dt)
        return phi
    gi.run_table = run_table
    gi.run_precalc = run_precalc


def record(e):
    """A Demes cache record as plain data."""
    out = {"type": type(e).__name__}
    for k, v in sorted(vars(e).items()):
        out[k] = np.asarray(v, dtype=object).tolist() if isinstance(v, (list, tuple)) else v
    return out


def cases(dadi):
    """(name, function of no arguments returning an array, exact?)."""
    I, N, PM = dadi.Integration, dadi.Numerics, dadi.PhiManip
    D2 = dadi.Demographics2D

    def im():
        return N.make_extrap_func(D2.IM)((0.5, 2.0, 0.6, 0.05, 1.5, 0.7), (8, 8), [12, 14, 16])

    def split_mig():
        return N.make_extrap_func(D2.split_mig)((2.0, 0.5, 0.05, 1.0), (8, 8), [12, 14, 16])

    def two_cached():
        xx = N.default_grid(14)
        phi = PM.phi_1D_to_2D(xx, PM.phi_1D(xx))
        return I.two_pops(phi, xx, 0.05, 2.0, 0.5, m12=1.0, m21=0.3, gamma1=-1.0,
                          enable_cuda_cached=True)

    def three_temporal():
        xx = N.default_grid(10)
        phi = PM.phi_2D_to_3D_split_2(xx, PM.phi_1D_to_2D(xx, PM.phi_1D(xx)))
        return I.three_pops(phi, xx, 0.03, lambda t: 1.0 + 3 * t, 0.5, 2.0, m12=1.0, m21=0.5,
                            m23=0.3, m32=0.6, gamma3=1.5, deme_ids=["a", "b", "c"])

    def three_cached():
        xx = N.default_grid(10)
        phi = PM.phi_2D_to_3D_split_2(xx, PM.phi_1D_to_2D(xx, PM.phi_1D(xx)))
        return I.three_pops(phi, xx, 0.03, 1.2, 0.5, 2.0, m12=1.0, m21=0.5, m13=0.2, m31=0.4,
                            enable_cuda_cached=True)

    def four():
        xx = N.default_grid(7)
        phi = PM.phi_2D_to_3D_split_2(xx, PM.phi_1D_to_2D(xx, PM.phi_1D(xx)))
        phi = PM.phi_3D_to_4D(phi, 0.2, 0.3, xx, xx, xx, xx)
        return I.four_pops(phi.copy(), xx, 0.01, nu1=lambda t: 1.0 + 10 * t, nu2=0.5,
                           nu3=1.0, nu4=2.0, m14=0.5, m41=0.5, m23=1.0)

    def five():
        xx = N.default_grid(5)
        phi = PM.phi_2D_to_3D_split_2(xx, PM.phi_1D_to_2D(xx, PM.phi_1D(xx)))
        phi = PM.phi_3D_to_4D(phi, 0.2, 0.3, xx, xx, xx, xx)
        phi = PM.phi_4D_to_5D(phi, 0.1, 0.2, 0.3, xx, xx, xx, xx, xx)
        return I.five_pops(phi.copy(), xx, 0.005, nu1=lambda t: 1.0 + 10 * t, nu2=0.5,
                           m15=0.5, m51=0.5, gamma5=1.0)

    def one_temporal():
        xx = N.default_grid(30)
        return I.one_pop(PM.phi_1D(xx), xx, 0.1, nu=lambda t: 0.5 + 5 * t, gamma=-2.0,
                         h=0.3, beta=1.4)

    def one_const():
        xx = N.default_grid(30)
        return I.one_pop(PM.phi_1D(xx), xx, 0.1, nu=2.0, gamma=1.0)

    return [("im_extrap", im, True), ("split_mig_extrap", split_mig, False),
            ("two_pops_cuda_cached", two_cached, True), ("three_pops_temporal",
                                                         three_temporal, True),
            ("three_pops_cuda_cached", three_cached, True), ("four_pops", four, True),
            ("five_pops", five, True), ("one_pop_temporal", one_temporal, True),
            ("one_pop_const", one_const, False)]


def main(ref, build):
    import make_golden
    dadi = make_golden.load_dadi(ref, build)
    import dadi_gb300
    assert dadi_gb300.install(dadi) is dadi
    shims()
    calls = {"run": 0}
    from dadi_gb300 import integration as gi
    rt, rp = gi.run_table, gi.run_precalc

    def counted(f):
        def g(*a, **k):
            calls["run"] += 1
            return f(*a, **k)
        return g
    gi.run_table, gi.run_precalc = counted(rt), counted(rp)
    out = {"cases": {}}
    for name, fn, exact in cases(dadi):
        dadi.cuda_enabled(False)
        dadi.Demes.cache.clear()
        ref = np.asarray(fn())
        ref_rec = [record(e) for e in dadi.Demes.cache]
        assert dadi.cuda_enabled(True) is True
        dadi.Demes.cache.clear()
        before = calls["run"]
        got = np.asarray(fn())
        got_rec = [record(e) for e in dadi.Demes.cache]
        dadi.cuda_enabled(False)
        with np.errstate(all="ignore"):
            rel = np.abs(got - ref) / np.maximum(np.abs(ref), 1e-12 * np.abs(ref).max())
        out["cases"][name] = {
            "through_dropin": calls["run"] > before,
            "bitwise": bool(np.array_equal(got, ref)),
            "max_rel": float(np.max(rel)),
            "exact_expected": exact,
            "records_equal": (got_rec == ref_rec) if exact else
                             ([r["type"] for r in got_rec], [r["type"] for r in ref_rec]),
        }
    out["cuda_module"] = sys.modules["dadi.cuda"].__name__
    print(json.dumps(out))


if __name__ == "__main__":
    main(sys.argv[1], sys.argv[2])
