"""Generate the golden vectors in tests/golden/ by running the reference dadi.

Run once in a container that holds the reference tree (it cannot run on a GPU
host, which has no reference):

    python tests/golden/make_golden.py --ref <reference tree> [--build <scratch dir>]
                                       [--only im_scale]

The reference is copied to the build directory, its pyproject.toml moved aside
(its licence field trips the installed setuptools), its Cython extensions built
in place, and the off-path imports demes / ruamel / nlopt replaced by stub
modules before `import dadi`.  Every fixture is produced by dadi's own public
functions; the inputs live in cases.py or are stored next to the outputs.
"""
import argparse
import os
import shutil
import subprocess
import sys
import tempfile
import time
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import cases  # noqa: E402


def load_dadi(ref, build):
    if not os.path.exists(os.path.join(build, "dadi", "integration_c.c")) or not any(
            f.startswith("integration_c") and f.endswith(".so")
            for f in os.listdir(os.path.join(build, "dadi"))):
        if os.path.exists(build):
            shutil.rmtree(build)
        shutil.copytree(ref, build)
        subprocess.run(["chmod", "-R", "u+w", build], check=True)
        os.rename(os.path.join(build, "pyproject.toml"),
                  os.path.join(build, "pyproject.toml.bak"))
        subprocess.run([sys.executable, "setup.py", "build_ext", "--inplace"], cwd=build,
                       check=True, stdout=subprocess.DEVNULL)

    class _Stub(types.ModuleType):
        def __getattr__(self, name):
            if name.startswith("__"):
                raise AttributeError(name)
            return 0
    for n in ["demes", "ruamel", "ruamel.yaml", "nlopt"]:
        sys.modules.setdefault(n, _Stub(n))
    sys.path.insert(0, build)
    import dadi
    return dadi


def args_of(case):
    return [cases.resolve(a) for a in case["args"]], {
        k: cases.resolve(v) for k, v in case.get("kw", {}).items()}


def gen_integrations(dadi, out):
    for group, fn, nd in [("two", dadi.Integration.two_pops, 2),
                          ("three", dadi.Integration.three_pops, 3),
                          ("four", dadi.Integration.four_pops, 4),
                          ("five", dadi.Integration.five_pops, 5),
                          ("one", dadi.Integration.one_pop, 1)]:
        lst = {"two": cases.TWO_POPS, "three": cases.THREE_POPS,
               "four": cases.FOUR_POPS, "five": cases.FIVE_POPS,
               "one": cases.ONE_POP}[group]
        for case in lst:
            xx = cases.grid(case["grid"], case["pts"])
            phi0 = cases.initial_phi(case["seed"], (case["pts"],) * nd)
            a, kw = args_of(case)
            res = fn(phi0.copy(), xx, *a, **kw)
            out["int_" + case["name"]] = res
            out["int_" + case["name"] + "_phi0"] = phi0


def gen_sweeps(dadi, out):
    ic = dadi.integration_c
    p = cases.SWEEP_PARAMS
    rng = np.random.default_rng(77)
    rng5 = np.random.default_rng(78)  # the 5-D cases, added later, draw apart
    for name, nd, axis, pts, g in cases.SWEEPS:
        xx = cases.grid(g, pts)
        phi0 = (rng5 if nd == 5 else rng).uniform(size=(pts,) * nd)
        for delj in (0, 1):
            phi = phi0.copy()
            mig = [p["mig"][j] for j in range(nd) if j != axis]
            if nd == 1:
                ic.implicit_1Dx(phi, xx, p["nu"], p["gamma"], p["h"], p["beta"], p["dt"], delj)
            else:
                f = getattr(ic, "implicit_" + name)
                f(phi, *([xx] * nd), p["nu"], *mig, p["gamma"], p["h"], p["dt"], delj)
            out["sweep_%s_delj%d" % (name, delj)] = phi
        out["sweep_%s_phi0" % name] = phi0
    # constant-coefficient sweeps on random coefficient arrays
    for nd in (2, 3):
        pts = 9
        phi0 = rng.uniform(size=(pts,) * nd)
        for axis in range(nd):
            a = -rng.uniform(size=phi0.shape)
            c = -rng.uniform(size=phi0.shape)
            b = rng.uniform(2, 3, size=phi0.shape)
            phi = phi0.copy()
            f = getattr(ic, "implicit_precalc_%dD%s" % (nd, "xyz"[axis]))
            f(phi, a, b, c, 0.01)
            key = "precalc_%dD%d" % (nd, axis)
            out[key] = phi
            out[key + "_abc"] = np.stack([a, b, c])
            out[key + "_phi0"] = phi0


def gen_host(dadi, out):
    N = dadi.Numerics
    PM = dadi.PhiManip
    S = dadi.Spectrum
    for pts in (5, 10, 40, 80, 100, 120):
        out["grid_%d" % pts] = N.default_grid(pts)
    xx = N.default_grid(30)
    out["phi1d_snm"] = PM.phi_1D(xx)
    out["phi1d_g2"] = PM.phi_1D(xx, nu=1.5, theta0=2.0, gamma=2.0)
    out["phi1d_gm5"] = PM.phi_1D(xx, gamma=-5.0, beta=1.4)
    out["phi1d_h03"] = PM.phi_1D(xx, gamma=-3.0, h=0.3)
    phi2 = PM.phi_1D_to_2D(xx, PM.phi_1D(xx))
    out["phi2d_split"] = phi2
    xs = N.default_grid(12)
    phi3 = PM.phi_2D_to_3D_split_2(xs, PM.phi_1D_to_2D(xs, PM.phi_1D(xs)))
    out["phi3d_split2"] = phi3
    out["phi4d_from3d"] = PM.phi_3D_to_4D(phi3, 0.3, 0.2, xs, xs, xs, xs)
    x6 = N.default_grid(6)
    p4 = PM.phi_3D_to_4D(PM.phi_2D_to_3D_split_2(x6, PM.phi_1D_to_2D(x6, PM.phi_1D(x6))),
                         0.3, 0.2, x6, x6, x6, x6)
    out["phi5d_from4d"] = PM.phi_4D_to_5D(p4, 0.2, 0.3, 0.1, x6, x6, x6, x6, x6)
    rng = np.random.default_rng(5)
    rng5 = np.random.default_rng(6)  # the 5-D case, added later, draws apart
    for nd, pts, ns in [(1, 25, (12,)), (2, 21, (8, 11)), (3, 11, (5, 6, 4)),
                        (4, 7, (3, 4, 2, 3)), (5, 6, (2, 3, 2, 2, 3))]:
        xg = N.default_grid(pts)
        phi = (rng5 if nd == 5 else rng).uniform(size=(pts,) * nd)
        fs = S.from_phi(phi, ns, (xg,) * nd)
        out["fromphi_%dd" % nd] = np.asarray(fs.data)
        out["fromphi_%dd_phi" % nd] = phi
        out["fromphi_%dd_ns" % nd] = np.array(ns)
    # extrapolation and likelihoods
    ys = [rng.uniform(1, 2, size=(5, 5)) for _ in range(3)]
    xsl = [0.01, 0.008, 0.006]
    out["extrap_in"] = np.stack(ys)
    out["extrap_q"] = N.quadratic_extrap(ys, xsl)
    out["extrap_l"] = N.linear_extrap(ys[:2], xsl[:2])
    model = dadi.Spectrum(rng.uniform(0.1, 5, size=(6, 7)))
    data = dadi.Spectrum(rng.poisson(3 * np.asarray(model)).astype(float))
    out["ll_model"] = np.asarray(model.data)
    out["ll_data"] = np.asarray(data.data)
    out["ll"] = np.array(dadi.Inference.ll(model, data))
    out["ll_multinom"] = np.array(dadi.Inference.ll_multinom(model, data))
    a, b, c, r = rng.uniform(size=(4, 100))
    b = b + 2
    out["tridiag_abcr"] = np.stack([a, b, c, r])
    out["tridiag_u"] = dadi.tridiag_cython.tridiag(a, b, c, r)


def growth3(dadi):
    def model(params, ns, pts):
        (nu0, nuF, (m12, m13, m23), g, T) = params
        xx = dadi.Numerics.default_grid(pts)
        phi = dadi.PhiManip.phi_1D(xx)
        phi = dadi.PhiManip.phi_1D_to_2D(xx, phi)
        phi = dadi.PhiManip.phi_2D_to_3D_split_2(xx, phi)
        nus = [(lambda a, b: (lambda t: a * np.exp(np.log(b / a) * t / T)))(a, b)
               for a, b in zip(nu0, nuF)]
        phi = dadi.Integration.three_pops(phi, xx, T, nus[0], nus[1], nus[2],
                                          m12=m12, m13=m13, m21=m12, m23=m23,
                                          m31=m13, m32=m23,
                                          gamma1=g[0], gamma2=g[1], gamma3=g[2])
        return dadi.Spectrum.from_phi(phi, ns, (xx, xx, xx))
    return model


def gen_models(dadi, out, big):
    D2 = dadi.Demographics2D
    sm = cases.SPLIT_MIG
    f = dadi.Numerics.make_extrap_func(D2.split_mig)
    out["splitmig_fs"] = np.asarray(f(sm["params"], sm["ns"], sm["pts_l"]).data)
    for pts in sm["pts_l"]:
        out["splitmig_fs_%d" % pts] = np.asarray(D2.split_mig(sm["params"], sm["ns"], pts).data)
    fim = dadi.Numerics.make_extrap_func(D2.IM)
    draws = cases.im_draws()
    out["im_draws_head"] = draws[:64]
    out["im_small_fs"] = np.asarray(fim(draws[0], (10, 10), [20, 25, 30]).data)
    # IM spectra of a few seed-0 draws at the batched workload's grids
    sel = [0, 1, 2, 3, 5]
    for i in sel:
        t = time.time()
        out["im_fs_%d" % i] = np.asarray(fim(draws[i], (40, 40), [80, 90, 100]).data)
        print("IM draw %d: %.1fs" % (i, time.time() - t), flush=True)
    for pts in (80, 90, 100):
        out["im0_fs_%d" % pts] = np.asarray(D2.IM(draws[0], (40, 40), pts).data)
    if big:
        g = cases.GROWTH3
        t = time.time()
        f3 = dadi.Numerics.make_extrap_func(growth3(dadi))
        out["growth3_fs"] = np.asarray(f3(g["params"], g["ns"], g["pts_l"]).data)
        print("growth3: %.1fs" % (time.time() - t), flush=True)
    # observed data for the batched workload's likelihood: Poisson(5e4 * model(set 0))
    m0 = fim(draws[0], (40, 40), [80, 90, 100])
    obs = np.random.default_rng(0).poisson(5e4 * np.asarray(m0.data)).astype(float)
    out["im_obs"] = obs
    data = dadi.Spectrum(obs)
    out["im_ll"] = np.array([dadi.Inference.ll(5e4 * fim(draws[i], (40, 40), [80, 90, 100]),
                                               data) for i in sel])


_DADI = None


def _im_extrap(p):
    fim = _DADI.Numerics.make_extrap_func(_DADI.Demographics2D.IM)
    return np.asarray(fim(p, (40, 40), [80, 90, 100]).data)


def gen_im_scale(dadi, out, procs):
    """Dadi spectra of the batched workload (seed-0 IM draws, pts [80,90,100],
    ns (40,40)) for the cases.IM_SCALE_GOLDEN longest schedules of the
    stratified parity sample (cases.im_parity_sample), computed by worker
    processes forked from this one (dadi's C integrator is single-threaded)."""
    global _DADI
    import multiprocessing as mp
    sys.path.insert(0, os.path.join(HERE, "..", ".."))
    from oracle import clib
    clib.build()
    draws = cases.im_draws()
    steps = clib.im_steps(draws)
    idx = cases.im_parity_sample(draws, steps)
    gold = idx[np.argsort(-steps[idx], kind="stable")][:cases.IM_SCALE_GOLDEN]
    _DADI = dadi
    t = time.time()
    with mp.get_context("fork").Pool(procs) as pool:
        fs = pool.map(_im_extrap, [draws[i] for i in gold], chunksize=1)
    print("im_scale: %d spectra in %.1fs" % (len(gold), time.time() - t), flush=True)
    out["sample_idx"] = idx
    out["sample_steps"] = steps[idx]
    out["golden_idx"] = gold
    out["golden_params"] = draws[gold]
    out["golden_fs"] = np.stack(fs)


def gen_grad(dadi, out):
    fim = dadi.Numerics.make_extrap_func(dadi.Demographics2D.IM)
    draws = cases.im_draws()
    p0 = draws[0]
    data = dadi.Spectrum(np.random.default_rng(1).poisson(
        1e4 * np.asarray(fim(p0, (10, 10), [20, 25, 30]).data)).astype(float))
    func = lambda p: dadi.Inference.ll(1e4 * fim(p, (10, 10), [20, 25, 30]), data)
    out["grad_p0"] = p0
    out["grad_data"] = np.asarray(data.data)
    out["grad_godambe"] = np.asarray(dadi.Godambe.get_grad(func, p0, 1e-4)).ravel()


def gen_settings(dadi, out):
    """The IM pipeline and single two_pops / three_pops integrations under
    each non-default setting of dadi.Integration."""
    I = dadi.Integration
    d = cases.SETTINGS_IM
    f = dadi.Numerics.make_extrap_func(dadi.Demographics2D.IM)
    for name, kw in cases.SETTINGS:
        saved = {k: getattr(I, k) for k in kw}
        try:
            for k, v in kw.items():
                setattr(I, k, v)
            out["set_%s_im" % name] = np.asarray(f(d["params"], d["ns"], d["pts_l"]).data)
            xx = dadi.Numerics.default_grid(18)
            phi = dadi.PhiManip.phi_1D_to_2D(xx, dadi.PhiManip.phi_1D(xx))
            out["set_%s_2d" % name] = I.two_pops(phi, xx, 0.04, 2.0, lambda t: 0.5 + t,
                                                 1.0, 0.4, gamma1=-1.0, gamma2=2.0, h1=0.3)
            phi3 = dadi.PhiManip.phi_2D_to_3D_split_2(xx, phi)
            # a time-dependent size keeps three_pops on its temporal loop (its
            # constant-parameter path raises IndexError under the delj trick,
            # dadi/Integration.py:976)
            out["set_%s_3d" % name] = I.three_pops(phi3, xx, 0.02, lambda t: 1.0 + t, 0.5,
                                                   2.0, m12=1.0, m21=0.5, m23=0.3, m32=0.6,
                                                   gamma3=1.5)
        finally:
            for k, v in saved.items():
                setattr(I, k, v)


def gen_known_answers(dadi, ref, out):
    """The ms-simulated IM spectrum the reference's tests/test_Results.py:24-41
    compares against (tests/IM.fs of the reference), as data and mask."""
    ms = dadi.Spectrum.from_file(os.path.join(ref, "tests", "IM.fs"))
    out["im_ms_data"] = np.asarray(ms.data)
    out["im_ms_mask"] = np.ma.getmaskarray(ms)


def gen_dfe(dadi, out):
    from dadi.DFE import Cache2D_mod, DemogSelModels, PDFs
    d = cases.DFE
    c = Cache2D_mod.Cache2D(d["params"], d["ns"], DemogSelModels.IM_sel, d["pts"],
                            gamma_pts=d["gamma_pts"], cpus=1)
    out["dfe_gammas"] = c.gammas
    out["dfe_spectra"] = np.asarray(c.spectra)
    fs = c.integrate(d["sel_params"], None, PDFs.biv_lognormal, d["theta"], None)
    out["dfe_fs"] = np.asarray(fs.data)
    fs = c.integrate(d["sel_params"], None, PDFs.biv_lognormal, d["theta"], None,
                     exterior_int=False)
    out["dfe_fs_interior"] = np.asarray(fs.data)
    x = np.array([0.5, 3.0, 40.0])
    out["dfe_pdf"] = PDFs.biv_lognormal(x, x, np.array(d["sel_params"]))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", required=True, help="the reference dadi source tree")
    ap.add_argument("--build", default=os.path.join(tempfile.gettempdir(), "dadi_ref"),
                    help="scratch directory for the reference build")
    ap.add_argument("--no-big", action="store_true", help="skip the 3-D model (~1 min)")
    ap.add_argument("--only", choices=["im_scale"], default=None,
                    help="write only this fixture")
    ap.add_argument("--procs", type=int, default=os.cpu_count() or 1)
    a = ap.parse_args()
    dadi = load_dadi(a.ref, a.build)
    if a.only == "im_scale":
        out = {}
        gen_im_scale(dadi, out, a.procs)
        np.savez_compressed(os.path.join(HERE, "im_scale.npz"), **out)
        print("wrote im_scale", len(out))
        return
    for name, gen in [("integrate", gen_integrations), ("sweeps", gen_sweeps),
                      ("host", gen_host), ("grad", gen_grad), ("dfe", gen_dfe),
                      ("settings", gen_settings)]:
        out = {}
        gen(dadi, out)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
        print("wrote", name, len(out), flush=True)
    out = {}
    gen_known_answers(dadi, a.ref, out)
    np.savez_compressed(os.path.join(HERE, "known.npz"), **out)
    print("wrote known", len(out))
    out = {}
    gen_models(dadi, out, not a.no_big)
    np.savez_compressed(os.path.join(HERE, "models.npz"), **out)
    print("wrote models", len(out))


if __name__ == "__main__":
    main()
