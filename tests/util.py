"""Helpers shared by the tests."""
import numpy as np

import cases


def max_rel(a, b, floor=0.0):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    den = np.maximum(np.abs(b), floor)
    with np.errstate(all="ignore"):
        r = np.abs(a - b) / den
    r[(a == b)] = 0
    return float(np.max(r)) if r.size else 0.0


def case_inputs(group, case):
    nd = {"one": 1, "two": 2, "three": 3, "four": 4, "five": 5}[group]
    xx = cases.grid(case["grid"], case["pts"])
    phi0 = cases.initial_phi(case["seed"], (case["pts"],) * nd)
    args = [cases.resolve(v) for v in case["args"]]
    kw = {k: cases.resolve(v) for k, v in case.get("kw", {}).items()}
    return xx, phi0, args, kw


GROUPS = [("one", cases.ONE_POP), ("two", cases.TWO_POPS), ("three", cases.THREE_POPS),
          ("four", cases.FOUR_POPS), ("five", cases.FIVE_POPS)]
ALL_CASES = [(g, c) for g, lst in GROUPS for c in lst]


#: Spectrum parity bar: entries at or above TINY_FRAC of the largest entry
#: must agree to FS_REL relative error; smaller entries (which arise from
#: cancellation and carry no likelihood weight) must agree to
#: FS_REL * TINY_FRAC * max|ref| absolutely.  The level is the reference's
#: own: over the stratified 64-instance sample of the batched workload,
#: dadi's arithmetic with the right-hand side rounded as its own
#: constant-parameter sweeps round it moves entries at or above 1e-9 of the
#: maximum by at most 7.9e-10 relative, and smaller ones by up to 1.5e-8
#: relative but at most 6.1e-19 of the maximum absolutely
#: (test_oracle.py::test_reference_noise_floor_at_scale), so a relative bar
#: below that level would test rounding, not correctness.
FS_REL = 1e-9
TINY_FRAC = 1e-9


def fs_parity(fs, ref):
    """(max relative error over entries >= TINY_FRAC*max, max absolute error
    over smaller entries divided by max|ref|, number of small entries), with
    the masked corners excluded."""
    fs = np.asarray(fs, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    m = np.zeros(ref.shape, dtype=bool)
    m.flat[0] = m.flat[-1] = True
    mx = np.max(np.abs(ref[~m]))
    big = (np.abs(ref) >= TINY_FRAC * mx) & ~m
    small = ~big & ~m
    with np.errstate(all="ignore"):
        rel = np.abs(fs - ref) / np.abs(ref)
    rel_big = float(np.max(rel[big])) if big.any() else 0.0
    abs_small = float(np.max(np.abs(fs - ref)[small]) / mx) if small.any() else 0.0
    return rel_big, abs_small, int(small.sum())


def assert_fs_parity(fs, ref):
    rel_big, abs_small, n_small = fs_parity(fs, ref)
    assert rel_big <= FS_REL, (rel_big, n_small)
    assert abs_small <= FS_REL * TINY_FRAC, (abs_small, n_small)


def table_rows(P, nsteps, seed):
    """A parameter table of nsteps rows for P populations: varying sizes,
    migration, selection and dominance (row layout of build_table)."""
    from dadi_gb300 import integration as gi
    rng = np.random.default_rng(seed)
    tab = np.empty((nsteps, gi.row_stride(P)))
    tab[:, 0] = rng.uniform(2e-4, 1e-3, nsteps)          # dt
    tab[:, 1] = rng.uniform(0.5, 2.0, nsteps)            # theta0
    tab[:, 2:2 + P] = rng.uniform(0.2, 5.0, (nsteps, P))  # nu
    tab[:, 2 + P:2 + 2 * P] = rng.uniform(-5, 5, (nsteps, P))  # gamma
    tab[:, 2 + 2 * P:2 + 3 * P] = rng.uniform(0.1, 0.9, (nsteps, P))  # h
    tab[:, 2 + 3 * P] = 1.0 if P > 1 else rng.uniform(0.5, 2.0, nsteps)  # beta
    tab[:, 3 + 3 * P:] = rng.uniform(0, 3, (nsteps, P * (P - 1)))  # migration
    return tab

