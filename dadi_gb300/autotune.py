"""Autotuner of the batched 2-D engine's launch configuration.

The knobs, each a real alternative the kernels implement:

* launch mode — "persistent": a device-sized grid whose CTAs pull (instance,
  grid) work items from an atomic queue, longest first; "one_per_cta": one
  CTA per work item, each retiring after its item (what lets concurrent
  launches share SMs);
* ... or "per_grid": one persistent launch per grid size, each shaped for
  its own L (CTAs per SM, three or four warps per CTA), on side streams so
  that one launch's tail overlaps the next;
* gam placement — the Thomas recurrence's scratch in shared memory (fewer
  CTAs per SM when the density already fills it) or in a per-CTA slice of
  the workspace (more CTAs per SM, L2 traffic on the back substitution).

`tune_batch2d` times every candidate on a sample of the batch — instances
spread over the batch's cost distribution, so the sample has the batch's mix
of long and short integrations — with CUDA events, keeps the fastest on the
engine, and caches the choice per (device, grids, sample size).  Every
candidate computes bitwise the same densities (tested): only the launch
differs.
"""
import numpy as np

from . import _lib, batch

CANDIDATES = [("persistent", 1), ("persistent", 2), ("one_per_cta", 1), ("one_per_cta", 2),
              ("per_grid", 1), ("per_grid", 2)]

_cache = {}


def _sample(rec, size, settings=None):
    """`size` instances evenly spaced over the 5-85 % quantiles of the step
    counts: the batch's mix, without the longest integrations whose serial
    time would set a small sample's duration (the full batch hides them
    behind the rest of the work)."""
    if size >= len(rec):
        return rec
    steps = batch.count_steps(rec, settings)
    order = np.argsort(steps, kind="stable")
    lo, hi = int(0.05 * (len(rec) - 1)), int(0.85 * (len(rec) - 1))
    pick = order[np.linspace(lo, hi, size).round().astype(int)]
    return rec[np.sort(pick)]


def tune_batch2d(eng, rec, sample_size=None, repeats=1, candidates=None):
    """Time the candidates on a sample of `rec` (dgb_inst2d records) with
    engine `eng` (a batch.Batch2D), set the fastest on the engine and return
    {"choice": (mode, gam), "ms": {candidate: ms}}."""
    torch = eng.torch
    props = torch.cuda.get_device_properties(torch.cuda.current_device())
    size = sample_size or 4 * props.multi_processor_count
    key = (props.name, tuple(eng.pts_l), int(size))
    if key in _cache:
        eng.launch_mode, eng.gam_placement = _cache[key]["choice"]
        return _cache[key]
    sample = _sample(np.ascontiguousarray(rec), size)
    times = {}
    saved = (eng.launch_mode, eng.gam_placement)
    for mode, gam in (candidates or CANDIDATES):
        eng.launch_mode, eng.gam_placement = mode, gam
        try:
            eng.integrate(sample)  # warm-up
        except _lib.DgbError as e:
            if e.status == _lib.DGB_ERR_UNSUPPORTED:  # gam does not fit shared memory
                continue
            raise
        best = None
        for _ in range(repeats):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            eng.integrate(sample, timer=(e0, e1))
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1)
            best = ms if best is None else min(best, ms)
        times[(mode, gam)] = best
    if not times:
        eng.launch_mode, eng.gam_placement = saved
        raise RuntimeError("no launch configuration applies")
    choice = min(times, key=times.get)
    eng.launch_mode, eng.gam_placement = choice
    _cache[key] = {"choice": choice, "ms": times, "sample": int(len(sample))}
    return _cache[key]
