"""Autotuners: the batched 2-D engine's launch configuration, and the line
solver of a lone 3-5 population integration.

The knobs, each a real alternative the kernels implement:

* launch mode — "persistent": a device-sized grid whose CTAs pull (instance,
  grid) work items from an atomic queue, longest first; "one_per_cta": one
  CTA per work item, each retiring after its item (what lets concurrent
  launches share SMs);
* ... or "per_grid": one persistent launch per grid size, each shaped for
  its own L (CTAs per SM, warps per CTA, two work items per CTA for a grid
  of 73-128 points where that fills the lanes better), on side streams so
  that one launch's tail overlaps the
  next;
* gam placement — the Thomas recurrence's scratch in shared memory (fewer
  CTAs per SM when the density already fills it) or in a per-CTA slice of
  the workspace (more CTAs per SM, L2 traffic on the back substitution);
* threads per CTA — 0 lets the engine choose the fewest warps that hold
  every line of the launch's largest grid (fuller warps: the FP64 pipe
  charges a warp instruction whatever its active lanes), so per_grid runs
  grids of up to 96 points on three warps; 128 forces four warps, the check
  on that rule.

`tune_batch2d` times every candidate on a sample of the batch — instances
spread over the batch's cost distribution, so the sample has the batch's mix
of long and short integrations — with CUDA events.  A small sample
overstates the tails of launches that run one after another (per_grid's
three launches each end on their longest item), so for a batch much larger
than the sample the best candidate and the best per_grid candidate are timed
again on a larger slice, which decides.  The choice is kept on the engine
and cached per (device, grids, batch size class).  Every candidate computes
bitwise the same densities (tested): only the launch differs.
"""
import numpy as np

from . import _lib, batch

CANDIDATES = [("persistent", 1, 0), ("persistent", 2, 0), ("one_per_cta", 1, 0),
              ("one_per_cta", 2, 0), ("per_grid", 1, 0), ("per_grid", 2, 0),
              ("per_grid", 2, 128)]

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


def _apply(eng, cand):
    eng.launch_mode, eng.gam_placement, eng.threads = cand


def _time(eng, rec, cand, warm=True):
    """ms of one integration of rec under candidate cand (None: it does not
    apply, e.g. gam does not fit shared memory)."""
    torch = eng.torch
    _apply(eng, cand)
    try:
        if warm:
            eng.integrate(rec[:min(len(rec), 64)])
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        eng.integrate(rec, timer=(e0, e1))
        torch.cuda.synchronize()
    except _lib.DgbError as e:
        if e.status == _lib.DGB_ERR_UNSUPPORTED:
            return None
        raise
    return e0.elapsed_time(e1)


def tune_batch2d(eng, rec, sample_size=None, candidates=None, large_size=2048):
    """Time the candidates on a sample of `rec` (dgb_inst2d records) with
    engine `eng` (a batch.Batch2D), set the fastest on the engine and return
    {"choice": (mode, gam, threads), "ms": {candidate: ms}, "ms_large":
    {finalist: ms} (empty when the batch is not much larger than the
    sample), "sample": n, "large_sample": n}."""
    torch = eng.torch
    props = torch.cuda.get_device_properties(torch.cuda.current_device())
    size = sample_size or 4 * props.multi_processor_count
    big = min(large_size, len(rec) // 2) if len(rec) >= 4 * size else 0
    key = (props.name, tuple(eng.pts_l), int(size), int(big))
    if key in _cache:
        _apply(eng, _cache[key]["choice"])
        return _cache[key]
    saved = (eng.launch_mode, eng.gam_placement, eng.threads)
    rec = np.ascontiguousarray(rec)
    sample = _sample(rec, size)
    times = {}
    for cand in (candidates or CANDIDATES):
        ms = _time(eng, sample, cand)
        if ms is not None:
            times[cand] = ms
    if not times:
        _apply(eng, saved)
        raise RuntimeError("no launch configuration applies")
    choice = min(times, key=times.get)
    large = {}
    if big:
        finalists = {choice}
        per_grid = [c for c in times if c[0] == "per_grid"]
        if per_grid:
            finalists.add(min(per_grid, key=times.get))
        if len(finalists) > 1:
            slice_ = _sample(rec, big)
            for cand in sorted(finalists):
                large[cand] = _time(eng, slice_, cand, warm=False)
            choice = min(large, key=large.get)
    _apply(eng, choice)
    _cache[key] = {"choice": choice, "ms": times, "ms_large": large,
                   "sample": int(len(sample)), "large_sample": int(big)}
    return _cache[key]


#: Segments per line of the partitioned Thomas solve tried for a lone N-D
#: grid (0: Thomas, one line per thread).
ND_SEGMENTS = (0, 2, 4, 8)

_nd_cache = {}
_nd_lock = None


def tune_nd_line_solver(P, L, steps=8):
    """Segments of the partitioned solve (0: Thomas) with which a lone
    P-population integration on L points runs fastest on this GPU.  Each
    candidate (segments of at least three rows that fit shared memory)
    integrates `steps` steps of a constant parameter table through
    dgb_batchnd_integrate as a batch of one, timed with CUDA events, best of
    3 after a warm-up.  Cached per (device, P, L); returns {"segments": s,
    "ms": {s: ms}}.  Where the few lines of one grid leave the FP64 pipes
    idle the partition wins (3-D grids of 40-90 points: 1.4-1.9x); where
    the grid's lines fill them, or the partition's shared memory leaves one
    CTA per SM, Thomas does (3-D at 120 points, 4-D at 30-40)."""
    import threading
    import torch
    from . import batchnd, integration
    global _nd_lock
    if _nd_lock is None:
        _nd_lock = threading.Lock()
    key = (torch.cuda.get_device_name(torch.cuda.current_device()), int(P), int(L))
    with _nd_lock:
        if key in _nd_cache:
            return _nd_cache[key]
        stride = integration.row_stride(P)
        tab = np.zeros((steps, stride))
        tab[:, 0] = 1e-4                     # dt
        tab[:, 1] = 1.0                      # theta0
        tab[:, 2:2 + P] = 1.0                # nu
        tab[:, 2 + 2 * P:2 + 3 * P] = 0.5    # h
        tab[:, 2 + 3 * P] = 1.0              # beta
        tab[:, 3 + 3 * P:] = 1.0             # migration
        phi0 = torch.ones((L,) * P, dtype=torch.float64, device="cuda")
        times = {}
        for seg in ND_SEGMENTS:
            if seg and L < 3 * seg:
                continue
            eng = batchnd.BatchND(P, L, line_solver=2 if seg else 0, segments=seg)
            try:
                best = None
                for rep in range(4):
                    ev = (torch.cuda.Event(enable_timing=True),
                          torch.cuda.Event(enable_timing=True))
                    eng.integrate(phi0, [tab], timer=ev)
                    torch.cuda.synchronize()
                    if rep:
                        ms = ev[0].elapsed_time(ev[1])
                        best = ms if best is None else min(best, ms)
            except _lib.DgbError as e:
                if e.status == _lib.DGB_ERR_UNSUPPORTED:
                    continue
                raise
            times[seg] = best
        choice = min(times, key=times.get)
        _nd_cache[key] = {"segments": int(choice), "ms": times}
        return _nd_cache[key]


_c2_cache = {}


def tune_2d_cluster(L, steps=16):
    """CTAs of the cluster (0: the one-CTA Thomas path of
    dgb_integrate_table) with which a lone 2-population integration on L
    points runs fastest on this GPU: each candidate (2, 4, 8, 16 CTAs where
    3 CTAs <= L <= 16 CTAs) integrates `steps` steps of a constant table,
    timed with CUDA events, best of 3 after a warm-up.  A cluster size the
    GPU cannot place is skipped.  Cached per (device, L); returns
    {"ctas": c, "ms": {c: ms}}."""
    import threading
    import torch
    from . import integration, numerics
    global _nd_lock
    if _nd_lock is None:
        _nd_lock = threading.Lock()
    key = (torch.cuda.get_device_name(torch.cuda.current_device()), int(L))
    with _nd_lock:
        if key in _c2_cache:
            return _c2_cache[key]
        lib = _lib.lib()
        tab = np.zeros((steps, integration.row_stride(2)))
        tab[:, 0] = 1e-4
        tab[:, 1] = 1.0
        tab[:, 2:4] = 1.0
        tab[:, 6:8] = 0.5
        tab[:, 8] = 1.0
        tab[:, 9:] = 1.0
        xx = numerics.default_grid(L)
        d_xx, d_tab = _lib.to_device(torch, xx), _lib.to_device(torch, tab)
        phi = torch.ones((L, L), dtype=torch.float64, device="cuda")
        ws, nws = _lib.workspace(torch, lib.dgb_workspace_bytes(0, 2, L, 0))
        sh = _lib.stream_handle(torch)

        def run(c):
            if c == 0:
                return lib.dgb_integrate_table(_lib.dptr(phi), 2, L, _lib.dptr(d_xx),
                                               _lib.dptr(d_tab), steps, 0, 0, 0, _lib.dptr(ws),
                                               nws, sh)
            return lib.dgb_integrate2d_cluster(_lib.dptr(phi), L, _lib.dptr(d_xx),
                                               _lib.dptr(d_tab), steps, 0, 0, c, sh)
        times = {}
        for c in (0, 2, 4, 8, 16):
            if c and not 3 * c <= L <= 16 * c:
                continue
            best = None
            for rep in range(4):
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record()
                rc = run(c)
                e1.record()
                if rc != _lib.DGB_OK:
                    break
                torch.cuda.synchronize()
                if rep:
                    ms = e0.elapsed_time(e1)
                    best = ms if best is None else min(best, ms)
            if best is not None:
                times[c] = best
        choice = min(times, key=times.get)
        _c2_cache[key] = {"ctas": int(choice), "ms": times}
        return _c2_cache[key]
