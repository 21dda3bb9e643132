"""Autotuner of the E-step's tile order and per-stage schedules.

The reference fixes its kernels' block sizes and schedules at compile time
(src/acc/cuda/cuda_settings.h); here the choices that depend on the shape of
an iteration -- the coarse tensor-core kernel's tile-order group and its
one-SM or SM-pair form, the fine pass as sparse jobs or dense contractions,
the sparse pass's slices summed per orientation before the backprojection or
inserted directly -- are measured on the iteration's first batch and the
fastest kept.

Each choice is timed on its own stage (CUDA events of the worker's stages):
the coarse-kernel candidates on the cross-term stage, the fine-pass forms on
the stages they run (fine diff2, fine weights, weighted sums,
backprojection; the dense form runs only where its arrays fit the device
budget, otherwise the library keeps the sparse one).  The coarse candidates
give bit-identical results; the fine-pass forms agree to FP32 rounding.
Tuning runs the E-step on the batch, which adds to the bundle's weighted
sums and volumes: tune() therefore clears them afterwards
(gbr_bundle_reset_wsum), so it belongs at the start of an iteration, before
the batches whose sums are kept.
"""
import numpy as np

from .estep import STAGES

# candidate settings, each a dict of worker options
COARSE_CANDIDATES = [dict(tile_group=g, pair=p) for p in (0, 1) for g in (16, 24, 32, 48)]
FINE_CANDIDATES = [dict(fine_mode="sparse", bp_direct=0), dict(fine_mode="sparse", bp_direct=1),
                   dict(fine_mode="dense", bp_direct=0)]
COARSE_STAGES = ("cross_gemm",)
FINE_STAGES = ("diff2_fine", "weights_fine", "wsum", "backproject")

_cache = {}


def shape_key(bundle, n):
    """What the choice depends on: box, sizes, grid and batch size."""
    d = bundle.desc
    return (int(d.ori_size), int(d.current_size), int(d.coarse_size), int(bundle.nr_classes), int(bundle.ndir),
            int(bundle.npsi), int(bundle.ntrans), int(d.precision), int(n))


def stage_cost(times_before, times_after, stages, calls):
    """Mean time per call of the given stages (ms) from two stage_times()."""
    idx = [STAGES.index(s) for s in stages]
    return float(np.sum((np.asarray(times_after) - np.asarray(times_before))[idx])) / calls


def time_candidate(worker, batch, options, stages, repeats=2, warmup=1, bail=None):
    """Set the options on the worker, run the batch warmup + repeats times
    and return the mean cost of the stages (ms per call); inf if the library
    refuses the setting for this shape (an error status, e.g. no memory).
    With bail (ms), a candidate whose warm-up call already costs more is not
    repeated: the warm-up cost is returned."""
    try:
        for k, v in options.items():
            worker.set_option(k, v)
        t_w = worker.stage_times().copy()
        for _ in range(warmup):
            worker.do_expectation_some_particles(batch)
        t0 = worker.stage_times().copy()
        if bail is not None and warmup > 0 and stage_cost(t_w, t0, stages, warmup) > bail:
            return stage_cost(t_w, t0, stages, warmup)
        for _ in range(repeats):
            worker.do_expectation_some_particles(batch)
    except RuntimeError:
        return float("inf")
    return stage_cost(t0, worker.stage_times(), stages, repeats)


def pick(measurements):
    """The fastest (options, ms) of a list of (options, ms); the first of
    equal ones."""
    best = None
    for opts, ms in measurements:
        if best is None or ms < best[1]:
            best = (opts, ms)
    return best


def tune(bundle, worker, batch, repeats=2, coarse=None, fine=None, use_cache=True):
    """Pick the coarse-kernel and fine-pass settings for this bundle's shape
    on `batch`, set them on the worker, clear the bundle's weighted sums and
    return {"options": chosen, "coarse": [(options, ms)], "fine": [...]}.
    With use_cache, a shape tuned before is not measured again."""
    key = shape_key(bundle, int(batch["n"]))
    if use_cache and key in _cache:
        chosen = _cache[key]
        for k, v in chosen.items():
            worker.set_option(k, v)
        return {"options": dict(chosen), "coarse": [], "fine": [], "cached": True}
    coarse = COARSE_CANDIDATES if coarse is None else coarse
    fine = FINE_CANDIDATES if fine is None else fine
    precision = int(bundle.desc.precision)
    cm = []
    if precision == 1:  # the coarse kernel choices exist on the tensor-core path only
        for opts in coarse:
            cm.append((opts, time_candidate(worker, batch, opts, COARSE_STAGES, repeats)))
        best_c = pick(cm)[0]
    else:
        best_c = {}
    for k, v in best_c.items():
        worker.set_option(k, v)
    # a fine-pass form whose warm-up call costs 4x the best so far is not
    # repeated (the dense form on a shape with few significant poses)
    fm = []
    for opts in fine:
        best = min([ms for _, ms in fm], default=float("inf"))
        fm.append((opts, time_candidate(worker, batch, opts, FINE_STAGES, repeats,
                                        bail=4 * best if best < float("inf") else None)))
    best_f = pick(fm)[0]
    chosen = dict(best_c)
    chosen.update(best_f)
    for k, v in chosen.items():
        worker.set_option(k, v)
    bundle.reset_wsum()
    _cache[key] = dict(chosen)
    return {"options": chosen, "coarse": cm, "fine": fm, "cached": False}
