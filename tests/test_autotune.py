"""CPU tests of the autotuner's logic (relion_gb300/autotune.py) with a
stand-in worker whose stage times depend on its options: per-stage costs,
the choice of the fastest candidate per stage group, refused settings, the
cache and the reset of the bundle's sums."""
import numpy as np
import pytest

from relion_gb300 import autotune
from relion_gb300.estep import STAGES


class FakeDesc:
    ori_size, current_size, coarse_size, precision = 64, 28, 24, 1


class FakeBundle:
    nr_classes, ndir, npsi, ntrans = 1, 48, 12, 13

    def __init__(self, precision=1):
        self.desc = FakeDesc()
        self.desc.precision = precision
        self.resets = 0

    def reset_wsum(self):
        self.resets += 1


class FakeWorker:
    """Cross-term time by tile group / pair, fine-stage time by fine mode and
    direct slice insertion (slower weighted sums, no backprojection pass)."""

    def __init__(self, refuse=None):
        self.opts = {}
        self.t = np.zeros(len(STAGES))
        self.refuse = refuse or {}

    def set_option(self, k, v):
        if self.refuse.get(k) == v:
            raise RuntimeError("refused")
        self.opts[k] = v

    def do_expectation_some_particles(self, batch):
        g, p = self.opts.get("tile_group", 32), self.opts.get("pair", 0)
        self.t[STAGES.index("cross_gemm")] += 6.0 + abs(g - 24) * 0.01 + 0.9 * p
        dense = self.opts.get("fine_mode") == "dense"
        direct = self.opts.get("bp_direct", 0) == 1
        self.t[STAGES.index("diff2_fine")] += 0.5 if dense else 0.3
        self.t[STAGES.index("wsum")] += 0.25 if direct else 0.2
        self.t[STAGES.index("backproject")] += 0.0 if direct else 0.1
        self.t[STAGES.index("prep")] += 0.05

    def stage_times(self):
        return self.t.copy()


def test_stage_cost():
    a, b = np.zeros(len(STAGES)), np.zeros(len(STAGES))
    b[STAGES.index("cross_gemm")] = 12.0
    b[STAGES.index("prep")] = 5.0
    assert autotune.stage_cost(a, b, ("cross_gemm",), 2) == 6.0


def test_tune_picks_fastest_per_stage_group_and_resets():
    autotune._cache.clear()
    bundle, worker = FakeBundle(), FakeWorker()
    out = autotune.tune(bundle, worker, {"n": 8}, repeats=2)
    assert out["options"] == dict(tile_group=24, pair=0, fine_mode="sparse", bp_direct=1)
    assert worker.opts == out["options"]
    assert bundle.resets == 1
    ms = dict((tuple(sorted(o.items())), v) for o, v in out["coarse"])
    assert ms[(("pair", 0), ("tile_group", 24))] == pytest.approx(6.0)
    assert ms[(("pair", 1), ("tile_group", 24))] == pytest.approx(6.9)


def test_tune_uses_cache_for_same_shape():
    autotune._cache.clear()
    bundle, w1 = FakeBundle(), FakeWorker()
    autotune.tune(bundle, w1, {"n": 8})
    w2 = FakeWorker()
    out = autotune.tune(bundle, w2, {"n": 8})
    assert out["cached"] and w2.opts == w1.opts and bundle.resets == 1
    out3 = autotune.tune(bundle, FakeWorker(), {"n": 16})   # another batch size: measured again
    assert not out3["cached"]


def test_refused_candidate_is_skipped():
    autotune._cache.clear()
    out = autotune.tune(FakeBundle(), FakeWorker(refuse={"pair": 1}), {"n": 4})
    assert out["options"]["pair"] == 0
    assert all(v == float("inf") for o, v in out["coarse"] if o["pair"] == 1)


def test_plain_path_skips_coarse_candidates():
    autotune._cache.clear()
    out = autotune.tune(FakeBundle(precision=0), FakeWorker(), {"n": 4})
    assert out["coarse"] == [] and out["options"] == dict(fine_mode="sparse", bp_direct=1)


class SlowDenseWorker(FakeWorker):
    """The dense fine-pass form 10x slower than the sparse ones."""

    def do_expectation_some_particles(self, batch):
        super().do_expectation_some_particles(batch)
        if self.opts.get("fine_mode") == "dense":
            self.t[STAGES.index("diff2_fine")] += 10.0
        self.calls = getattr(self, "calls", 0) + 1


def test_slow_fine_candidate_is_not_repeated():
    autotune._cache.clear()
    w = SlowDenseWorker()
    out = autotune.tune(FakeBundle(), w, {"n": 8}, repeats=2)
    ms = {(o["fine_mode"], o["bp_direct"]): v for o, v in out["fine"]}
    assert ms[("dense", 0)] > 4 * min(ms[("sparse", 0)], ms[("sparse", 1)])
    # 8 coarse candidates x 3 calls, 2 sparse forms x 3 calls, the dense form's warm-up call only
    assert w.calls == 8 * 3 + 2 * 3 + 1
    assert out["options"]["fine_mode"] == "sparse"
