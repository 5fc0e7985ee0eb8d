"""Monte Carlo campaigns over an Eb/N0 grid with com-sim's semantics.

Mirrors the parts of com-sim that drive the BICM-LDPC trial:

* ``Runner::run_condition`` (crates/com-sim/src/runner.rs:417-473): conditions in grid
  order; batches of ``batch`` trials; trial t of condition c draws from
  ``stream(seed, name, c, t)``; the last batch ends at the rule's trial bound
  (``end = min(trials + batch, limit)``, at least one trial);
* ``Stop`` (crates/com-sim/src/stopping.rs:64-188): max_trials, min_trials,
  min_errors, ``or``/``and``, ``trial_limit``, ``is_bounded``;
* ``ErrorRate`` with its Wilson interval and ``Mean`` (crates/com-sim/src/stats.rs:49-160).

One trial is one frame, so a campaign gives the counts of the reference's
one-frame-per-trial scenario under the same seed, name and batch size.
"""

import math
import time
from dataclasses import dataclass, field


class Stop:
    """A stopping rule (crates/com-sim/src/stopping.rs:64-265)."""

    def __init__(self, kind, value=None, metric=None, rules=()):
        self.kind, self.value, self.metric, self.rules = kind, value, metric, tuple(rules)

    @staticmethod
    def max_trials(n):
        return Stop("max_trials", n)

    @staticmethod
    def min_trials(n):
        return Stop("min_trials", n)

    @staticmethod
    def min_errors(metric, errors):
        return Stop("min_errors", errors, metric)

    def or_(self, other):
        return Stop("any", rules=(self, other))

    def and_(self, other):
        return Stop("all", rules=(self, other))

    def is_met(self, trials, record):
        if self.kind in ("max_trials", "min_trials"):
            return trials >= self.value
        if self.kind == "min_errors":
            r = record.get(self.metric)
            return isinstance(r, ErrorRate) and r.errors >= self.value
        if self.kind == "any":
            return any(s.is_met(trials, record) for s in self.rules)
        return all(s.is_met(trials, record) for s in self.rules)

    def is_bounded(self):
        if self.kind == "max_trials":
            return True
        if self.kind in ("min_trials", "min_errors"):
            return False
        if self.kind == "any":
            return any(s.is_bounded() for s in self.rules)
        return all(s.is_bounded() for s in self.rules)

    def trial_limit(self):
        if self.kind in ("max_trials", "min_trials"):
            return self.value
        if self.kind == "min_errors":
            return None
        lims = [s.trial_limit() for s in self.rules]
        if self.kind == "any":
            lims = [x for x in lims if x is not None]
            return min(lims) if lims else None
        return None if any(x is None for x in lims) else max(lims)


def _z_score(confidence):
    # the normal quantile of (1 + confidence) / 2 by bisection on erfc (stats.rs:40-45)
    p = (1.0 - min(max(confidence, 0.0), 1.0 - 1e-16)) / 2.0
    lo, hi = 0.0, 40.0
    for _ in range(200):
        mid = 0.5 * (lo + hi)
        if 0.5 * math.erfc(mid / math.sqrt(2.0)) > p:
            lo = mid
        else:
            hi = mid
    return 0.5 * (lo + hi)


@dataclass
class ErrorRate:
    """Errors among trials (stats.rs:49-90)."""

    errors: int = 0
    total: int = 0

    def add(self, errors, total):
        self.errors += int(errors)
        self.total += int(total)

    def rate(self):
        return float("nan") if self.total == 0 else self.errors / self.total

    def wilson(self, confidence=0.95):
        if self.total == 0:
            return 0.0, 1.0
        n, p, z = float(self.total), self.rate(), _z_score(confidence)
        z2 = z * z
        centre = (p + z2 / (2 * n)) / (1 + z2 / n)
        half = z * math.sqrt(p * (1 - p) / n + z2 / (4 * n * n)) / (1 + z2 / n)
        lower = 0.0 if self.errors == 0 else max(centre - half, 0.0)
        return lower, min(centre + half, 1.0)


@dataclass
class Mean:
    """Running mean (stats.rs:93-160), merged exactly from sums."""

    n: int = 0
    total: float = 0.0

    def add_many(self, count, s):
        self.n += int(count)
        self.total += float(s)

    def value(self):
        return float("nan") if self.n == 0 else self.total / self.n


@dataclass
class ConditionResult:
    index: int
    condition: dict
    trials: int
    wall_s: float
    record: dict = field(default_factory=dict)
    status: str = "completed"

    def metric(self, name):
        return self.record.get(name)


class Grid:
    """The conditions of a campaign: axes in order, the first outermost (grid.rs:321-361)."""

    def __init__(self):
        self.axes = []

    def axis(self, name, values):
        self.axes.append((name, list(values)))
        return self

    def conditions(self):
        out = [{}]
        for name, values in self.axes:
            out = [dict(c, **{name: v}) for c in out for v in values]
        return out


def run(code, grid, stop, seed=0, name="bicm_ldpc", batch=32, modulation=4, on_batch=None, rank=0, world=1,
        all_reduce=None):
    """A campaign of `code` (an NrLdpc) over `grid` (conditions with ``ebn0_db``).

    Returns one ConditionResult per condition with the metrics ``ber``, ``fer``
    (ErrorRate) and ``iterations`` (Mean).

    Several processes (one GPU each) run one campaign together: with ``world`` > 1
    every batch is split into ``world`` contiguous frame ranges, process ``rank`` runs
    its own, and ``all_reduce`` (a function summing an int64 numpy vector over the
    processes, e.g. over torch.distributed) merges the integer counts before the stop
    rule is evaluated.  The result equals the one-process campaign with the same batch.
    """
    import numpy as np

    if not stop.is_bounded():
        raise ValueError("the stopping rule can run forever: add Stop.max_trials with or_")
    if world > 1 and all_reduce is None:
        raise ValueError("a multi-process campaign needs all_reduce")
    batch = max(1, int(batch))
    results = []
    for index, cond in enumerate(grid.conditions()):
        t0 = time.perf_counter()
        rec = {"ber": ErrorRate(), "fer": ErrorRate(), "iterations": Mean()}
        trials = 0
        limit = stop.trial_limit()
        while True:
            end = trials + batch if limit is None else max(min(trials + batch, limit), trials + 1)
            n = end - trials
            lo, hi = trials + n * rank // world, trials + n * (rank + 1) // world
            counts = np.zeros(4, np.int64)
            if hi > lo:
                fr = code.run_frames(seed, name, index, lo, hi - lo, cond["ebn0_db"], modulation)
                counts[:] = (fr["bit_errors"].sum(dtype="u8"), fr["frame_error"].sum(dtype="u8"),
                             fr["iterations"].sum(dtype="u8"), len(fr))
            if world > 1:
                counts = all_reduce(counts)
            rec["ber"].add(counts[0], code.k_info * counts[3])
            rec["fer"].add(counts[1], counts[3])
            rec["iterations"].add_many(counts[3], counts[2])
            trials = end
            if on_batch:
                on_batch(index, trials, rec)
            if stop.is_met(trials, rec):
                break
        results.append(ConditionResult(index, cond, trials, time.perf_counter() - t0, rec))
    return results
