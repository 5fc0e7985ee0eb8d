"""Monte Carlo campaigns over an Eb/N0 grid with com-sim's semantics.

Mirrors the parts of com-sim that drive the BICM-LDPC trial:

* ``Runner::run_condition`` (crates/com-sim/src/runner.rs:417-473): conditions in grid
  order; batches of ``batch`` trials; trial t of condition c draws from
  ``stream(seed, name, c, t)``; the last batch ends at the rule's trial bound
  (``end = min(trials + batch, limit)``, at least one trial);
* ``Stop`` (crates/com-sim/src/stopping.rs:64-188): max_trials, min_trials,
  min_errors, ``or``/``and``, ``trial_limit``, ``is_bounded``;
* ``ErrorRate`` with its Wilson interval and ``Mean`` (crates/com-sim/src/stats.rs:49-160),
  the z-score by ``qfuncinv`` (crates/com-math/src/special.rs:227-293).

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


# Cody's rational Chebyshev coefficients of erfc (W. J. Cody, Math. Comp. 23(107), 1969;
# his CALERF of SPECFUN, ACM TOMS 19(1), 1993), the ones the reference's erfc uses
# (crates/com-math/src/special.rs:157-262): published numbers, kept digit for digit so
# that the Wilson bounds equal the reference's
_CA = (3.16112374387056560e00, 1.13864154151050156e02, 3.77485237685302021e02, 3.20937758913846947e03,
       1.85777706184603153e-1)
_CB = (2.36012909523441209e01, 2.44024637934444173e02, 1.28261652607737228e03, 2.84423683343917062e03)
_CC = (5.64188496988670089e-1, 8.88314979438837594e00, 6.61191906371416295e01, 2.98635138197400131e02,
       8.81952221241769090e02, 1.71204761263407058e03, 2.05107837782607147e03, 1.23033935479799725e03,
       2.15311535474403846e-8)
_CD = (1.57449261107098347e01, 1.17693950891312499e02, 5.37181101862009858e02, 1.62138957456669019e03,
       3.29079923573345963e03, 4.36261909014324716e03, 3.43936767414372164e03, 1.23033935480374942e03)
_CP = (3.05326634961232344e-1, 3.60344899949804439e-1, 1.25781726111229246e-1, 1.60837851487422766e-2,
       6.58749161529837803e-4, 1.63153871373020978e-2)
_CQ = (2.56852019228982242e00, 1.87295284992346725e00, 5.27905102951428412e-1, 6.05183413124413191e-2,
       2.33520497626869185e-3)


def erfc(x):
    """erfc by Cody's three rational approximations, in the reference's operation order
    (crates/com-math/src/special.rs:227-262); exp is the platform libm's, as in Rust."""
    y = abs(x)
    if y <= 0.46875:
        ysq = y * y if y > 1.11e-16 else 0.0
        num, den = _CA[4] * ysq, ysq
        for i in range(3):
            num = (num + _CA[i]) * ysq
            den = (den + _CB[i]) * ysq
        return 1.0 - x * (num + _CA[3]) / (den + _CB[3])
    if y > 27.3:
        r = 0.0
    else:
        if y <= 4.0:
            num, den = _CC[8] * y, y
            for i in range(7):
                num = (num + _CC[i]) * y
                den = (den + _CD[i]) * y
            r = (num + _CC[7]) / (den + _CD[7])
        else:
            ysq = 1.0 / (y * y)
            num, den = _CP[5] * ysq, ysq
            for i in range(4):
                num = (num + _CP[i]) * ysq
                den = (den + _CQ[i]) * ysq
            r = (5.6418958354775628695e-1 - ysq * (num + _CP[4]) / (den + _CQ[4])) / y
        u = math.trunc(y * 16.0) / 16.0
        r = math.exp(-u * u) * math.exp(-(y - u) * (y + u)) * r
    return 2.0 - r if x < 0.0 else r


def _bisect(below, lo, hi, iters):
    # crates/com-math/src/search.rs:69-80
    for _ in range(iters):
        mid = 0.5 * (lo + hi)
        if below(mid):
            lo = mid
        else:
            hi = mid
    return 0.5 * (lo + hi)


def erfcinv(y):
    """Inverse of erfc on (0, 2) by 200 bisection steps on [-27, 27] (special.rs:264-273)."""
    if y <= 0.0:
        return math.inf
    if y >= 2.0:
        return -math.inf
    return _bisect(lambda x: erfc(x) > y, -27.0, 27.0, 200)


def qfuncinv(p):
    """Q^{-1}(p) = sqrt(2) erfcinv(2 p) (special.rs:291-293)."""
    return math.sqrt(2.0) * erfcinv(2.0 * p)


def z_score(confidence):
    """The two-sided quantile Q^{-1}((1 - confidence) / 2), the level clamped to [0, 1)
    (crates/com-sim/src/stats.rs:43-45)."""
    return qfuncinv((1.0 - min(max(confidence, 0.0), 1.0 - 1e-16)) / 2.0)


_z_score = z_score


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
    """Running mean and variance (crates/com-sim/src/stats.rs:93-160): Welford's update
    for single values, Chan-Golub-LeVeque's exact merge for accumulators.

    Integer-valued batches (the decoder's iteration counts) arrive as (count, sum, sum of
    squares), which the GPU records and a multi-process all-reduce give exactly; the
    batch's mean and squared deviations are formed from those integers and merged.
    ``total`` is the running sum of the values."""

    n: int = 0
    mean_: float = 0.0
    m2: float = 0.0
    total: float = 0

    def add(self, x):
        x = float(x)
        self.n += 1
        d = x - self.mean_
        self.mean_ += d / self.n
        self.m2 += d * (x - self.mean_)
        self.total += x

    def merge(self, o):
        if o.n == 0:
            return
        if self.n == 0:
            self.n, self.mean_, self.m2, self.total = o.n, o.mean_, o.m2, o.total
            return
        n = self.n + o.n
        d = o.mean_ - self.mean_
        self.mean_ += d * o.n / n
        self.m2 += o.m2 + d * d * self.n * o.n / n
        self.n = n
        self.total += o.total

    def add_counts(self, count, s, s2=None):
        """`count` integer values with sum `s` and sum of squares `s2` (None: unknown, the
        variance of this batch is then taken as 0)."""
        count, s = int(count), int(s)
        if count <= 0:
            return
        b = Mean()
        b.n, b.mean_, b.total = count, s / count, s
        if s2 is not None:
            b.m2 = (count * int(s2) - s * s) / count
        self.merge(b)

    def add_many(self, count, s):
        self.add_counts(count, s)

    def count(self):
        return self.n

    def mean(self):
        return float("nan") if self.n == 0 else self.mean_

    value = mean

    def variance(self):
        return float("nan") if self.n < 2 else self.m2 / (self.n - 1)

    def std(self):
        return math.sqrt(self.variance())

    def sem(self):
        return self.std() / math.sqrt(self.n)

    def interval(self, confidence=0.95):
        if self.n < 2:
            return -math.inf, math.inf
        h = z_score(confidence) * self.sem()
        return self.mean_ - h, self.mean_ + h


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
            counts = np.zeros(5, np.int64)
            if hi > lo:
                fr = code.run_frames(seed, name, index, lo, hi - lo, cond["ebn0_db"], modulation)
                it = fr["iterations"].astype(np.int64)
                counts[:] = (fr["bit_errors"].sum(dtype="u8"), fr["frame_error"].sum(dtype="u8"), it.sum(),
                             len(fr), (it * it).sum())
            if world > 1:
                counts = all_reduce(counts)
            rec["ber"].add(counts[0], code.k_info * counts[3])
            rec["fer"].add(counts[1], counts[3])
            rec["iterations"].add_counts(counts[3], counts[2], counts[4])
            trials = end
            if on_batch:
                on_batch(index, trials, rec)
            if stop.is_met(trials, rec):
                break
        results.append(ConditionResult(index, cond, trials, time.perf_counter() - t0, rec))
    return results
