"""Campaign semantics (com-sim's Runner, Stop, ErrorRate) on the CPU, with the oracle's
frames standing in for the GPU's: one process and two gloo processes."""

import os

import numpy as np
import pytest

from conftest import ROOT

NAME = "bicm_ldpc"


class OracleFrames:
    """The run_frames/k_info surface of NrLdpc, computed by the oracle (CPU)."""

    def __init__(self, O, k, e, bg, z):
        self.O = O
        self.code = O.Code(k, e, bg=bg, z=z).set_decoder(O.RULE_NMS, 0.75, True, 20)
        self.k_info = k

    def run_frames(self, seed, name, cond, first, n, ebn0, modulation):
        return self.code.run_frames(modulation, seed, self.O.fnv1a64(name), cond, first, n, ebn0, 0,
                                    self.O.NOISE_CR, 1)


def test_stop_rules(cb):
    S = cb.Stop
    # crates/com-sim/src/stopping.rs:170-177 doc examples
    assert S.min_errors("ber", 100).or_(S.max_trials(1000)).trial_limit() == 1000
    assert S.max_trials(1000).and_(S.min_trials(10)).trial_limit() == 1000
    assert S.min_errors("ber", 100).and_(S.max_trials(1000)).trial_limit() is None
    assert not S.min_errors("fer", 5).is_bounded() and S.min_errors("fer", 5).or_(S.max_trials(9)).is_bounded()


def test_wilson_interval(cb):
    e = cb.campaign.ErrorRate(0, 100)
    lo, hi = e.wilson(0.95)
    assert lo == 0.0 and 0.03 < hi < 0.04
    assert cb.campaign.ErrorRate().wilson() == (0.0, 1.0)
    lo, hi = cb.campaign.ErrorRate(50, 100).wilson(0.95)
    assert abs((lo + hi) / 2 - 0.5) < 1e-12 and abs(hi - lo - 2 * 0.0962) < 2e-3


def test_grid_order(cb):
    g = cb.Grid().axis("a", [1, 2]).axis("b", [10, 20])
    assert g.conditions() == [{"a": 1, "b": 10}, {"a": 1, "b": 20}, {"a": 2, "b": 10}, {"a": 2, "b": 20}]


@pytest.mark.parametrize("batch", [1, 7, 64])
def test_max_trials_is_met_exactly_whatever_the_batch(cb, O, batch):
    # crates/com-sim/src/runner.rs:495-520
    code = OracleFrames(O, 520, 1040, 2, 52)
    res = cb.run(code, cb.Grid().axis("ebn0_db", [3.0]), cb.Stop.max_trials(100), seed=7, batch=batch)
    assert res[0].trials == 100 and res[0].record["fer"].total == 100


def test_min_errors_stops_after_the_batch(cb, O):
    code = OracleFrames(O, 520, 1040, 2, 52)
    res = cb.run(code, cb.Grid().axis("ebn0_db", [0.0]), cb.Stop.min_errors("fer", 5).or_(cb.Stop.max_trials(1000)),
                 seed=7, batch=16)
    assert res[0].trials == 16 and res[0].record["fer"].errors >= 5


def _rank(rank, world, port, out):
    import sys

    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import torch.distributed as dist

    import oracle as O
    from conftest import load_package

    cb = load_package()
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)

    def all_reduce(v):
        import torch

        t = torch.from_numpy(np.asarray(v, np.int64).copy())
        dist.all_reduce(t)
        return t.numpy()

    code = OracleFrames(O, 520, 1040, 2, 52)
    res = cb.run(code, cb.Grid().axis("ebn0_db", [0.5, 2.0]), cb.Stop.min_errors("fer", 20).or_(cb.Stop.max_trials(300)),
                 seed=7, name=NAME, batch=50, rank=rank, world=world, all_reduce=all_reduce)
    out[rank] = [(r.trials, r.record["fer"].errors, r.record["ber"].errors, r.record["iterations"].total)
                 for r in res]
    dist.destroy_process_group()


def test_two_process_campaign_equals_one_process(cb, O):
    import socket

    import torch.multiprocessing as mp

    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    out = ctx.Manager().dict()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    code = OracleFrames(O, 520, 1040, 2, 52)
    one = cb.run(code, cb.Grid().axis("ebn0_db", [0.5, 2.0]), cb.Stop.min_errors("fer", 20).or_(cb.Stop.max_trials(300)),
                 seed=7, name=NAME, batch=50)
    want = [(r.trials, r.record["fer"].errors, r.record["ber"].errors, r.record["iterations"].total) for r in one]
    assert out[0] == out[1] == want


def test_statistics_known_answers_of_the_reference(cb):
    # crates/com-sim/src/stats.rs:20-36 (module example), :230-249
    # (wilson_with_no_error_and_merges); crates/com-math/src/special.rs:221-224, :286-289
    c = cb.campaign
    e = c.ErrorRate()
    e.add(3, 1000)
    e.add(7, 1000)
    assert e.rate() == 5e-3
    lo, hi = e.wilson(0.95)
    assert lo < 5e-3 < hi
    m = c.Mean()
    for v in (1.0, 2.0, 3.0, 4.0):
        m.add(v)
    assert (m.mean(), m.variance()) == (2.5, 5.0 / 3.0)
    assert abs(c.z_score(0.95) - 1.959964) < 1e-5
    assert abs(c.qfuncinv(0.025) - 1.959964) < 1e-6
    q = 0.5 * c.erfc(c.qfuncinv(1e-6) / 2 ** 0.5)
    assert abs(q / 1e-6 - 1.0) < 1e-9
    assert abs(c.erfc(1.0) / 0.15729920705028513 - 1.0) < 1e-15
    assert abs(c.erfc(10.0) / 2.0884875837625448e-45 - 1.0) < 1e-15
    lo, hi = c.ErrorRate(0, 1000).wilson(0.95)
    assert lo == 0.0 and abs(hi - 3.83e-3) < 1e-4
    import math

    a, b, whole = c.Mean(), c.Mean(), c.Mean()
    for i in range(100):
        v = math.sin(i * 0.37)
        (a if i < 30 else b).add(v)
        whole.add(v)
    a.merge(b)
    assert abs(a.mean() - whole.mean()) < 1e-14 and abs(a.variance() - whole.variance()) < 1e-14


def test_integer_batches_give_the_exact_mean_and_variance(cb):
    import numpy as np

    c = cb.campaign
    x = np.random.default_rng(1).integers(0, 21, 5000)
    m = c.Mean()
    for part in np.array_split(x, 7):
        m.add_counts(len(part), int(part.sum()), int((part * part).sum()))
    assert m.count() == 5000 and m.total == int(x.sum())
    assert abs(m.mean() - x.mean()) < 1e-12 and abs(m.variance() - x.var(ddof=1)) < 1e-9
