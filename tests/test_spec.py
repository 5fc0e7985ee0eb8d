"""Specifications on the host: the YAML reader, the grid axes, the stopping rule and the
link settings of com-spec (crates/com-spec/src/spec.rs), and the GPU link's host tables
(the random interleaver against the oracle's Interleaver::random).  No GPU needed."""

import os

import numpy as np
import pytest
from conftest import gpu_available

# the com-rs project tree, when a checkout is at hand (COMRS_REFERENCE=<its root>)
REF_ROOT = os.environ.get("COMRS_REFERENCE", "")
REF_SPEC = os.path.join(REF_ROOT, "specs", "bicm_ldpc.yaml") if REF_ROOT else ""

# specs/bicm_ldpc.yaml of com-rs, as its YAML reads (the configuration, restated)
BICM_LDPC = {
    "name": "bicm_ldpc",
    "description": "LDPC (1024, 512) BICM with 16-QAM over AWGN",
    "seed": 6,
    "batch": 8,
    "grid": {"ebn0_db": {"from": 2.5, "to": 5.0, "step": 0.5}},
    "link": [
        {"type": "fec_encode", "code": {"type": "ldpc", "n": 1024, "k": 512, "seed": 1}, "blocks": 8,
         "interleave": True},
        {"type": "map", "constellation": "16-QAM"},
        {"type": "awgn_ebn0", "ebn0_db": "$ebn0_db"},
        "demap",
        {"type": "fec_decode", "code": {"type": "ldpc", "n": 1024, "k": 512, "seed": 1}, "interleave": True},
    ],
    "metrics": {"report": ["ber", "coded_ber", "bler"]},
    "stop": {"min_errors": {"bler": 100}, "min_trials": 8, "max_trials": 400},
    "callbacks": {"skip_below": {"metric": "bler", "threshold": 1e-3, "along": "ebn0_db"}},
}


@pytest.mark.skipif(not REF_SPEC or not os.path.exists(REF_SPEC), reason="COMRS_REFERENCE names no com-rs checkout")
def test_the_reference_specification_reads_as_restated(cb):
    assert cb.load_yaml(open(REF_SPEC).read()) == BICM_LDPC


def test_yaml_subset(cb):
    text = """
# a comment
name: 'x # not a comment'
list:
  - a
  - {k: 1, f: 2.5e-3, t: true, n: null}
  - - nested
    - 7
  - key: v
    other: [1, 2,
            3]
anchor: &a {p: 1}
alias: *a
block: &b
  q: -4
again: *b
quoted: "tab\\tend"
"""
    d = cb.load_yaml(text)
    assert d["name"] == "x # not a comment"
    assert d["list"] == ["a", {"k": 1, "f": 2.5e-3, "t": True, "n": None}, ["nested", 7],
                         {"key": "v", "other": [1, 2, 3]}]
    assert d["alias"] == {"p": 1} and d["again"] == {"q": -4}
    assert d["quoted"] == "tab\tend"
    with pytest.raises(ValueError, match="unknown alias"):
        cb.load_yaml("a: *nothing")
    with pytest.raises(ValueError, match="subset"):
        cb.load_yaml("a: !tag x")


def test_grid_axes_and_stop_rule(cb):
    from importlib import import_module

    spec = import_module("com-rs_gb300.spec")
    # spec.rs:373-406
    assert spec._axis("e", {"from": 2.5, "to": 5.0, "step": 0.5}) == [2.5, 3.0, 3.5, 4.0, 4.5, 5.0]
    assert spec._axis("m", {"from": 0, "to": 10, "step": 5}) == [0, 5, 10]
    assert spec._axis("r", {"linspace": [1.0, 2.0, 3]}) == [1.0, 1.5, 2.0]
    assert spec._axis("x", 3) == [3] and spec._axis("x", [1, 2]) == [1, 2]
    with pytest.raises(ValueError, match="an axis is"):
        spec._axis("e", {"from": 1, "to": 0, "step": 1})
    # spec.rs:118-150: (min_errors and min_trials) or max_trials
    stop = spec._stop(BICM_LDPC["stop"])
    assert stop.is_bounded() and stop.trial_limit() == 400
    E = cb.campaign.ErrorRate
    assert not stop.is_met(8, {"bler": E(99, 64)}) and stop.is_met(8, {"bler": E(100, 64)})
    assert not stop.is_met(7, {"bler": E(150, 56)}) and stop.is_met(400, {"bler": E(0, 3200)})
    assert spec._stop({}).trial_limit() == 100 and spec._stop({"min_trials": 5}).trial_limit() == 5
    with pytest.raises(ValueError, match="reads max_trials"):
        spec._stop({"max_time_s": 3})


def test_link_settings(cb):
    from importlib import import_module

    spec = import_module("com-rs_gb300.spec")
    s = spec._link_settings(BICM_LDPC["link"])
    assert s == {"n": 1024, "k": 512, "var_degree": 3, "peg_seed": 1, "rule": "sum_product", "alpha": 0.8,
                 "layered": True, "iterations": 50, "blocks": 8, "interleave": True, "interleaver_seed": 0,
                 "modulation": 16, "ebn0_db": "$ebn0_db", "demap": "exact"}
    assert spec._modulation("qpsk") == 4 and spec._modulation("64_QAM") == 64
    with pytest.raises(ValueError, match="order 4, 16, 64 or 256"):
        spec._modulation("8-PSK")
    bad = [dict(b) if isinstance(b, dict) else b for b in BICM_LDPC["link"]]
    bad[4] = dict(bad[4], interleave=False)
    with pytest.raises(ValueError, match="same interleaver"):
        spec._link_settings(bad)
    with pytest.raises(ValueError, match="the GPU runs"):
        spec._link_settings(BICM_LDPC["link"][:3])
    bad = [dict(b) if isinstance(b, dict) else b for b in BICM_LDPC["link"]]
    bad[2] = {"type": "awgn_ebn0"}
    with pytest.raises(ValueError, match="ebn0_db is required"):
        spec._link_settings(bad)


def test_link_host_tables(cb, O):
    # Interleaver::random(n blocks, seed) (interleaving.rs:63-67) equals the oracle's
    code = cb.Ldpc.peg(96, 48)
    link = cb.Link(code, blocks=3, modulation=64, interleave=True, interleaver_seed=5)
    assert (link.k, link.n, link.blocks, link.payload_bits) == (48, 96, 3, 144)
    assert link.sent_bits == 288 and link.padding == 0
    assert link.interleaver().tolist() == O.random_perm(288, 5).tolist()
    link2 = cb.Link(code, blocks=1, modulation=64)
    assert link2.padding == 0 and link2.sent_bits == 96
    link3 = cb.Link(cb.Ldpc.peg(100, 50), blocks=1, modulation=64)
    assert link3.padding == 2 and link3.sent_bits == 102
    with pytest.raises(cb.ComrsError, match="no interleaver"):
        link3.interleaver()
    with pytest.raises(cb.ComrsError, match="from_rows encoder"):
        n, _, rows = cb.dvbs2.ldpc_rows("short", "1/2")
        cb.Link(cb.Ldpc.accumulate(n, rows))
    with pytest.raises(cb.ComrsError, match="modulation order"):
        cb.Link(code, modulation=8)


@pytest.mark.skipif(gpu_available(), reason="checks the behaviour without a GPU")
def test_link_without_a_gpu_fails_loudly(cb):
    link = cb.Link(cb.Ldpc.peg(96, 48), blocks=2, modulation=16)
    with pytest.raises(cb.ComrsError) as e:
        link.run_trials(1, "x", 0, 0, 4, 3.0)
    assert e.value.status == -6


class OracleLink:
    """The run_trials surface of the GPU Link, computed by the oracle (CPU)."""

    def __init__(self, O, cb, n, k, blocks, m, il_seed, exact, rule, alpha, iters):
        self.O = O
        self.code = O.Code(rows=cb.ldpc.peg_rows(n, k), n=n)
        self.code.set_decoder(rule, alpha, True, iters)
        self.code.set_demapper(exact)
        self.blocks, self.m, self.il_seed = blocks, m, il_seed
        self.sent_bits = n * blocks + (-(n * blocks)) % int(np.log2(m))
        self.payload_bits = k * blocks

    def run_trials(self, seed, name, cond, first, n, ebn0):
        out, _, _ = self.code.link_trials(self.blocks, self.il_seed, self.m, seed, self.O.fnv1a64(name), cond, first,
                                          n, ebn0, self.O.NOISE_CR, 1)
        rec = np.zeros(n, [("raw_bit_errors", "<u4"), ("coded_bit_errors", "<u4"), ("block_errors", "<u4"),
                           ("iterations", "<u4")])
        rec["raw_bit_errors"], rec["coded_bit_errors"] = out[:, 0], out[:, 2]
        rec["block_errors"], rec["iterations"] = out[:, 4], out[:, 6]
        return rec


SMALL = {"name": "bicm_small", "seed": 3, "batch": 6, "grid": {"ebn0_db": [2.0, 5.0, 7.0, 9.0]},
         "link": [{"type": "fec_encode", "code": {"type": "ldpc", "n": 96, "k": 48, "rule": "normalized_min_sum",
                                                  "alpha": 0.75, "iterations": 20}, "blocks": 3, "interleave": True},
                  {"type": "map", "constellation": "16-QAM"}, {"type": "awgn_ebn0", "ebn0_db": "$ebn0_db"},
                  {"type": "demap", "max_log": True},
                  {"type": "fec_decode", "code": {"type": "ldpc", "n": 96, "k": 48, "rule": "normalized_min_sum",
                                                  "alpha": 0.75, "iterations": 20}, "interleave": True}],
         "stop": {"min_errors": {"bler": 12}, "min_trials": 6, "max_trials": 40},
         "callbacks": {"skip_below": {"metric": "bler", "threshold": 0.05, "along": "ebn0_db"}}}


def _small_link(O, cb):
    return OracleLink(O, cb, 96, 48, 3, 16, 0, False, O.RULE_NMS, 0.75, 20)


def _summary(res):
    return [(r.status, r.trials) + tuple((e.errors, e.total) for k, e in sorted(r.record.items()) if k != "iterations")
            + ((r.record["iterations"].total,) if "iterations" in r.record else ()) for r in res]


def _spec_rank(rank, world, port, out):
    import sys

    from conftest import ROOT
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

    spec = __import__("importlib").import_module("com-rs_gb300.spec")
    out[rank] = _summary(spec.run_spec_with(_small_link(O, cb), SMALL, rank=rank, world=world, all_reduce=all_reduce))
    dist.destroy_process_group()


def test_spec_campaign_semantics_and_two_processes(cb, O):
    # run_spec's loop on the oracle's trials: batches of 6, (min_errors and min_trials) or
    # max_trials, skip_below; two gloo processes give the one-process result
    import socket

    import torch.multiprocessing as mp

    spec = __import__("importlib").import_module("com-rs_gb300.spec")
    one = spec.run_spec_with(_small_link(O, cb), SMALL)
    assert [r.status for r in one][:1] == ["completed"]
    for r in one:
        if r.status == "completed":
            b = r.record["bler"]
            assert r.trials == 40 or (b.errors >= 12 and r.trials >= 6)
            assert r.trials % 6 == 0 or r.trials == 40
    assert [r.status for r in one] == ["completed"] * 3 + ["skipped"]  # the floor is reached at 7 dB
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    out = ctx.Manager().dict()
    procs = [ctx.Process(target=_spec_rank, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    assert out[0] == out[1] == _summary(one)
