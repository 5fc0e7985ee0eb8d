"""The spec link (fec_encode -> map -> awgn_ebn0 -> demap -> fec_decode over a PEG code,
specs/bicm_ldpc.yaml of com-rs) on the GPU against the oracle's restatement of the same
trials (oracle.cpp link_trial):

* max-log demapper and min-sum decoder: every count of every trial (uncoded, coded and
  block errors, iterations) equals the oracle's;
* the specification's own settings (exact demapper, sum-product): the decoder inputs
  equal the oracle's within CUDA's exp/log against libm, the payload and the uncoded
  errors exactly, the coded outcome on nearly every trial;
* run_spec: the campaign of a specification equals the oracle's trials batch by batch,
  and skip_below skips the rest of a sweep.
"""

import copy

import numpy as np
import pytest
from test_spec import BICM_LDPC

pytestmark = pytest.mark.gpu

NAME = "bicm_ldpc"


def _pair(cb, O, n, k, blocks, m, interleave, demap, rule, alpha, iters, il_seed=0):
    rows = cb.ldpc.peg_rows(n, k)
    code = cb.Ldpc(n, rows, rule=rule, alpha=alpha, max_iterations=iters)
    link = cb.Link(code, blocks, m, interleave, il_seed, demap)
    ref = O.Code(rows=rows, n=n)
    ref.set_decoder({"sum_product": O.RULE_SUM_PRODUCT, "normalized_min_sum": O.RULE_NMS}[rule], alpha, True, iters)
    ref.set_demapper(demap == "exact")
    return link, ref


@pytest.mark.parametrize("n, k, blocks, m, interleave", [(1024, 512, 8, 16, True), (100, 50, 1, 64, False),
                                                         (96, 48, 5, 4, True), (256, 128, 2, 256, True)])
def test_max_log_min_sum_link_equals_the_oracle(cb, O, n, k, blocks, m, interleave):
    link, ref = _pair(cb, O, n, k, blocks, m, interleave, "max_log", "normalized_min_sum", 0.75, 20, il_seed=3)
    assert link.padding == -(n * blocks) % int(np.log2(m))
    trials, seen = 48, set()
    for cond, ebn0 in enumerate((1.5, 3.0, 4.5, 6.0, 9.0)):
        rec = link.run_trials(6, NAME, cond, 5, trials, ebn0)
        out, _, _ = ref.link_trials(blocks, 3 if interleave else None, m, 6, O.fnv1a64(NAME), cond, 5, trials, ebn0)
        assert (out[:, 1] == link.sent_bits).all() and (out[:, 3] == link.payload_bits).all()
        assert np.array_equal(rec["raw_bit_errors"], out[:, 0]), ebn0
        assert np.array_equal(rec["coded_bit_errors"], out[:, 2]), ebn0
        assert np.array_equal(rec["block_errors"], out[:, 4]), ebn0
        assert np.array_equal(rec["iterations"], out[:, 6]), ebn0
        seen |= {int(x > 0) for x in rec["block_errors"]}
    assert seen == {0, 1}


def test_the_specification_settings_agree_with_the_oracle(cb, O):
    # specs/bicm_ldpc.yaml: PEG(1024, 512), 8 blocks, interleaved, 16-QAM, exact LLRs,
    # layered sum-product with 50 iterations
    link, ref = _pair(cb, O, 1024, 512, 8, 16, True, "exact", "sum_product", 0.8, 50)
    trials = 64
    same = total = 0
    for cond, ebn0 in enumerate((2.5, 3.5)):
        llr, pay, raw = link.generate(6, NAME, cond, 0, trials, ebn0)
        out, llr_o, pay_o = ref.link_trials(8, 0, 16, 6, O.fnv1a64(NAME), cond, 0, trials, ebn0, want_llr=True,
                                            want_payload=True)
        assert np.array_equal(pay, pay_o)
        assert np.array_equal(raw, out[:, 0])
        np.testing.assert_allclose(llr, llr_o, rtol=1e-12, atol=1e-11)
        rec = link.run_trials(6, NAME, cond, 0, trials, ebn0)
        assert np.array_equal(rec["raw_bit_errors"], out[:, 0])
        same += int((rec["block_errors"] == out[:, 4]).sum())
        total += trials
    assert same >= 0.98 * total


def test_f32_decoder_link_equals_the_oracle_on_rounded_llrs(cb, O):
    # an f32 code: the f64 LLRs rounded once to f32, decoded in f32; the counts equal the
    # oracle's f32 decoder (min-sum, bit-exact) on the same rounded LLRs
    rows = cb.ldpc.peg_rows(1024, 512)
    code = cb.Ldpc(1024, rows, rule="normalized_min_sum", alpha=0.75, max_iterations=20, precision="f32")
    link = cb.Link(code, 8, 16, True, 0, "max_log")
    link64 = cb.Link(cb.Ldpc(1024, rows, rule="normalized_min_sum", alpha=0.75, max_iterations=20), 8, 16, True, 0,
                     "max_log")
    ref = O.Code(rows=rows, n=1024)
    ref.set_decoder(O.RULE_NMS, 0.75, True, 20)
    info = code.info_positions()
    for cond, ebn0 in enumerate((3.5, 4.5)):
        llr32, pay, raw = link.generate(6, NAME, cond, 0, 32, ebn0)
        llr64, pay64, raw64 = link64.generate(6, NAME, cond, 0, 32, ebn0)
        assert np.array_equal(pay, pay64) and np.array_equal(raw, raw64)
        assert np.array_equal(llr32, llr64.astype(np.float32).astype(np.float64))
        post, its = ref.decode_llr_many(llr32.reshape(-1, 1024).astype(np.float32), "f32")
        dec = (post[:, info] < 0).astype(np.uint8)
        err = (dec != pay.reshape(-1, 512)).sum(axis=1).reshape(32, 8)
        rec = link.run_trials(6, NAME, cond, 0, 32, ebn0)
        assert np.array_equal(rec["coded_bit_errors"], err.sum(axis=1))
        assert np.array_equal(rec["block_errors"], (err > 0).sum(axis=1))
        assert np.array_equal(rec["iterations"], its.reshape(32, 8).sum(axis=1))
        assert np.array_equal(rec["raw_bit_errors"], raw)


def _spec(**over):
    s = copy.deepcopy(BICM_LDPC)
    s.update(over)
    return s


def test_run_spec_equals_the_oracle_trials(cb, O):
    # the campaign of the specification with a min-sum decoder and the max-log demapper,
    # 24 trials per condition in batches of 8: every count equals the oracle's
    spec = _spec(grid={"ebn0_db": [3.0, 4.0]}, stop={"max_trials": 24})
    spec["link"][3] = {"type": "demap", "max_log": True}
    for i in (0, 4):
        spec["link"][i]["code"].update(rule="normalized_min_sum", alpha=0.75, iterations=20)
    res = cb.run_spec(spec)
    assert [r.trials for r in res] == [24, 24]
    rows = cb.ldpc.peg_rows(1024, 512)
    ref = O.Code(rows=rows, n=1024)
    ref.set_decoder(O.RULE_NMS, 0.75, True, 20)
    ref.set_demapper(False)
    for r in res:
        out, _, _ = ref.link_trials(8, 0, 16, 6, O.fnv1a64(NAME), r.index, 0, 24, r.condition["ebn0_db"])
        assert (r.record["ber"].errors, r.record["ber"].total) == (out[:, 0].sum(), out[:, 1].sum())
        assert (r.record["coded_ber"].errors, r.record["coded_ber"].total) == (out[:, 2].sum(), out[:, 3].sum())
        assert (r.record["bler"].errors, r.record["bler"].total) == (out[:, 4].sum(), out[:, 5].sum())


def test_run_spec_of_the_specification_and_skip_below(cb):
    # the specification as written, fewer trials: the bler falls along Eb/N0
    res = cb.run_spec(_spec(grid={"ebn0_db": [2.5, 4.0]}, stop={"max_trials": 16}))
    b = [r.record["bler"].rate() for r in res]
    assert b[0] > b[1] and all(r.status == "completed" for r in res)
    # skip_below: once the bler is under the threshold the rest of the sweep is skipped
    spec = _spec(grid={"ebn0_db": [5.0, 5.5, 6.0]}, stop={"max_trials": 8},
                 callbacks={"skip_below": {"metric": "bler", "threshold": 0.9, "along": "ebn0_db"}})
    res = cb.run_spec(spec)
    assert [r.status for r in res] == ["completed", "skipped", "skipped"]
    assert res[0].trials == 8 and res[1].trials == 0


def test_link_follows_the_codes_decoder(cb, O):
    # set_decoder on the code after the link ran: the next trials use the new decoder
    rows = cb.ldpc.peg_rows(96, 48)
    code = cb.Ldpc(96, rows, rule="normalized_min_sum", alpha=0.75, max_iterations=20)
    link = cb.Link(code, 4, 16, True, 1, "max_log")
    link.run_trials(6, NAME, 0, 0, 8, 4.0)
    code.set_decoder("offset_min_sum", alpha=0.15, layered=False, max_iterations=20)
    rec = link.run_trials(6, NAME, 0, 0, 32, 4.0)
    ref = O.Code(rows=rows, n=96)
    ref.set_decoder(O.RULE_OMS, 0.15, False, 20)
    ref.set_demapper(False)
    out, _, _ = ref.link_trials(4, 1, 16, 6, O.fnv1a64(NAME), 0, 0, 32, 4.0)
    assert np.array_equal(rec["coded_bit_errors"], out[:, 2]) and np.array_equal(rec["iterations"], out[:, 6])
    assert np.array_equal(rec["raw_bit_errors"], out[:, 0])
