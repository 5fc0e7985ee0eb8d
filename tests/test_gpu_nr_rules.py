"""NR codes with the flooding schedule and the sum-product rule, which run on the generic
sparse decoder over the lifted rows, against the oracle's NrLdpc with the same decoder
settings (LdpcDecoder, crates/com-fec/src/ldpc.rs:165-172).

* min-sum rules, flooding: decisions, a posteriori LLRs, iterations and the per-frame
  Monte Carlo records equal the oracle's bit for bit (f64, correctly rounded noise);
* sum-product (layered, the reference's default, and flooding): the oracle calls the
  platform libm's tanh/atanh and the GPU CUDA's, so frames agree on their outcome and
  iteration count, and early-converging frames on their LLRs to rounding.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NAME = "nr_rules"


def _pair(cb, O, rule, alpha, layered, iters, k=520, e=1040, bg=2, z=52):
    nr = cb.NrLdpc(k, e, base_graph=bg, lifting_size=z, rule=rule, alpha=alpha, layered=layered,
                   max_iterations=iters, precision="f64")
    ref = O.Code(k, e, bg, z)
    ref.set_decoder({"sum_product": O.RULE_SUM_PRODUCT, "normalized_min_sum": O.RULE_NMS,
                     "offset_min_sum": O.RULE_OMS}[rule], alpha, layered, iters)
    return nr, ref


@pytest.mark.parametrize("rule, alpha", [("normalized_min_sum", 0.75), ("offset_min_sum", 0.5)])
def test_flooding_min_sum_equals_the_oracle(cb, O, rule, alpha):
    nr, ref = _pair(cb, O, rule, alpha, False, 20)
    for cond, ebn0 in enumerate((1.0, 2.0)):
        llr, info = nr.generate_frames(7, NAME, cond, 0, 96, ebn0, modulation=4)
        bits, app, it = nr.decode_full(llr)
        for f in range(len(llr)):
            ob, oit, oapp, _ = ref.decode(llr[f], want_app=True)
            assert oit == it[f]
            assert np.array_equal(bits[f], ob)
            assert np.array_equal(app[f].view(np.uint64), oapp.view(np.uint64))
        # the Monte Carlo records through the same decoder
        got = nr.run_frames(7, NAME, cond, 0, 96, ebn0, modulation=4)
        want = ref.run_frames(4, 7, O.fnv1a64(NAME), cond, 0, 96, ebn0)
        for key in ("bit_errors", "frame_error", "iterations"):
            assert np.array_equal(got[key], want[key]), key
    assert len(set(got["iterations"].tolist())) > 3


@pytest.mark.parametrize("layered, iters", [(True, 20), (False, 50)])
def test_sum_product_agrees_with_the_oracle(cb, O, layered, iters):
    nr, ref = _pair(cb, O, "sum_product", 0.0, layered, iters)
    total = same_outcome = same_it = 0
    worst = 0.0
    for cond, ebn0 in enumerate((0.5, 1.25, 2.0)):
        llr, info = nr.generate_frames(7, NAME, 10 + cond, 0, 100, ebn0, modulation=4)
        bits, app, it = nr.decode_full(llr)
        for f in range(len(llr)):
            ob, oit, oapp, _ = ref.decode(llr[f], want_app=True)
            gb = bits[f]
            total += 1
            same_outcome += int(np.array_equal(gb, info[f]) == np.array_equal(ob, info[f]))
            same_it += int(oit == it[f])
            if oit == it[f] and oit <= 5:
                worst = max(worst, float(np.max(np.abs(app[f] - oapp) / np.maximum(1.0, np.abs(oapp)))))
    print(f"NR sum-product layered={layered}: {same_outcome}/{total} same outcome, {same_it}/{total} same "
          f"iterations, worst relative gap (<= 5 iterations) {worst:.3g}")
    assert same_outcome >= 0.99 * total and same_it >= 0.97 * total and worst <= 1e-9


def test_large_code_sum_product_decodes(cb):
    # C2's code with the reference's default rule (sum-product, layered), f32: above the
    # waterfall every frame decodes
    code = cb.NrLdpc(8448, 25344, base_graph=1, lifting_size=384, rule="sum_product", max_iterations=20,
                     precision="f32")
    rec = code.run_frames(7, NAME, 0, 0, 64, 3.0, modulation=16)
    assert rec["frame_error"].sum() == 0 and rec["iterations"].max() < 20
