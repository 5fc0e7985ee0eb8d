"""The learned min-sum's CPU oracle: plain weights reproduce the min-sum, and the
adjoint gradients match finite differences (f64)."""

import numpy as np
import pytest

NAME = "learned"


def frames(O, code, n, ebn0, m=4, cond=0):
    h = O.fnv1a64(NAME)
    llr = np.zeros((n, code.e))
    cw = np.zeros((n, code.n_full), np.uint8)
    for f in range(n):
        info, llr[f], _ = code.trial(m, 3, h, cond, f, ebn0)
        u = np.zeros(code.k, np.uint8)
        u[:code.k_info] = info
        cw[f] = code.encode_full(u)
    return llr, cw


@pytest.mark.parametrize("shared", [False, True])
def test_plain_weights_are_the_min_sum(O, shared):
    code = O.Code(520, 1040, bg=2, z=52)
    T = 6
    nw = code.learned_num_weights(T, shared)
    alpha, beta = np.full(nw, 0.75), np.zeros(nw)
    llr, cw = frames(O, code, 6, 0.5)
    _, post, _ = code.learned(T, shared, alpha, beta, llr, cw, want_post=True)
    code.set_decoder(O.RULE_NMS, 0.75, True, T)
    compared = 0
    for f in range(6):
        _, it, _, ref = code.decode(llr[f], "f64", want_post=True)
        if it == T:  # no early stop: the same T iterations
            assert np.array_equal(post[f], ref)
            compared += 1
    assert compared >= 3


@pytest.mark.parametrize("shared,multi,info_only", [(False, 0, False), (True, 0, False), (False, 1, False),
                                                     (True, 2, False), (True, 1, True), (False, 0, True)])
def test_gradients_match_finite_differences(O, shared, multi, info_only):
    code = O.Code(40, 80, bg=2, z=4)  # a small lifted code
    T = 4
    nw = code.learned_num_weights(T, shared)
    rng = np.random.default_rng(5)
    alpha = 0.75 + 0.1 * rng.standard_normal(nw)
    beta = 0.05 * np.abs(rng.standard_normal(nw))
    llr, cw = frames(O, code, 3, 1.0)
    loss, _, (ga, gb) = code.learned(T, shared, alpha, beta, llr, cw, want_grad=True, multi=multi, info_only=info_only)
    h = 1e-6
    idx = rng.choice(nw, 12, replace=False)
    for i in idx:
        for w, g in ((alpha, ga), (beta, gb)):
            w0 = w[i]
            w[i] = w0 + h
            lp, _, _ = code.learned(T, shared, alpha, beta, llr, cw, multi=multi, info_only=info_only)
            w[i] = w0 - h
            lm, _, _ = code.learned(T, shared, alpha, beta, llr, cw, multi=multi, info_only=info_only)
            w[i] = w0
            fd = (lp - lm) / (2 * h)
            assert abs(fd - g[i]) <= 1e-6 + 1e-4 * abs(fd), (i, fd, g[i])
    assert np.abs(ga).max() > 0 and np.abs(gb).max() > 0
