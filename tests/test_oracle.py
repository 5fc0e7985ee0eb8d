"""The CPU oracle pinned to the reference's own known answers and golden vectors."""

import json
import os

import numpy as np
import pytest

from conftest import GOLDEN, sionna_vectors


def test_rng_known_answers(O):
    # crates/com-core/src/rng.rs:300-305
    assert O.rng_first(0) == 0x99EC5F36CB75F2B4
    assert O.fnv1a64("a") == 0xAF63DC4C8601EC8C


def test_streams_are_independent_and_reproducible(O):
    # rng.rs:27-36: two trials of a condition get different streams; a stream repeats
    h = O.fnv1a64("ber")
    a = O.stream_draws(1, h, 3, 0, 4)
    b = O.stream_draws(1, h, 3, 1, 4)
    assert not np.array_equal(a, b)
    assert np.array_equal(a, O.stream_draws(1, h, 3, 0, 4))


def test_base_graph_dimensions(O):
    # crates/com-fec/src/nr/ldpc.rs:249-262 (through the lifted code at Z = 2)
    for bg, rows, cols_k, nnz in ((1, 46, 22, 316), (2, 42, 10, 197)):
        code = O.Code(cols_k * 2, cols_k * 2 * 3, bg=bg, z=2)
        assert code.n_rows == rows * 2 and code.edges == nnz * 2
        assert code.n_full == (cols_k + rows) * 2


def test_every_small_lifting_size_encodes_codewords(O):
    # nr/ldpc.rs:265-282: every lifting size <= 64, both base graphs
    sets = [[2, 4, 8, 16, 32, 64], [3, 6, 12, 24, 48], [5, 10, 20, 40], [7, 14, 28, 56], [9, 18, 36],
            [11, 22, 44], [13, 26, 52], [15, 30, 60]]
    for s in sets:
        for z in s:
            for bg, kb in ((1, 22), (2, 10)):
                k_info = kb * z - 3
                code = O.Code(k_info, 3 * k_info, bg=bg)
                info = np.array([(i * 7 + z) % 5 < 2 for i in range(k_info)], np.uint8)
                u = np.zeros(code.k, np.uint8)
                u[:k_info] = info
                assert code.is_codeword(code.encode_full(u))
                assert len(code.encode(info)) == 3 * k_info


def test_rate_matching_is_the_index_formula(O):
    # nr/ldpc.rs:287-330: the bit interleaver by its index formula
    for k_info, e, rv, qm in ((100, 300, 0, 1), (500, 1200, 2, 4), (1000, 1500, 3, 6), (60, 1000, 1, 2)):
        code = O.Code(k_info, e, rv=rv, qm=qm)
        z, k, ncb = code.z, code.k, code.n_full - 2 * code.z
        num, den = {(0,): (0, 1)}.get((rv,), None) or {
            (1, 1): (17, 66), (1, 2): (33, 66), (1, 3): (56, 66), (2, 1): (13, 50), (2, 2): (25, 50),
            (2, 3): (43, 50)}[(code.bg, rv)]
        k0 = num * ncb // (den * z) * z
        sel, j = [], 0
        while len(sel) < e:
            col = 2 * z + (k0 + j) % ncb
            if not (k_info <= col < k):
                sel.append(col)
            j += 1
        want = [sel[(t % qm) * (e // qm) + t // qm] for t in range(e)]
        assert list(code.bit_map()) == want


@pytest.mark.parametrize("idx", range(28))
def test_sionna_nr_ldpc_vectors(O, idx):
    # tests/test_sionna_vectors.py:104-115 of com-rs: encode == c; decode(4 - 8c) == u
    vec, pairs = sionna_vectors()
    k, n = pairs[idx]
    u, c = vec[f"ldpc.k{k}_n{n}.u"], vec[f"ldpc.k{k}_n{n}.c"]
    code = O.Code(k, n).set_decoder(O.RULE_SUM_PRODUCT, 0.8, True, 50)
    for i in range(len(u)):
        assert np.array_equal(code.encode(u[i]), c[i])
    if k <= 1024:
        bits, it, _, _ = code.decode(4.0 - 8.0 * c[0].astype(np.float64))
        assert np.array_equal(bits, u[0])


def test_layered_converges_no_slower_than_flooding(O):
    # crates/com-fec/src/ldpc.rs:997-1020 (on an NR code instead of a PEG code)
    code = O.Code(520, 1040, bg=2, z=52)
    info, llr, _ = code.trial(4, 5, O.fnv1a64("x"), 0, 0, 2.0)
    its = []
    for layered in (False, True):
        code.set_decoder(O.RULE_SUM_PRODUCT, 0.8, layered, 50)
        bits, it, _, _ = code.decode(llr)
        assert np.array_equal(bits, info)
        its.append(it)
    assert its[1] <= its[0]


def test_qam_is_gray_and_unit_energy(O):
    for m in (4, 16, 64, 256):
        pts, _ = O.qam(m)
        assert abs(np.mean(np.abs(pts) ** 2) - 1.0) < 1e-12
        # Gray: nearest neighbours differ in one bit
        d = np.abs(pts[:, None] - pts[None, :])
        dmin = d[d > 1e-9].min()
        for i in range(m):
            for j in range(m):
                if abs(d[i, j] - dmin) < 1e-9:
                    assert bin(i ^ j).count("1") == 1
    pts, _ = O.qam(4)
    s = 1 / np.sqrt(2)
    assert np.allclose(pts, [(-1 + 1j) * s, (1 + 1j) * s, (-1 - 1j) * s, (1 - 1j) * s])


def test_qam_label_bits_split_by_dimension(O):
    # the premise of the GPU's f64 max-log demapper (half minima per dimension): in the
    # reference's Gray square QAM the last log2(side) label bits fix the real part and the
    # first log2(side) bits the imaginary part, the same doubles for every such label
    for m in (4, 16, 64, 256):
        pts, _ = O.qam(m)
        side = int(round(np.sqrt(m)))
        lab = np.arange(m)
        re, im = pts.real.view(np.uint64), pts.imag.view(np.uint64)
        for low in range(side):
            assert len(set(re[(lab % side) == low].tolist())) == 1
        for high in range(side):
            assert len(set(im[(lab // side) == high].tolist())) == 1
        assert len(set(re.tolist())) == side and len(set(im.tolist())) == side


def test_demapper_max_log_matches_brute_force(O):
    rng = np.random.default_rng(1)
    for m in (4, 16, 64):
        pts, lm = O.qam(m)
        y = rng.normal(size=50) + 1j * rng.normal(size=50)
        got = O.demap_maxlog(m, y, 0.3).reshape(50, -1)
        b = m.bit_length() - 1
        for s in range(50):
            met = -np.abs(y[s] - pts) ** 2 / 0.3 - lm
            for o in range(b):
                sh = b - 1 - o
                bit = (np.arange(m) >> sh) & 1
                assert abs(got[s, o] - (met[bit == 0].max() - met[bit == 1].max())) < 1e-12


def test_noise_libm_and_correct_rounding_rarely_differ(O):
    # the reference's noise uses the platform libm; the oracle's correctly-rounded mode
    # differs from glibc in the last bit only, and rarely
    n = 200_000
    a = O.complex_gaussians(99, n, O.NOISE_LIBM)
    b = O.complex_gaussians(99, n, O.NOISE_CR)
    diff = (a[0] != b[0]) | (a[1] != b[1])
    assert diff.mean() < 0.01
    rel = np.abs(a[0] - b[0]) / np.maximum(np.abs(b[0]), 1e-300)
    assert rel.max() < 4.5e-16


def test_libm_and_cr_frames_count_alike(O):
    code = O.Code(520, 1040, bg=2, z=52).set_decoder(O.RULE_NMS, 0.75, True, 20)
    h = O.fnv1a64("bicm_ldpc")
    a = code.run_frames(4, 7, h, 2, 0, 300, 1.5, 0, O.NOISE_LIBM, 0)
    b = code.run_frames(4, 7, h, 2, 0, 300, 1.5, 0, O.NOISE_CR, 0)
    differ = (a["bit_errors"] != b["bit_errors"]) | (a["iterations"] != b["iterations"])
    assert differ.sum() <= 3


def test_aff3ct_layered_nms_curve(O):
    # validation/tests/aff3ct.rs:222-224, :265-338: PEG(576, 288), layered NMS 0.75, 20
    # iterations, BPSK; FER intervals overlap AFF3CT's at 99 % (quick statistics)
    from importlib import import_module

    fx = json.load(open(os.path.join(GOLDEN, "ldpc_peg_n576_k288_layered_nms075_i20.json")))
    code = O.Code(alist=open(os.path.join(GOLDEN, "peg_n576_k288.alist")).read())
    code.set_decoder(O.RULE_NMS, 0.75, True, 20)
    assert (code.n_full, code.k) == (576, 288)
    campaign = import_module("com-rs_gb300.campaign")
    name = "ldpc_peg_n576_k288_layered_nms075_i20"
    seed = O.fnv1a64(name)
    rate = 288 / 576
    checked = 0
    for idx, p in enumerate(fx["data"]):
        if p["fer"] < 0.02:
            continue
        noise_var = 1.0 / (2.0 * rate * 10 ** (p["ebn0_db"] / 10))  # bpsk_noise_variance
        fe = n = 0
        while fe < 60 and n < 4000:
            be, _ = code.bpsk_frame(seed, O.fnv1a64(name), idx, n, noise_var)
            fe += be > 0
            n += 1
        ours = campaign.ErrorRate(fe, n)
        theirs = campaign.ErrorRate(p["frame_errors"], p["frames"])
        (a_lo, a_hi), (c_lo, c_hi) = theirs.wilson(0.99), ours.wilson(0.99)
        assert not (a_hi < c_lo or c_hi < a_lo), (p["ebn0_db"], ours.rate(), theirs.rate())
        checked += 1
    assert checked >= 4


@pytest.mark.parametrize("m", [4, 16, 64, 256])
def test_exact_demapper_is_the_log_sum_exp_of_the_label_halves(O, m):
    # Jacobian::Exact (crates/com-mapping/src/demapper.rs:82-133) against an independent
    # log-sum-exp over the two halves of the labels, MSB first
    pts, log_m = O.qam(m)
    rng = np.random.default_rng(m)
    y = pts[rng.integers(0, m, 200)] + 0.3 * (rng.standard_normal(200) + 1j * rng.standard_normal(200))
    sigma2 = 0.18
    got = O.demap_exact(m, y, sigma2).reshape(200, -1)
    b = m.bit_length() - 1
    metric = -np.abs(y[:, None] - pts[None, :]) ** 2 / sigma2 - log_m
    labels = np.arange(m)
    for o in range(b):
        half = (labels >> (b - 1 - o)) & 1
        want = np.logaddexp.reduce(metric[:, half == 0], axis=1) - np.logaddexp.reduce(metric[:, half == 1], axis=1)
        assert np.allclose(got[:, o], want, rtol=1e-12, atol=1e-12)
    # max-log keeps the largest term only: the exact LLR is smaller in magnitude near
    # the decision boundary and equal in sign far from it; QPSK has one point per half
    ml = O.demap_maxlog(m, y, sigma2).reshape(200, -1)
    if m == 4:
        assert np.allclose(got, ml, rtol=1e-13, atol=1e-13)
    else:
        assert not np.allclose(got, ml)


def test_counts_do_not_depend_on_the_thread_count(O):
    # every frame draws from its own stream (runner.rs:435-447), so the records are the
    # same whatever the number of worker threads
    code = O.Code(520, 1040, 2, 52).set_decoder(O.RULE_NMS, 0.75, True, 20)
    h = O.fnv1a64("bicm_ldpc")
    one = code.run_frames(4, 7, h, 2, 100, 64, 1.0, 0, O.NOISE_CR, 1)
    many = code.run_frames(4, 7, h, 2, 100, 64, 1.0, 0, O.NOISE_CR, 4)
    assert np.array_equal(one, many)
    peg = O.Code(alist=open(os.path.join(GOLDEN, "peg_n576_k288.alist")).read())
    peg.set_decoder(O.RULE_NMS, 0.75, True, 20)
    a, _, _ = peg.link_trials(2, 0, 16, 6, h, 0, 0, 24, 3.0, threads=1)
    b, _, _ = peg.link_trials(2, 0, 16, 6, h, 0, 0, 24, 3.0, threads=4)
    assert np.array_equal(a, b)
