"""Generic sparse codes on the GPU (cb_ldpc_*) against the oracle's LdpcCode and
against AFF3CT's recorded curves.

* min-sum rules (normalised, offset; layered, flooding): posteriors equal the oracle's
  bit for bit, f64 and f32, iterations equal;
* sum-product: the oracle calls the platform libm's tanh/atanh, the GPU CUDA's, so the
  comparison is statistical per frame (same decoding outcome, same iterations) and by
  tolerance on the posteriors of frames that converge early;
* the four LDPC fixtures of validation/tests/aff3ct.rs:219-230 (PEG(576, 288) and
  PEG(648, 540); BPSK, sigma^2 = 1 / (2 R Eb/N0)): frame error rates whose 99 % Wilson
  intervals overlap AFF3CT's;
* the generic decoder on the lifted rows of an NR code equals the NR decoder;
* the encoders (from_rows' GF(2) sums, accumulate) equal the oracle's codewords, and
  set_decoder gives the decoder a fresh code with the same settings has.
"""

import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
EBN0 = {"peg_n576_k288.alist": (1.5, 2.5), "peg_n648_k540.alist": (3.5, 4.5)}


def _codes(cb, O, matrix, rule, alpha, layered, iters, precision):
    text = open(os.path.join(GOLDEN, matrix)).read()
    ref = O.Code(alist=text)
    ref.set_decoder({"sum_product": O.RULE_SUM_PRODUCT, "normalized_min_sum": O.RULE_NMS,
                     "offset_min_sum": O.RULE_OMS}[rule], alpha, layered, iters)
    n, rows = cb.parse_alist(text)
    gpu = cb.Ldpc(n, rows, rule=rule, alpha=alpha, layered=layered, max_iterations=iters, precision=precision)
    return ref, gpu


def _frames(O, ref, ebn0, first, n, seed=5):
    rate = ref.k / ref.n_full
    noise_var = 1.0 / (2.0 * rate * 10 ** (ebn0 / 10))
    return ref.bpsk_llr(seed, O.fnv1a64("sparse"), int(ebn0 * 100), first, n, noise_var)


@pytest.mark.parametrize("precision", ["f64", "f32"])
@pytest.mark.parametrize("rule, alpha, layered", [("normalized_min_sum", 0.75, True), ("offset_min_sum", 0.15, False),
                                                  ("normalized_min_sum", 0.8, False), ("offset_min_sum", 0.5, True)])
@pytest.mark.parametrize("matrix", ["peg_n576_k288.alist", "peg_n648_k540.alist"])
def test_min_sum_equals_the_oracle_bit_for_bit(cb, O, matrix, rule, alpha, layered, precision):
    ref, gpu = _codes(cb, O, matrix, rule, alpha, layered, 20, precision)
    dt, it_all = (np.float64, np.uint64) if precision == "f64" else (np.float32, np.uint32), []
    for ebn0 in EBN0[matrix]:
        _, llr = _frames(O, ref, ebn0, 0, 200)
        post_g, it_g = gpu.decode_llr(llr)
        post_o, it_o = ref.decode_llr_many(llr, precision)
        assert np.array_equal(it_g, it_o), ebn0
        assert np.array_equal(post_g.view(dt[1]), post_o.view(dt[1])), ebn0
        it_all.append(it_g)
    it_all = np.concatenate(it_all)
    assert (it_all == 20).any() and (it_all < 20).any() and len(set(it_all.tolist())) > 4


@pytest.mark.parametrize("layered, iters", [(True, 20), (False, 50)])
def test_sum_product_agrees_with_the_oracle(cb, O, layered, iters):
    matrix = "peg_n576_k288.alist"
    ref, gpu = _codes(cb, O, matrix, "sum_product", 0.0, layered, iters, "f64")
    total = same_outcome = same_it = 0
    worst_early = 0.0
    for ebn0 in (1.0, 1.75, 2.5):
        cw, llr = _frames(O, ref, ebn0, 0, 300)
        post_g, it_g = gpu.decode_llr(llr)
        post_o, it_o = ref.decode_llr_many(llr, "f64")
        ok_g = ((post_g < 0) == cw.astype(bool)).all(axis=1)
        ok_o = ((post_o < 0) == cw.astype(bool)).all(axis=1)
        total += len(cw)
        same_outcome += int((ok_g == ok_o).sum())
        same_it += int((it_g == it_o).sum())
        early = (it_g == it_o) & (it_o <= 5)
        if early.any():
            rel = np.abs(post_g[early] - post_o[early]) / np.maximum(1.0, np.abs(post_o[early]))
            worst_early = max(worst_early, float(rel.max()))
    print(f"sum-product layered={layered}: {same_outcome}/{total} same outcome, {same_it}/{total} same "
          f"iterations, worst relative posterior gap (<= 5 iterations) {worst_early:.3g}")
    assert same_outcome >= 0.99 * total
    assert same_it >= 0.97 * total
    assert worst_early <= 1e-9


def _wilson(k, n, z=2.5758293035489004):
    p = k / n
    d = 1 + z * z / n
    c = (p + z * z / (2 * n)) / d
    h = z * np.sqrt(p * (1 - p) / n + z * z / (4 * n * n)) / d
    return c - h, c + h


@pytest.mark.parametrize("name, matrix, rule, alpha, layered, iters", [
    ("ldpc_peg_n576_k288_layered_nms075_i20", "peg_n576_k288.alist", "normalized_min_sum", 0.75, True, 20),
    ("ldpc_peg_n576_k288_flooding_oms015_i20", "peg_n576_k288.alist", "offset_min_sum", 0.15, False, 20),
    ("ldpc_peg_n576_k288_flooding_spa_i50", "peg_n576_k288.alist", "sum_product", 0.0, False, 50),
    ("ldpc_peg_n648_k540_layered_spa_i20", "peg_n648_k540.alist", "sum_product", 0.0, True, 20),
])
def test_frame_error_rates_overlap_aff3ct(cb, O, name, matrix, rule, alpha, layered, iters):
    fx = json.load(open(os.path.join(GOLDEN, name + ".json")))
    ref, gpu = _codes(cb, O, matrix, rule, alpha, layered, iters, "f64")
    num, den = fx["bit_rate"]
    rate = num / den
    checked = 0
    for idx, p in enumerate(fx["data"]):
        if p["fer"] < 2e-3:
            continue
        noise_var = 1.0 / (2.0 * rate * 10 ** (p["ebn0_db"] / 10))
        fe = nf = 0
        while fe < 200 and nf < 200_000:
            cw, llr = ref.bpsk_llr(O.fnv1a64(name), O.fnv1a64(name), idx, nf, 20_000, noise_var)
            post, _ = gpu.decode_llr(llr)
            fe += int((((post < 0) != cw.astype(bool)).sum(axis=1) > 0).sum())
            nf += len(cw)
        a_lo, a_hi = _wilson(p["frame_errors"], p["frames"])
        c_lo, c_hi = _wilson(fe, nf)
        assert not (a_hi < c_lo or c_hi < a_lo), (p["ebn0_db"], fe / nf, p["fer"])
        checked += 1
    assert checked >= 4


def test_nr_rows_through_the_generic_decoder_equal_the_nr_decoder(cb, O):
    # C1: BG2 Z = 52, K' = 520, E = 1040; no filler bits, so the full word is 2Z zeros,
    # the E LLRs, then zeros for the unsent parity bits
    nr = cb.NrLdpc(520, 1040, base_graph=2, lifting_size=52, precision="f64", max_iterations=20)
    ref = O.Code(520, 1040, 2, 52)
    assert (ref.n_full, ref.k) == (2704, 520)
    r, v = ref.edges_list()
    rows = [[] for _ in range(int(r.max()) + 1)]
    for a, b in zip(r.tolist(), v.tolist()):
        rows[a].append(b)
    gpu = cb.Ldpc(ref.n_full, rows, rule="normalized_min_sum", alpha=0.75, layered=True, max_iterations=20)
    rng = np.random.default_rng(3)
    for ebn0 in (1.0, 2.0):
        cw = rng.integers(0, 2, (64, 520), dtype=np.uint8)
        sent = nr.encode(cw)
        sigma2 = 1.0 / (2 * 0.5 * 10 ** (ebn0 / 10))
        llr = 2 * (1 - 2.0 * sent + np.sqrt(sigma2) * rng.standard_normal(sent.shape)) / sigma2
        full = np.zeros((64, ref.n_full))
        full[:, 104:104 + 1040] = llr
        post, it = gpu.decode_llr(full)
        bits, app, it_nr = nr.decode_full(llr)
        assert np.array_equal(it, it_nr)
        assert np.array_equal(post[:, :520].view(np.uint64), app.view(np.uint64))


@pytest.mark.parametrize("precision", ["f64", "f32"])
@pytest.mark.parametrize("layered", [True, False])
def test_min_sum_signed_zeros_and_extremes_equal_the_oracle(cb, O, layered, precision):
    # channel LLRs of +0.0 and -0.0 (`l < 0` is false for both, though -0.0 has the sign
    # bit) and of huge magnitudes, finite in the precision: posteriors and iterations
    # equal the oracle's bit for bit
    ref, gpu = _codes(cb, O, "peg_n576_k288.alist", "normalized_min_sum", 0.75, layered, 20, precision)
    _, llr = _frames(O, ref, 1.5, 0, 64)
    llr = llr.copy()
    u = np.random.default_rng(3).random(llr.shape)
    llr[u < 0.05] = 0.0
    llr[(u >= 0.05) & (u < 0.10)] = -0.0
    big = (u >= 0.10) & (u < 0.12)
    llr[big] *= 1e250 if precision == "f64" else 1e30
    dt = np.uint64 if precision == "f64" else np.uint32
    post_g, it_g = gpu.decode_llr(llr)
    post_o, it_o = ref.decode_llr_many(llr, precision)
    assert np.array_equal(it_g, it_o)
    assert np.array_equal(post_g.view(dt), post_o.view(dt))


def test_edge_cases(cb):
    from test_sparse_host import HAMMING

    n, rows = cb.parse_alist(HAMMING)
    code = cb.Ldpc(n, rows, rule="normalized_min_sum", alpha=0.75, max_iterations=0)
    x = np.array([1.0, -2.0, 3.0, 0.5, -0.25, 4.0, 2.0])
    post, it = code.decode_llr(x)
    # zero iterations: the channel LLRs come back as they are
    assert np.array_equal(post, x) and it == 0
    code.close()
    code = cb.Ldpc(n, rows, rule="min_sum", max_iterations=10)
    post, it = code.decode_llr(np.full(7, 2.0))  # the all-zero word is a codeword
    assert it == 0 and np.array_equal(post, np.full(7, 2.0))
    post, its = code.decode_llr(np.zeros((0, 7)))
    assert post.shape == (0, 7) and its.shape == (0,)


def test_dvbs2_short_rate_half_overlaps_aff3ct(cb):
    # validation/tests/aff3ct.rs:231-233: the LDPC code of the short FECFRAME of rate 1/2,
    # layered sum-product, 50 iterations; BPSK over AWGN at sigma^2 = 1 / (2 R Eb/N0), R =
    # 4/9.  All-zero codewords (the decoders are symmetric, so the frame error rate does
    # not depend on the codeword).  By default the points with FER >= 0.1 on 1024 frames
    # each; COMRS_GB300_FULL=1 runs every point to 200 frame errors or 12 288 frames.
    full = os.environ.get("COMRS_GB300_FULL") == "1"
    fx = json.load(open(os.path.join(GOLDEN, "ldpc_dvbs2_short_r1_2_layered_spa_i50.json")))
    code = cb.Dvbs2Ldpc("short", "1/2", max_iterations=50)
    num, den = fx["bit_rate"]
    rate = num / den
    rng = np.random.default_rng(11)
    checked = 0
    points = fx["data"] if full else [p for p in fx["data"] if p["fer"] >= 0.1]
    for p in points:
        noise_var = 1.0 / (2.0 * rate * 10 ** (p["ebn0_db"] / 10))
        fe = nf = 0
        while fe < 200 and nf < (12_288 if full else 1024):
            y = 1.0 + np.sqrt(noise_var) * rng.standard_normal((1024, 16200))
            post, _ = code.decode_llr(2.0 * y / noise_var)
            fe += int((post < 0).any(axis=1).sum())
            nf += 1024
        a_lo, a_hi = _wilson(p["frame_errors"], p["frames"])
        c_lo, c_hi = _wilson(fe, nf)
        assert not (a_hi < c_lo or c_hi < a_lo), (p["ebn0_db"], fe / nf, p["fer"])
        checked += 1
    assert checked == (5 if full else 3)


@pytest.mark.parametrize("rule", ["normalized_min_sum", "sum_product"])
def test_dvbs2_normal_frame_decodes_with_posteriors_in_global_memory(cb, rule):
    # n = 64 800: the f64 posteriors (518 KB) exceed shared memory and live in the CTAs'
    # global slots with the messages.  Above the decoding threshold every all-zero frame
    # decodes, in more than one iteration, and a second run gives the same posteriors.
    code = cb.Dvbs2Ldpc("normal", "1/2", rule=rule, alpha=0.75, max_iterations=30)
    assert code.info()["n"] == 64800
    rng = np.random.default_rng(5)
    rate = 0.5
    # above the threshold of each rule (the normalised min-sum needs about 0.2 dB more,
    # fec.rs:262-263)
    ebn0 = 1.6 if rule == "sum_product" else 2.3
    noise_var = 1.0 / (2.0 * rate * 10 ** (ebn0 / 10))
    y = 1.0 + np.sqrt(noise_var) * rng.standard_normal((8, 64800))
    llr = 2.0 * y / noise_var
    post, its = code.decode_llr(llr)
    assert (post > 0).all() and (its < 30).all() and (its > 1).all()
    post2, its2 = code.decode_llr(llr)
    assert np.array_equal(post.view(np.uint64), post2.view(np.uint64)) and np.array_equal(its, its2)


# ---------------------------------------------------------------- encoders

def _encoder_case(cb, kind):
    """(GPU code, oracle rows, n, accumulate) of a named case."""
    from test_sparse_host import HAMMING

    if kind.startswith("peg"):
        n, k = {"peg576": (576, 288), "peg648": (648, 540)}[kind]
        return n, cb.ldpc.peg_rows(n, k), False
    if kind == "hamming":
        n, rows = cb.parse_alist(HAMMING)
        return n, rows, False
    if kind == "rank_deficient":
        rng = np.random.default_rng(4)
        rows = [sorted(rng.choice(120, size=7, replace=False).tolist()) for _ in range(50)]
        return 120, rows + rows[:6] + [sorted(set(rows[0]) ^ set(rows[1]))], False
    frame, rate = {"dvbs2_short_1_2": ("short", "1/2"), "dvbs2_normal_1_4": ("normal", "1/4")}[kind]
    n, _, rows = cb.dvbs2.ldpc_rows(frame, rate)
    return n, rows, True


@pytest.mark.parametrize("kind, frames", [("peg576", 5000), ("peg648", 300), ("hamming", 64),
                                          ("rank_deficient", 200), ("dvbs2_short_1_2", 96),
                                          ("dvbs2_normal_1_4", 24)])
def test_encode_equals_the_oracle(cb, O, kind, frames):
    # LdpcCode::encode_block (ldpc.rs:753-791): Encoder::Sums of from_rows, or
    # Encoder::Accumulate of the DVB-S2 codes; 5000 frames run the grid-stride loop
    n, rows, acc = _encoder_case(cb, kind)
    code = cb.Ldpc.accumulate(n, rows) if acc else cb.Ldpc(n, rows)
    ref = O.Code(rows=rows, n=n, accumulate=acc)
    assert code.k == ref.k
    rng = np.random.default_rng(len(kind) * 1000 + frames)
    u = rng.integers(0, 2, (frames, code.k), dtype=np.uint8)
    # only bit 0 of every byte counts (c[p] = b & 1)
    noisy = u | (rng.integers(0, 128, u.shape, dtype=np.uint8) << 1).astype(np.uint8)
    c = code.encode(noisy)
    check = range(frames) if frames <= 300 else rng.choice(frames, 300, replace=False)
    for f in check:
        want = ref.encode_full(u[f])
        assert np.array_equal(c[f], want), f
        assert ref.is_codeword(c[f]), f
    assert np.array_equal(c[:, code.info_positions()], u)
    assert np.array_equal(code.encode(u.reshape(-1)), c.reshape(-1))
    assert code.encode(np.zeros((0, code.k), np.uint8)).shape == (0, n)


def test_encode_on_device_buffers(cb):
    import ctypes as C

    torch = pytest.importorskip("torch")
    code = cb.Ldpc.peg(576, 288)
    rng = np.random.default_rng(8)
    u = rng.integers(0, 2, (700, 288), dtype=np.uint8)
    want = code.encode(u)
    u_d = torch.from_numpy(u).cuda()
    c_d = torch.full((700, 576), 7, dtype=torch.uint8, device="cuda")
    s = torch.cuda.current_stream()
    st = cb.lib().cb_ldpc_encode_device(code._h, C.c_void_p(u_d.data_ptr()), 700, C.c_void_p(c_d.data_ptr()),
                                        C.c_void_p(s.cuda_stream))
    assert st == 0
    s.synchronize()
    assert np.array_equal(c_d.cpu().numpy(), want)


def test_encode_decode_round_trip(cb):
    # bindings/com-py/src/fec/ldpc_code.rs:150-156: decode(2 - 4 encode(b)) == b with the
    # default decoder (layered sum-product, 50 iterations)
    code = cb.Ldpc.peg(96, 48)
    b = np.random.default_rng(1).integers(0, 2, 48 * 10, dtype=np.uint8)
    c = code.encode(b)
    assert c.size == 960
    assert np.array_equal(code.decode(2.0 - 4.0 * c), b)
    assert np.array_equal(code.decode((2.0 - 4.0 * c).reshape(10, 96)), b.reshape(10, 48))


def test_set_decoder_equals_a_fresh_code(cb, O):
    # a code whose decoder is changed decodes as a code built with the new settings
    text = open(os.path.join(GOLDEN, "peg_n576_k288.alist")).read()
    n, rows = cb.parse_alist(text)
    ref = O.Code(alist=text)
    _, llr = _frames(O, ref, 2.0, 0, 128)
    code = cb.Ldpc(n, rows, rule="normalized_min_sum", alpha=0.75, max_iterations=20)
    code.decode_llr(llr)
    for rule, alpha, layered, iters in (("offset_min_sum", 0.15, False, 20), ("normalized_min_sum", 0.8, True, 7),
                                        ("sum_product", 0.0, True, 30), ("min_sum", 0.3, False, 12)):
        code.set_decoder(rule, alpha=alpha, layered=layered, max_iterations=iters)
        post, its = code.decode_llr(llr)
        fresh = cb.Ldpc(n, rows, rule=rule, alpha=alpha, layered=layered, max_iterations=iters)
        post_f, its_f = fresh.decode_llr(llr)
        assert np.array_equal(post.view(np.uint64), post_f.view(np.uint64)), rule
        assert np.array_equal(its, its_f), rule


@pytest.mark.parametrize("precision", ["f64", "f32"])
@pytest.mark.parametrize("rule, alpha", [("normalized_min_sum", 0.75), ("offset_min_sum", 0.3)])
def test_dense_rows_take_the_warp_path_and_equal_the_oracle(cb, O, rule, alpha, precision):
    # dense random rows (20 to 60 of 120 variables): levels of at most 8 rows, so one warp
    # decodes each row with shuffle reductions of the minimum, its first index, the second
    # minimum and the sign parity; signed zeros among the LLRs; min-sum bit for bit
    rng = np.random.default_rng(11)
    n, m = 120, 40
    rows = [sorted(rng.choice(n, size=int(rng.integers(20, 61)), replace=False).tolist()) for _ in range(m)]
    gpu = cb.Ldpc(n, rows, rule=rule, alpha=alpha, max_iterations=12, precision=precision, encoder=None)
    assert gpu.info()["max_level_rows"] <= 8 and gpu.info()["max_row_degree"] <= 128
    ref = O.Code(rows=rows, n=n)
    ref.set_decoder({"normalized_min_sum": O.RULE_NMS, "offset_min_sum": O.RULE_OMS}[rule], alpha, True, 12)
    llr = rng.normal(4.0, 2.0, (128, n))  # about half the frames stop early
    llr[:, :4] = 0.0
    llr[:40, 4:8] = -0.0
    dt = np.uint64 if precision == "f64" else np.uint32
    post_g, it_g = gpu.decode_llr(llr)
    post_o, it_o = ref.decode_llr_many(llr, precision)
    assert np.array_equal(it_g, it_o)
    assert np.array_equal(post_g.view(dt), post_o.view(dt))
    assert (it_g < 12).any() and (it_g == 12).any()


@pytest.mark.parametrize("n, m, dmax, seed", [(300, 150, 6, 1), (1200, 900, 5, 2), (2000, 600, 14, 3),
                                              (4000, 2000, 8, 4)])
def test_random_codes_equal_the_oracle(cb, O, n, m, dmax, seed):
    # random rows (degree 2..dmax): levels of many rows (several codewords per CTA when
    # they fit), rows longer than the register sum-product's 8 edges, messages in shared
    # or global memory; min-sum bit for bit, sum-product by outcome
    rng = np.random.default_rng(seed)
    rows = [sorted(rng.choice(n, size=int(rng.integers(2, dmax + 1)), replace=False).tolist()) for _ in range(m)]
    start = [0]
    for r in rows:
        start.append(start[-1] + len(r))
    llr = rng.normal(2.0, 2.5, (96, n))
    for precision, dt in (("f64", np.uint64), ("f32", np.uint32)):
        gpu = cb.Ldpc(n, rows, rule="normalized_min_sum", alpha=0.75, max_iterations=15, precision=precision,
                      encoder=None)
        ref = O.Code(rows=rows, n=n)
        ref.set_decoder(O.RULE_NMS, 0.75, True, 15)
        post_g, it_g = gpu.decode_llr(llr)
        post_o, it_o = ref.decode_llr_many(llr, precision)
        assert np.array_equal(it_g, it_o), precision
        assert np.array_equal(post_g.view(dt), post_o.view(dt)), precision
    gpu = cb.Ldpc(n, rows, rule="sum_product", max_iterations=15, encoder=None)
    ref.set_decoder(O.RULE_SUM_PRODUCT, 0.0, True, 15)
    post_g, it_g = gpu.decode_llr(llr)
    post_o, it_o = ref.decode_llr_many(llr, "f64")
    assert ((post_g < 0) == (post_o < 0)).all(axis=1).mean() >= 0.95 and (it_g == it_o).mean() >= 0.9
