"""GPU Monte Carlo trial parity: frames regenerated on the device from their streams.

f64: the E channel LLRs and the K' info bits of every frame are bit-identical to the
oracle's (correctly-rounded noise mode), and so are the per-frame bit errors, frame
errors and iteration counts.  f32: same bits, noise in f32, statistically equal FER;
on the timed configuration (BG1 Z = 384, 16-QAM) the f32 trial is compared with the
oracle's f64 trial with the platform libm's noise at the waterfall and on the bench grid.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NAME = "bicm_ldpc"

CODES = [
    dict(k=520, e=1040, bg=2, z=52, m=4),           # benchmark config 1
    dict(k=100, e=302, m=16),                       # 2 padding bits, fillers
    dict(k=500, e=1200, rv=2, qm=4, m=64),
    dict(k=1000, e=1504, m=256),
    dict(k=8448, e=25344, bg=1, z=384, m=16),       # benchmark config 2
    dict(k=8448, e=16896, bg=1, z=384, m=64),       # benchmark config 5
    dict(k=60, e=1000, rv=1, qm=2, m=4),            # repeated bits (E > N_cb)
    dict(k=1000, e=1500, rv=3, qm=6, m=64),         # rv 3, bit interleaver of 6 rows
    dict(k=1000, e=1502, m=64),                     # 4 padding bits: a last symbol of 2 LLRs
    dict(k=700, e=1500, m=256),                     # 4 padding bits: a last symbol of 4 LLRs
]


def codes(cb, O, spec, precision="f64"):
    g = cb.NrLdpc(spec["k"], spec["e"], base_graph=spec.get("bg"), lifting_size=spec.get("z"),
                  rv=spec.get("rv", 0), qm=spec.get("qm", 1), precision=precision)
    r = O.Code(spec["k"], spec["e"], bg=spec.get("bg", 0), z=spec.get("z", 0), rv=spec.get("rv", 0),
               qm=spec.get("qm", 1)).set_decoder(O.RULE_NMS, 0.75, True, 20)
    return g, r


@pytest.mark.parametrize("spec", CODES, ids=lambda s: f"k{s['k']}_e{s['e']}_m{s['m']}")
def test_f64_frames_are_the_oracle_frames(cb, O, spec):
    g, r = codes(cb, O, spec)
    n = 3 if spec["k"] > 4000 else 12
    for cond, eb in enumerate((0.5, 2.0)):
        llr, info = g.generate_frames(7, NAME, cond, 5, n, eb, spec["m"])
        for f in range(n):
            rinfo, rllr, _ = r.trial(spec["m"], 7, O.fnv1a64(NAME), cond, 5 + f, eb, 0, O.NOISE_CR)
            assert np.array_equal(info[f], rinfo), (cond, f)
            assert np.array_equal(llr[f].view(np.uint64), rllr.view(np.uint64)), (cond, f)


@pytest.mark.parametrize("eb", [0.0, 1.0, 2.0, 3.0])
def test_f64_counts_equal_the_oracle(cb, O, eb):
    spec = CODES[0]
    g, r = codes(cb, O, spec)
    got = g.run_frames(7, NAME, 3, 0, 400, eb, 4)
    want = r.run_frames(4, 7, O.fnv1a64(NAME), 3, 0, 400, eb, 0, O.NOISE_CR, 0)
    for key in ("bit_errors", "frame_error", "iterations"):
        assert np.array_equal(got[key], want[key]), key


def test_f32_frames_draw_the_same_bits_and_close_llrs(cb, O):
    spec = CODES[4]
    g32, _ = codes(cb, O, spec, "f32")
    g64, _ = codes(cb, O, spec, "f64")
    l32, i32 = g32.generate_frames(7, NAME, 0, 0, 4, 1.0, 16)
    l64, i64 = g64.generate_frames(7, NAME, 0, 0, 4, 1.0, 16)
    assert np.array_equal(i32, i64)
    err = np.abs(l32.astype(np.float64) - l64) / np.maximum(np.abs(l64), 1.0)
    assert np.median(err) < 1e-5 and err.max() < 1e-3
    assert np.mean(np.sign(l32) == np.sign(l64)) > 0.9999


@pytest.mark.parametrize("m", [64, 256])
def test_f32_high_order_llrs_are_close_to_f64(cb, O, m):
    spec = dict(k=1000, e=1512, m=m) if m == 64 else dict(k=1000, e=1504, m=m)
    g32, _ = codes(cb, O, spec, "f32")
    g64, _ = codes(cb, O, spec, "f64")
    l32, i32 = g32.generate_frames(7, NAME, 0, 0, 8, 8.0, m)
    l64, i64 = g64.generate_frames(7, NAME, 0, 0, 8, 8.0, m)
    assert np.array_equal(i32, i64)
    err = np.abs(l32.astype(np.float64) - l64) / np.maximum(np.abs(l64), 1.0)
    assert np.median(err) < 1e-5 and np.mean(np.sign(l32) == np.sign(l64)) > 0.9999


def test_f32_fer_is_statistically_the_f64_fer(cb, O):
    from conftest import load_package

    ErrorRate = load_package().campaign.ErrorRate
    spec = CODES[0]
    g32, _ = codes(cb, O, spec, "f32")
    g64, _ = codes(cb, O, spec, "f64")
    for eb in (1.0, 1.5):
        a = g32.run_frames(7, NAME, 0, 0, 20000, eb, 4)
        b = g64.run_frames(7, NAME, 0, 0, 20000, eb, 4)
        ra = ErrorRate(int(a["frame_error"].sum()), len(a))
        rb = ErrorRate(int(b["frame_error"].sum()), len(b))
        (a0, a1), (b0, b1) = ra.wilson(0.99), rb.wilson(0.99)
        assert not (a1 < b0 or b1 < a0), (eb, ra.rate(), rb.rate())


def test_frames_do_not_depend_on_the_batching(cb, O):
    spec = CODES[0]
    g, _ = codes(cb, O, spec, "f32")
    whole = g.run_frames(7, NAME, 1, 100, 3000, 1.0, 4)
    parts = np.concatenate([g.run_frames(7, NAME, 1, 100, 1234, 1.0, 4),
                            g.run_frames(7, NAME, 1, 1334, 1766, 1.0, 4)])
    assert np.array_equal(whole, parts)
    assert np.array_equal(whole, g.run_frames(7, NAME, 1, 100, 3000, 1.0, 4))


def _overlap(a, b, confidence=0.99):
    (a0, a1), (b0, b1) = a.wilson(confidence), b.wilson(confidence)
    return not (a1 < b0 or b1 < a0)


def _paired_z(x, y):
    d = np.asarray(x, np.float64) - np.asarray(y, np.float64)
    sd = d.std(ddof=1)
    return 0.0 if sd == 0 else d.mean() / (sd / np.sqrt(len(d)))


def _ber_agrees(x, y, bits_per_frame, z=3.3):
    # The bit errors of a frame come in bursts (a failed frame has hundreds), so the bits
    # are not independent trials and a binomial interval over bits is far too narrow; the
    # frames are independent, so the BER's standard error is that of the mean per-frame
    # count.  The two BERs agree when they differ by less than z of those errors.
    x, y = np.asarray(x, np.float64), np.asarray(y, np.float64)
    se = np.hypot(x.std(ddof=1) / np.sqrt(len(x)), y.std(ddof=1) / np.sqrt(len(y)))
    return abs(x.mean() - y.mean()) <= z * se, (x.mean() / bits_per_frame, y.mean() / bits_per_frame)


# The timed configuration (benchmark config 2: BG1 Z = 384, 16-QAM, f32 generator and f32
# decoder through cb_run_frames) against the oracle's f64 trial with the platform libm's
# noise, i.e. the reference's own arithmetic (crates/com-core/src/rng.rs:161-167,
# crates/com-channel/src/awgn.rs:139-141, crates/com-fec/src/ldpc.rs:509-557).  Both draw
# every frame from the same stream, so besides the 99 % Wilson overlap of the rates
# (validation/tests/aff3ct.rs:265-338) and of the bit error rates (frame-clustered), the
# frames can be compared in pairs: most end alike, and the per-frame differences of bit
# errors and iterations centre on zero.
@pytest.mark.parametrize("eb,n,cond", [(2.6, 1024, 31), (2.7, 3072, 32)])
def test_c2_f32_trial_matches_the_oracle_at_the_waterfall(cb, O, eb, n, cond):
    from conftest import load_package

    ErrorRate = load_package().campaign.ErrorRate
    g32, r = codes(cb, O, CODES[4], "f32")
    a = g32.run_frames(7, NAME, cond, 0, n, eb, 16)
    b = r.run_frames(16, 7, O.fnv1a64(NAME), cond, 0, n, eb, 0, O.NOISE_LIBM, 0)
    fa, fb = int(a["frame_error"].sum()), int(b["frame_error"].sum())
    assert fb >= 200, fb  # enough frame errors for the comparison to mean something
    assert _overlap(ErrorRate(fa, n), ErrorRate(fb, n)), (fa, fb)
    ok, bers = _ber_agrees(a["bit_errors"], b["bit_errors"], 8448)
    assert ok, bers
    assert np.mean(a["frame_error"] == b["frame_error"]) >= 0.85
    assert abs(_paired_z(a["bit_errors"], b["bit_errors"])) < 3.3
    assert abs(_paired_z(a["iterations"], b["iterations"])) < 3.3


def test_c2_f32_trial_ber_on_the_bench_grid(cb, O):
    # 2 dB, the top of the benchmark grid: every frame fails (FER 1), so the bit errors
    # are the informative count
    n, eb = 256, 2.0
    g32, r = codes(cb, O, CODES[4], "f32")
    a = g32.run_frames(7, NAME, 30, 0, n, eb, 16)
    b = r.run_frames(16, 7, O.fnv1a64(NAME), 30, 0, n, eb, 0, O.NOISE_LIBM, 0)
    assert a["frame_error"].all() and b["frame_error"].all()
    assert (a["iterations"] == 20).all() and (b["iterations"] == 20).all()
    ok, bers = _ber_agrees(a["bit_errors"], b["bit_errors"], 8448)
    assert ok, bers
    assert abs(_paired_z(a["bit_errors"], b["bit_errors"])) < 3.3


def test_large_code_high_snr_decodes_everything(cb, O):
    spec = CODES[4]
    g, _ = codes(cb, O, spec, "f32")
    r = g.run_frames(7, NAME, 0, 0, 512, 4.0, 16)
    assert r["frame_error"].sum() == 0 and r["iterations"].max() <= 12


def test_campaign_counts_match_the_frames(cb, O):
    spec = CODES[0]
    g, r = codes(cb, O, spec)
    grid = cb.Grid().axis("ebn0_db", [0.0, 2.0])
    res = cb.run(g, grid, cb.Stop.min_errors("fer", 50).or_(cb.Stop.max_trials(700)), seed=7, name=NAME,
                 batch=256, modulation=4)
    assert res[0].trials == 256 and res[1].trials == 700  # the bound is met exactly
    for c, eb in enumerate((0.0, 2.0)):
        want = r.run_frames(4, 7, O.fnv1a64(NAME), c, 0, res[c].trials, eb, 0, O.NOISE_CR, 0)
        assert res[c].record["fer"].errors == int(want["frame_error"].sum())
        assert res[c].record["ber"].errors == int(want["bit_errors"].sum())


@pytest.mark.parametrize("spec", [CODES[1], CODES[3], CODES[5]], ids=lambda s: f"k{s['k']}_m{s['m']}")
def test_exact_demapper_f64_llrs_equal_the_oracle_to_rounding(cb, O, spec):
    # Jacobian::Exact: the GPU calls CUDA's exp/log where the oracle calls libm, so the
    # LLRs agree to a few ulps, and the bits and noise draws stay identical
    g = cb.NrLdpc(spec["k"], spec["e"], base_graph=spec.get("bg"), lifting_size=spec.get("z"), precision="f64",
                  demapper="exact")
    r = O.Code(spec["k"], spec["e"], bg=spec.get("bg", 0), z=spec.get("z", 0)).set_decoder(O.RULE_NMS, 0.75, True, 20)
    r.set_demapper(True)
    n = 2 if spec["k"] > 4000 else 6
    llr, info = g.generate_frames(7, NAME, 4, 0, n, 1.5, spec["m"])
    ml, _ = cb.NrLdpc(spec["k"], spec["e"], base_graph=spec.get("bg"), lifting_size=spec.get("z"),
                      precision="f64").generate_frames(7, NAME, 4, 0, n, 1.5, spec["m"])
    for f in range(n):
        rinfo, rllr, _ = r.trial(spec["m"], 7, O.fnv1a64(NAME), 4, f, 1.5, 0, O.NOISE_CR)
        assert np.array_equal(info[f], rinfo)
        assert np.allclose(llr[f], rllr, rtol=1e-13, atol=1e-13), np.max(np.abs(llr[f] - rllr))
    assert not np.allclose(llr, ml)  # the exact LLRs are not the max-log ones


def test_exact_demapper_f32_is_close_to_f64_and_decodes_alike(cb, O):
    from conftest import load_package

    ErrorRate = load_package().campaign.ErrorRate
    spec = CODES[4]
    kw = dict(base_graph=1, lifting_size=384, demapper="exact")
    g32 = cb.NrLdpc(spec["k"], spec["e"], precision="f32", **kw)
    g64 = cb.NrLdpc(spec["k"], spec["e"], precision="f64", **kw)
    l32, i32 = g32.generate_frames(7, NAME, 0, 0, 4, 1.0, 16)
    l64, i64 = g64.generate_frames(7, NAME, 0, 0, 4, 1.0, 16)
    assert np.array_equal(i32, i64)
    err = np.abs(l32.astype(np.float64) - l64) / np.maximum(np.abs(l64), 1.0)
    assert np.median(err) < 1e-5 and np.mean(np.sign(l32) == np.sign(l64)) > 0.9999
    # near the waterfall (about 2.5 dB) the two precisions give the same FER
    a = g32.run_frames(7, NAME, 1, 0, 2048, 2.4, 16)["frame_error"].sum()
    b = g64.run_frames(7, NAME, 1, 0, 2048, 2.4, 16)["frame_error"].sum()
    (lo_a, hi_a), (lo_b, hi_b) = ErrorRate(int(a), 2048).wilson(0.99), ErrorRate(int(b), 2048).wilson(0.99)
    assert not (hi_a < lo_b or hi_b < lo_a), (a, b)
