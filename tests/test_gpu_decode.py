"""GPU decoder parity: the CUDA layered min-sum against the oracle on LLR dumps.

f64: hard decisions, iteration counts and a posteriori LLRs bit-identical to the oracle's
restatement of LdpcCode::propagate.  f32: bit-identical to the same algorithm in f32;
within 1e-5 relative of the f64 decoder after one iteration, and the same outcome after a
whole decode.
"""

import numpy as np
import pytest

from conftest import sionna_vectors

pytestmark = pytest.mark.gpu

SEED = 7

CODES = [
    dict(k=520, e=1040, bg=2, z=52, m=4, ebn0=(0.5, 1.5, 2.5)),      # benchmark config 1
    dict(k=100, e=300, m=4, ebn0=(1.0, 3.0)),                         # fillers (K' < K)
    dict(k=500, e=1200, rv=2, qm=4, m=16, ebn0=(2.0, 4.0)),
    dict(k=60, e=1000, rv=1, qm=2, m=4, ebn0=(-2.0,)),               # repeated bits
    dict(k=1056, e=3168, bg=1, z=48, m=16, ebn0=(1.5, 3.0)),
    dict(k=8448, e=25344, bg=1, z=384, m=16, ebn0=(2.5, 3.0)),       # benchmark config 2
]


def dump(O, spec, n, ebn0, cond=0):
    code = O.Code(spec["k"], spec["e"], bg=spec.get("bg", 0), z=spec.get("z", 0), rv=spec.get("rv", 0),
                  qm=spec.get("qm", 1))
    code.set_decoder(O.RULE_NMS, 0.75, True, 20)
    llr = np.zeros((n, spec["e"]))
    h = O.fnv1a64("dump")
    for f in range(n):
        _, llr[f], _ = code.trial(spec["m"], SEED, h, cond, f, ebn0)
    return code, llr


def gpu_code(cb, spec, precision, rule="normalized_min_sum", alpha=0.75, it=20):
    return cb.NrLdpc(spec["k"], spec["e"], base_graph=spec.get("bg"), lifting_size=spec.get("z"),
                     rv=spec.get("rv", 0), qm=spec.get("qm", 1), precision=precision, rule=rule, alpha=alpha,
                     max_iterations=it)


@pytest.mark.parametrize("spec", CODES, ids=lambda s: f"k{s['k']}_e{s['e']}")
def test_f64_decode_is_bit_exact(cb, O, spec):
    n = 6 if spec["k"] > 4000 else 24
    g = gpu_code(cb, spec, "f64")
    for eb in spec["ebn0"]:
        ref, llr = dump(O, spec, n, eb)
        bits, app, it = g.decode_full(llr)
        for f in range(n):
            rb, rit, rapp, _ = ref.decode(llr[f], "f64", want_app=True)
            assert np.array_equal(bits[f], rb), (eb, f)
            assert it[f] == rit, (eb, f, it[f], rit)
            assert np.array_equal(app[f].view(np.uint64), rapp.view(np.uint64)), (eb, f)


@pytest.mark.parametrize("spec", CODES, ids=lambda s: f"k{s['k']}_e{s['e']}")
def test_f32_decode_is_bit_exact_to_the_f32_oracle(cb, O, spec):
    n = 6 if spec["k"] > 4000 else 24
    g = gpu_code(cb, spec, "f32")
    for eb in spec["ebn0"]:
        ref, llr = dump(O, spec, n, eb)
        l32 = llr.astype(np.float32)
        bits, app, it = g.decode_full(l32)
        for f in range(n):
            rb, rit, rapp, _ = ref.decode(l32[f], "f32", want_app=True)
            assert np.array_equal(bits[f], rb) and it[f] == rit
            assert np.array_equal(app[f].view(np.uint32), rapp.view(np.uint32))


# The f32 decoder against com-fec's f64 decoder on the same (f64-dumped) LLRs.  One
# layered iteration keeps every a posteriori LLR within 1e-5 relative of the f64 one
# (measured: 1.2e-6 on the C2 code, 6.5e-7 on C1).  Further iterations amplify the
# rounding differences as the min-sum dynamics amplify any perturbation: about 8x per
# iteration on BG1 Z = 384 (1.1e-5 after two, 8.5e-5 after three, O(1) after eight) and
# 2.5x on BG2 Z = 52.  A whole decode therefore agrees on the outcome (decisions and
# iteration counts), not on the last digits of the LLRs.
@pytest.mark.parametrize("spec,eb", [(CODES[0], 2.0), (CODES[5], 3.0)], ids=["c1", "c2"])
def test_f32_first_iteration_is_within_1e5_of_the_f64_decoder(cb, O, spec, eb):
    n = 8 if spec["k"] > 4000 else 64
    g32, g64 = gpu_code(cb, spec, "f32", it=1), gpu_code(cb, spec, "f64", it=1)
    _, llr = dump(O, spec, n, eb)
    _, a32, _ = g32.decode_full(llr.astype(np.float32))
    _, a64, _ = g64.decode_full(llr)
    rel = np.abs(a32.astype(np.float64) - a64) / np.maximum(np.abs(a64), 1.0)
    assert rel.max() <= 1e-5, rel.max()


@pytest.mark.parametrize("spec,eb,n", [(CODES[0], 2.0, 256), (CODES[5], 3.0, 32)], ids=["c1", "c2"])
def test_f32_decode_agrees_with_the_f64_decoder_on_the_outcome(cb, O, spec, eb, n):
    g32, g64 = gpu_code(cb, spec, "f32"), gpu_code(cb, spec, "f64")
    _, llr = dump(O, spec, n, eb)
    b32, _, i32 = g32.decode_full(llr.astype(np.float32))
    b64, _, i64 = g64.decode_full(llr)
    same = np.all(b32 == b64, axis=1) & (i32 == i64)
    assert same.mean() >= 0.95, same.mean()


@pytest.mark.parametrize("rule,alpha", [("offset_min_sum", 0.15), ("min_sum", 1.0), ("normalized_min_sum", 0.8)])
def test_other_min_sum_rules(cb, O, rule, alpha):
    spec = CODES[0]
    ref, llr = dump(O, spec, 16, 1.5)
    ref.set_decoder(O.RULE_OMS if rule == "offset_min_sum" else O.RULE_NMS, alpha, True, 20)
    g = gpu_code(cb, spec, "f64", rule=rule, alpha=alpha)
    bits, app, it = g.decode_full(llr)
    for f in range(16):
        rb, rit, rapp, _ = ref.decode(llr[f], "f64", want_app=True)
        assert np.array_equal(bits[f], rb) and it[f] == rit
        assert np.array_equal(app[f].view(np.uint64), rapp.view(np.uint64))


def test_sionna_vectors_decode_on_the_gpu(cb):
    # tests/test_sionna_vectors.py:104-115 of com-rs: decode(4 - 8c) == u for K' <= 1024
    vec, pairs = sionna_vectors()
    for k, n in pairs:
        if k > 1024:
            continue
        u, c = vec[f"ldpc.k{k}_n{n}.u"], vec[f"ldpc.k{k}_n{n}.c"]
        for precision in ("f64", "f32"):
            g = cb.NrLdpc(k, n, max_iterations=50, precision=precision)
            assert np.array_equal(g.decode(4.0 - 8.0 * c.astype(np.float64)), u), (k, n, precision)


def test_edge_cases(cb, O):
    spec = CODES[0]
    g = gpu_code(cb, spec, "f64")
    # no frames
    assert g.decode(np.zeros((0, 1040))).shape == (0, 520)
    # all-zero LLRs: the all-zero word is a codeword, zero iterations
    bits, app, it = g.decode_full(np.zeros(1040))
    assert it == 0 and not bits.any()
    # negative zeros, huge magnitudes and a codeword: as the oracle
    ref = O.Code(520, 1040, bg=2, z=52).set_decoder(O.RULE_NMS, 0.75, True, 20)
    rng = np.random.default_rng(3)
    info = rng.integers(0, 2, 520, dtype=np.uint8)
    cw = ref.encode(info)
    for llr in (np.where(cw == 1, -0.0, 0.0), 1e300 * (1 - 2.0 * cw), (1 - 2.0 * cw) * 3.0,
                np.where(rng.random(1040) < 0.3, -0.0, (1 - 2.0 * cw) * rng.random(1040))):
        b, a, i = g.decode_full(llr)
        rb, ri, ra, _ = ref.decode(llr, "f64", want_app=True)
        assert np.array_equal(b, rb) and i == ri
        assert np.array_equal(a.view(np.uint64), ra.view(np.uint64))
    # max_iterations = 0 returns the channel decisions
    g0 = gpu_code(cb, spec, "f64", it=0)
    ref.set_decoder(O.RULE_NMS, 0.75, True, 0)
    _, llr = dump(O, spec, 4, 0.0)
    b, a, i = g0.decode_full(llr)
    for f in range(4):
        rb, ri, _, _ = ref.decode(llr[f], "f64")
        assert np.array_equal(b[f], rb) and i[f] == ri == 0


def test_many_frames_in_one_launch(cb, O):
    # more frames than resident CTAs: the persistent grid's work stealing covers them all
    spec = CODES[0]
    ref, llr = dump(O, spec, 40, 1.0)
    big = np.tile(llr, (60, 1))
    g = gpu_code(cb, spec, "f64")
    bits, app, it = g.decode_full(big)
    bits1, app1, it1 = g.decode_full(llr)
    assert np.array_equal(bits, np.tile(bits1, (60, 1))) and np.array_equal(it, np.tile(it1, 60))


def test_decode_device_accepts_a_buffer_of_any_alignment(cb):
    # the f32 decoder loads the LLRs 128 bits at a time from 16-byte aligned buffers and
    # 32 bits at a time from any other: both give the same results
    import ctypes as C

    import torch

    g = cb.NrLdpc(8448, 25344, base_graph=1, lifting_size=384, precision="f32")
    llr, _ = g.generate_frames(7, "align", 0, 0, 16, 1.5, 16)
    flat = torch.zeros(16 * 25344 + 4, dtype=torch.float32, device="cuda")
    outs = []
    for off in (0, 1):
        flat[off:off + 16 * 25344] = torch.from_numpy(llr.reshape(-1)).cuda()
        bits = torch.zeros((16, 264), dtype=torch.int32, device="cuda")
        its = torch.zeros(16, dtype=torch.int32, device="cuda")
        torch.cuda.synchronize()  # the decoder runs on the code's own stream
        st = cb.lib().cb_decode_device(g._h, C.c_void_p(flat.data_ptr() + 4 * off), 16, C.c_void_p(bits.data_ptr()),
                                       None, C.c_void_p(its.data_ptr()), None)
        assert st == 0
        torch.cuda.synchronize()
        outs.append((bits.cpu(), its.cpu()))
    assert torch.equal(outs[0][0], outs[1][0]) and torch.equal(outs[0][1], outs[1][1])
    # and they are the host-buffer decoder's
    ref_bits, _, ref_it = g.decode_full(llr)
    assert np.array_equal(outs[0][1].numpy(), ref_it)
    got = np.unpackbits(outs[0][0].numpy().view(np.uint8), axis=1, bitorder="little")[:, :8448]
    assert np.array_equal(got, ref_bits)


def test_concurrent_callers_on_one_code_object(cb):
    # calls on one code object are serialised by its mutex: four host threads decoding
    # through the same object get what one thread gets
    import threading

    g = cb.NrLdpc(520, 1040, base_graph=2, lifting_size=52, precision="f32")
    llr, _ = g.generate_frames(7, "threads", 0, 0, 4 * 256, 1.0, 4)
    want = [g.decode_full(llr[i * 256:(i + 1) * 256]) for i in range(4)]
    got = [None] * 4

    def work(i):
        for _ in range(3):
            got[i] = g.decode_full(llr[i * 256:(i + 1) * 256])

    threads = [threading.Thread(target=work, args=(i,)) for i in range(4)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    for (wb, wa, wi), (gb, ga, gi) in zip(want, got):
        assert np.array_equal(wb, gb) and np.array_equal(wi, gi)
        assert np.array_equal(wa.view(np.uint32), ga.view(np.uint32))


@pytest.mark.parametrize("spec", [dict(k=8448, e=25344, bg=1, z=384, n=600, m=16, eb=2.6, precision="f32"),
                                  dict(k=8448, e=25344, bg=1, z=384, n=300, m=16, eb=2.6, precision="f64"),
                                  dict(k=520, e=1040, bg=2, z=52, n=70000, m=4, eb=1.5, precision="f32")],
                         ids=["c2_f32", "c2_f64", "c1_f32_two_chunks"])
def test_host_decode_reads_page_locked_llrs_in_place(cb, spec):
    # page-locked host LLRs are read by the decoder where they are, without staging copies
    # (C1: two launches of 65,536 and 4,464 frames): the same decisions, a posteriori LLRs
    # and iterations as from pageable memory
    torch = pytest.importorskip("torch")
    g = cb.NrLdpc(spec["k"], spec["e"], base_graph=spec["bg"], lifting_size=spec["z"], precision=spec["precision"])
    llr, _ = g.generate_frames(7, "page_locked", 0, 0, spec["n"], spec["eb"], spec["m"])
    pinned = torch.empty(llr.shape, dtype=torch.float32 if spec["precision"] == "f32" else torch.float64,
                         pin_memory=True)
    pinned.numpy()[:] = llr
    b1, a1, i1 = g.decode_full(llr)
    b2, a2, i2 = g.decode_full(pinned.numpy())
    assert np.array_equal(b1, b2) and np.array_equal(i1, i2)
    assert np.array_equal(a1.view(np.uint8), a2.view(np.uint8))
    assert len(set(i1.tolist())) > 2


@pytest.mark.parametrize("precision", ["f32", "f64"])
def test_host_decode_in_chunks_equals_small_calls(cb, precision):
    # cb_decode splits a large host batch into chunks whose copies overlap the decoding of
    # the previous chunk; the results equal those of small calls, one chunk each
    g = cb.NrLdpc(520, 1040, base_graph=2, lifting_size=52, precision=precision)
    llr, _ = g.generate_frames(7, "chunks", 0, 0, 12000, 1.5, 4)
    bits, app, it = g.decode_full(llr)
    for a in range(0, 12000, 1500):
        b2, a2, i2 = g.decode_full(llr[a:a + 1500])
        assert np.array_equal(b2, bits[a:a + 1500]) and np.array_equal(i2, it[a:a + 1500])
        assert np.array_equal(a2.view(np.uint8), app[a:a + 1500].view(np.uint8))
    assert 0 < it.mean() < 20
