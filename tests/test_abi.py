"""The C ABI library: it builds, loads, exports every declared symbol, and its host-side
construction agrees with the oracle (no GPU needed)."""

import os
import re

import numpy as np
import pytest

from conftest import ROOT, gpu_available, sionna_vectors


def declared_symbols():
    text = open(os.path.join(ROOT, "include", "comrs_gb300.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(cb_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol(cb):
    names = declared_symbols()
    assert len(names) >= 12
    lib = cb.lib()
    for n in names:
        assert hasattr(lib, n), n
    assert sorted(n for n, _, _ in cb.SYMBOLS) == names


def test_version(cb):
    assert "sm_103a" in cb.version()


def test_fnv_and_jump_match_the_oracle(cb, O):
    assert cb.fnv1a64("a") == O.fnv1a64("a") == 0xAF63DC4C8601EC8C
    # the state of Rng::new(seed) after n draws, by jump-ahead, equals stepping
    import oracle as orc  # noqa: F401

    seed = 1234
    # the stream's first draws come from Rng::new(c); xoshiro_jump works on raw states
    st = np.array([0x0123456789ABCDEF, 0x1111, 0x2222, 0x3333], np.uint64)
    for n in (0, 1, 5, 300, 21120):
        a = cb.xoshiro_jump(st, n)
        b = st.copy()
        for _ in range(n):
            s0, s1, s2, s3 = (int(x) for x in b)
            t = (s1 << 17) & 0xFFFFFFFFFFFFFFFF
            s2 ^= s0
            s3 ^= s1
            s1 ^= s2
            s0 ^= s3
            s2 ^= t
            s3 = ((s3 << 45) | (s3 >> 19)) & 0xFFFFFFFFFFFFFFFF
            b = np.array([s0, s1, s2, s3], np.uint64)
        assert np.array_equal(a, b), n
    del seed


CODES = [
    dict(k=520, e=1040, bg=2, z=52),          # benchmark config 1
    dict(k=8448, e=25344, bg=1, z=384),       # benchmark config 2
    dict(k=8448, e=16896, bg=1, z=384),       # benchmark config 5
    dict(k=100, e=300),                       # the reference's doc example (BG2, Z=18)
    dict(k=500, e=1200, rv=2, qm=4),
    dict(k=1000, e=1500, rv=3, qm=6),
    dict(k=60, e=1000, rv=1, qm=2),           # repetition (E > N_cb)
    dict(k=3000, e=4500),
]


@pytest.mark.parametrize("spec", CODES)
def test_construction_equals_the_oracle(cb, O, spec):
    code = cb.NrLdpc(spec["k"], spec["e"], base_graph=spec.get("bg"), lifting_size=spec.get("z"),
                     rv=spec.get("rv", 0), qm=spec.get("qm", 1))
    ref = O.Code(spec["k"], spec["e"], bg=spec.get("bg", 0), z=spec.get("z", 0), rv=spec.get("rv", 0),
                 qm=spec.get("qm", 1))
    assert (code.bg, code.z, code.n_full, code.edges) == (ref.bg, ref.z, ref.n_full, ref.edges)
    ent, bm = code.tables()
    assert np.array_equal(bm, ref.bit_map())
    # the lifted rows of the entries equal the oracle's edge list
    rows, vars_ = ref.edges_list()
    z = code.z
    got_rows, got_vars = [], []
    for L in range(ent[:, 0].max() + 1):
        sub = ent[ent[:, 0] == L]
        for r in range(z):
            for _, j, sh in sub:
                got_rows.append(L * z + r)
                got_vars.append(j * z + (r + sh) % z)
    assert np.array_equal(np.array(got_rows), rows) and np.array_equal(np.array(got_vars), vars_)
    rng = np.random.default_rng(spec["k"])
    info = rng.integers(0, 2, (3, spec["k"]), dtype=np.uint8)
    enc = code.encode(info)
    for i in range(3):
        assert np.array_equal(enc[i], ref.encode(info[i]))


def test_host_encoder_on_the_sionna_vectors(cb):
    vec, pairs = sionna_vectors()
    for k, n in pairs:
        u, c = vec[f"ldpc.k{k}_n{n}.u"], vec[f"ldpc.k{k}_n{n}.c"]
        assert np.array_equal(cb.NrLdpc(k, n).encode(u), c), (k, n)


@pytest.mark.parametrize("kw,msg", [
    (dict(k=9000, e=10000), "code block"),
    (dict(k=100, e=301, qm=2), "Qm"),
    (dict(k=100, e=300, rv=4), "rv"),
    (dict(k=100, e=300, base_graph=3), "base graph"),
    (dict(k=100, e=300, lifting_size=17), "lifting size"),
    (dict(k=8448, e=25344, base_graph=1, lifting_size=352), "systematic"),
    (dict(k=100, e=300, rule="bogus"), "rule"),
    (dict(k=100, e=300, precision="f16"), "precision"),
])
def test_bad_settings_are_config_errors(cb, kw, msg):
    k, e = kw.pop("k"), kw.pop("e")
    with pytest.raises(cb.ComrsError) as ei:
        cb.NrLdpc(k, e, **kw)
    assert ei.value.kind == "Config" and msg in str(ei.value)


@pytest.mark.skipif(gpu_available(), reason="checks the behaviour without a GPU")
@pytest.mark.parametrize("kw", [dict(rule="sum_product"), dict(layered=False), dict(rule="offset_min_sum", alpha=0.5,
                                                                                  layered=False)])
def test_sum_product_and_flooding_codes_build_and_fail_loudly_without_a_gpu(cb, kw):
    # these settings run on the generic sparse decoder over the lifted rows
    code = cb.NrLdpc(520, 1040, base_graph=2, lifting_size=52, **kw)
    assert (code.z, code.n_full) == (52, 2704)
    with pytest.raises(cb.ComrsError) as ei:
        code.decode(np.zeros(1040))
    assert ei.value.kind == "Cuda"


@pytest.mark.skipif(gpu_available(), reason="checks the behaviour without a GPU")
def test_device_calls_fail_loudly_without_a_gpu(cb):
    code = cb.NrLdpc(520, 1040, base_graph=2, lifting_size=52)
    with pytest.raises(cb.ComrsError) as ei:
        code.decode(np.zeros(1040))
    assert ei.value.kind == "Cuda"
    with pytest.raises(cb.ComrsError):
        code.run_frames(7, "x", 0, 0, 4, 1.0)
