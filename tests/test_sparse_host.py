"""Generic sparse codes, host side: the alist parser against the reference's rules
(crates/com-fec/src/ldpc.rs:638-741 and its doc example), the code tables the library
builds without a GPU, and the level schedule that keeps the layered order exact."""

import os

import numpy as np
import pytest
from conftest import gpu_available

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

# the (7, 4) Hamming code of LdpcCode::from_alist's example (ldpc.rs:361-370)
HAMMING = ("7 3\n3 4\n3 2 2 2 1 1 1\n4 4 4\n"
           "1 2 3\n1 2 0\n1 3 0\n2 3 0\n1 0 0\n2 0 0\n3 0 0\n"
           "1 2 3 5\n1 2 4 6\n1 3 4 7\n")


def test_parse_alist_reads_the_reference_example(cb):
    n, rows = cb.parse_alist(HAMMING)
    assert n == 7 and len(rows) == 3
    assert rows[1] == [0, 1, 3, 5]
    # the same matrix without padding, with comments
    text = ("7 3 # n m\n3 4\n3 2 2 2 1 1 1\n4 4 4\n1 2 3\n1 2\n1 3\n2 3\n1\n2\n3\n"
            "1 2 3 5\n1 2 4 6\n1 3 4 7  # last row\n")
    assert cb.parse_alist(text) == (n, rows)


@pytest.mark.parametrize("text, words", [
    ("7 3\n3 4\n", "ends before"),
    ("0 3\n", "a matrix of"),
    (HAMMING.replace("3 2 2 2 1 1 1", "2 2 2 2 1 1 1", 1), "column degrees do not have the maximum"),
    (HAMMING.replace("1 2 3 5\n", "1 2 3 9\n"), "outside 1 to 7"),
    (HAMMING.replace("1 2 3 5\n", "1 2 2 5\n"), "repeated"),
    (HAMMING.replace("1 0 0\n2 0 0", "1 0 0\n2 1 0", 1), "more entries than its degree"),
    (HAMMING.replace("1 2 4 6\n", "1 2 4 5\n"), "does not list it"),
    (HAMMING + "1\n", "numbers after the degrees"),
    (HAMMING.replace("3 4\n", "3 x\n", 1), "is not a number"),
])
def test_parse_alist_rejects_malformed_files(cb, text, words):
    with pytest.raises(ValueError, match=words):
        cb.parse_alist(text)


def _levels_python(n, rows):
    last = [-1] * n
    lv = []
    for r in rows:
        level = max([last[v] + 1 for v in r] + [0])
        lv.append(level)
        for v in r:
            last[v] = level
    return lv


@pytest.mark.parametrize("matrix", ["peg_n576_k288.alist", "peg_n648_k540.alist"])
def test_tables_and_level_schedule(cb, O, matrix):
    text = open(os.path.join(GOLDEN, matrix)).read()
    n, rows = cb.parse_alist(text)
    # the oracle parses the same file into the same rows
    ref = O.Code(alist=text)
    _, vars_ = ref.edges_list()
    assert [v for r in rows for v in r] == vars_.tolist()
    code = cb.Ldpc(n, rows, rule="normalized_min_sum", alpha=0.75, max_iterations=20)
    info = code.info()
    assert (info["n"], info["m"], info["edges"]) == (n, len(rows), sum(map(len, rows)))
    assert info["max_row_degree"] == max(map(len, rows))
    ls, lr = code.levels()
    want = _levels_python(n, rows)
    assert info["levels"] == max(want) + 1 and ls[-1] == len(rows)
    for L in range(info["levels"]):
        members = lr[ls[L]:ls[L + 1]].tolist()
        assert members == sorted(members) and all(want[r] == L for r in members)
        seen = set()
        for r in members:  # rows of one level share no variable
            assert not seen & set(rows[r])
            seen |= set(rows[r])
    # every variable meets its rows in increasing row order
    order = {r: want[r] for r in range(len(rows))}
    for v in range(n):
        lv = [order[r] for r in range(len(rows)) if v in rows[r]]
        assert lv == sorted(lv) and len(set(lv)) == len(lv)
    assert info["max_level_rows"] == max(np.diff(ls)) and info["levels"] <= len(rows)
    code.close()


def test_bad_codes_are_config_errors(cb):
    for rows, words in (([[0, 7]], "missing variable"), ([[0, 1, 0]], "twice")):
        with pytest.raises(cb.ComrsError, match=words) as e:
            cb.Ldpc(7, rows)
        assert e.value.status == -1
    with pytest.raises(cb.ComrsError, match="rule must be"):
        cb.Ldpc(7, [[0, 1]], rule="bit_flipping")
    with pytest.raises(cb.ComrsError, match="max_iterations"):
        cb.Ldpc(7, [[0, 1]], max_iterations=-1)
    with pytest.raises(cb.ComrsError, match="a matrix of"):
        cb.Ldpc(7, [])


@pytest.mark.skipif(gpu_available(), reason="checks the behaviour without a GPU")
def test_decoding_without_a_gpu_fails_loudly(cb):
    code = cb.Ldpc(7, cb.parse_alist(HAMMING)[1])
    with pytest.raises(cb.ComrsError) as e:
        code.decode_llr(np.ones(7))
    assert e.value.status == -6  # a CUDA error, no CPU fallback


# ---------------------------------------------------------------- constructions

@pytest.mark.parametrize("matrix, n, k", [("peg_n576_k288.alist", 576, 288), ("peg_n648_k540.alist", 648, 540)])
def test_peg_reproduces_the_reference_matrices(cb, matrix, n, k):
    # validation/tests/aff3ct.rs:344-369: the matrices given to AFF3CT are
    # LdpcCode::peg(n, k, 3, 1).to_alist(), and H has full rank
    code = cb.Ldpc.peg(n, k)
    assert code.to_alist() == open(os.path.join(GOLDEN, matrix)).read()
    assert (code.n, code.k) == (n, k)
    assert cb.Ldpc.from_alist(code.to_alist()).rows == code.rows


def test_peg_known_answers(cb):
    # bindings/com-py/src/fec/ldpc_code.rs:51-54
    code = cb.Ldpc.peg(96, 48)
    assert (code.n, code.k, code.girth() >= 6) == (96, 48, True)
    # crates/com-fec/src/ldpc.rs:978-995: regular, no four-cycles, full rank
    code = cb.Ldpc.peg(504, 252, seed=2)
    assert code.k == 252 and code.girth() >= 6
    assert np.bincount([v for r in code.rows for v in r], minlength=504).tolist() == [3] * 504
    # ldpc.rs:1081-1095 (Hu, Eleftheriou & Arnold 2005, Sec. VI): girth 8, check degrees
    # 5, 6 and 7, as many of degree 5 as of degree 7
    for seed in (0, 1, 2):
        code = cb.Ldpc.peg(504, 252, var_degree=3, seed=seed)
        assert code.girth() == 8, seed
        deg = np.bincount([len(r) for r in code.rows])
        assert np.nonzero(deg)[0].tolist() == [5, 6, 7] and deg[5] == deg[7], seed


@pytest.mark.parametrize("n, k, d, words", [(10, 10, 3, "PEG needs 0 < k < n, got k = 10, n = 10"),
                                            (10, 0, 3, "PEG needs 0 < k < n"),
                                            (10, 6, 5, "variable degree 5 for 4 checks"),
                                            (10, 6, 0, "variable degree 0 for 4 checks")])
def test_peg_rejects_bad_sizes(cb, n, k, d, words):
    with pytest.raises(cb.ComrsError, match=words):
        cb.Ldpc.peg(n, k, var_degree=d)


def test_alist_round_trip_and_hamming(cb):
    # ldpc.rs:357-369: (n, k) = (7, 4), row 1, and to_alist gives the file back
    code = cb.Ldpc.from_alist(HAMMING)
    assert (code.n, code.k) == (7, 4)
    assert code.rows[1] == [0, 1, 3, 5]
    assert code.to_alist() == HAMMING
    assert code.girth() == 4 and abs(code.rate - 4 / 7) < 1e-15
    assert code.info_positions().tolist() == [0, 1, 2, 3]


def _random_rows(rng, n, m, dmax):
    return [sorted(rng.choice(n, size=rng.integers(1, dmax + 1), replace=False).tolist()) for _ in range(m)]


def test_information_positions_equal_the_oracle(cb, O):
    # LdpcCode::from_rows (ldpc.rs:216-231): k = n - rank H, the columns without a pivot
    # when H is reduced from the last column; rank-deficient matrices included
    rng = np.random.default_rng(11)
    cases = [(576, cb.ldpc.peg_rows(576, 288)), (648, cb.ldpc.peg_rows(648, 540))]
    for n, m, d in ((40, 20, 6), (64, 70, 5), (33, 10, 33), (100, 50, 3)):
        cases.append((n, _random_rows(rng, n, m, d)))
    rows = _random_rows(rng, 50, 25, 8)
    cases.append((50, rows + rows[:5]))  # repeated checks
    for n, rows in cases:
        code = cb.Ldpc(n, rows)
        ref = O.Code(rows=rows, n=n)
        assert code.k == ref.k and code.info_positions().tolist() == ref.info_positions().tolist(), n


def test_codes_without_information_bits_and_encoder_errors(cb):
    code = cb.Ldpc(2, [[0], [1]])
    with pytest.raises(cb.ComrsError, match="no information bits"):
        code.k
    with pytest.raises(cb.ComrsError, match="without an encoder"):
        cb.Ldpc(7, cb.parse_alist(HAMMING)[1], encoder=None).k


def test_accumulate_checks_the_dual_diagonal(cb):
    # LdpcCode::accumulate (ldpc.rs:241-256)
    n, k, rows = cb.dvbs2.ldpc_rows("short", "1/2")
    code = cb.Ldpc.accumulate(n, rows)
    assert code.k == k == 7200 and code.info_positions().tolist() == list(range(k))
    bad = [list(r) for r in rows]
    bad[3] = [v for v in bad[3] if v != k + 2]
    with pytest.raises(cb.ComrsError, match=r"check 3 is not dual-diagonal: parity bits \[7203\], "
                                            r"expected \[7202, 7203\]"):
        cb.Ldpc.accumulate(n, bad)
    with pytest.raises(cb.ComrsError, match="5 checks for 5 bits"):
        cb.Ldpc.accumulate(5, [[0], [1], [2], [3], [4]])


def test_set_decoder_checks_its_settings(cb):
    code = cb.Ldpc(7, cb.parse_alist(HAMMING)[1])
    code.set_decoder("Offset_Min_Sum", alpha=0.25, layered=False, max_iterations=7)
    assert (code.rule, code.alpha, code.layered, code.max_iterations) == ("offset_min_sum", 0.25, False, 7)
    with pytest.raises(cb.ComrsError, match="rule must be"):
        code.set_decoder("bit_flipping")
    with pytest.raises(cb.ComrsError, match="max_iterations"):
        code.set_decoder("min_sum", max_iterations=-2)
    with pytest.raises(cb.ComrsError, match="alpha must be finite"):
        code.set_decoder("normalized_min_sum", alpha=float("nan"))


def test_block_shapes_are_checked(cb):
    code = cb.Ldpc.from_alist(HAMMING)
    with pytest.raises(ValueError, match="not a multiple of 4"):
        code.encode(np.zeros(6, np.uint8))
    with pytest.raises(ValueError, match="expected 7"):
        code.decode(np.zeros((2, 6)))


def test_docstring_examples(cb):
    # the examples of Ldpc (the reference's LdpcCode examples, bindings/com-py/src/fec/
    # ldpc_code.rs:51-54, :130-156); those that need a GPU are skipped here and run in
    # tests/test_gpu_sparse.py
    import doctest

    finder, runner = doctest.DocTestFinder(), doctest.DocTestRunner(optionflags=doctest.ELLIPSIS)
    for t in finder.find(cb.Ldpc, "Ldpc"):
        runner.run(t)
    assert runner.failures == 0 and runner.tries >= 6
