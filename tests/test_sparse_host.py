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
