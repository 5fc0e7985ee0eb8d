"""DVB-S2 LDPC construction (crates/com-systems/src/dvbs2/fec.rs) on the host: the
dimensions of Tables 5a and 5b, the degree distribution of the standard, the
dual-diagonal accumulator, and accumulated codewords that satisfy every check."""

import importlib

import numpy as np
import pytest


@pytest.fixture(scope="module")
def dv():
    from conftest import load_package

    load_package()
    return importlib.import_module("com-rs_gb300.dvbs2")


def test_every_code_has_the_dimensions_of_tables_5a_and_5b(dv):
    for frame in ("normal", "short"):
        for rate in ("1/4", "1/3", "2/5", "1/2", "3/5", "2/3", "3/4", "4/5", "5/6", "8/9", "9/10"):
            if frame == "short" and rate == "9/10":
                with pytest.raises(ValueError):
                    dv.params(frame, rate)
                continue
            n, k_bch, k_ldpc, t, groups = dv.params(frame, rate)
            assert len(groups) * 360 == k_ldpc and k_bch < k_ldpc < n


def test_the_variable_degrees_are_those_of_the_standard(dv):
    # normal frame of rate 1/2: 12 960 bits of degree 8, 19 440 of degree 3, parity bits
    # of degree 2, the last of degree 1 (fec.rs:394-407)
    n, k, rows = dv.ldpc_rows("normal", "1/2")
    deg = np.zeros(n, np.int64)
    for r in rows:
        deg[r] += 1
    assert (int((deg[:k] == 8).sum()), int((deg[:k] == 3).sum())) == (12960, 19440)
    assert int((deg[k:n - 1] == 2).sum()) == n - k - 1 and deg[n - 1] == 1


@pytest.mark.parametrize("rate", ["1/4", "2/3", "8/9"])
def test_accumulated_codewords_satisfy_the_checks(dv, rate):
    # the IRA encoder (LdpcCode::accumulate): p_r = p_{r-1} + sum of the information
    # bits of check r
    n, k, rows = dv.ldpc_rows("short", rate)
    rng = np.random.default_rng(7)
    c = np.zeros(n, np.uint8)
    c[:k] = rng.integers(0, 2, k)
    p = 0
    for r, row in enumerate(rows):
        p ^= int(np.bitwise_xor.reduce(c[[v for v in row if v < k]]))
        c[k + r] = p
    assert all(int(np.bitwise_xor.reduce(c[row])) == 0 for row in rows)


def test_the_short_rate_half_code_builds_a_gpu_decoder(cb):
    code = cb.Dvbs2Ldpc("short", "1/2", max_iterations=50)
    info = code.info()
    assert (info["n"], info["m"], code.k) == (16200, 9000, 7200)
    # the accumulator chain makes the layered order sequential: one row per level
    assert info["levels"] == 9000
