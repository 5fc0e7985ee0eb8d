"""The f64 2 atanh of the sum-product rule (csrc/atanh2.cuh) on the host: its table
against its generator, its accuracy against long double, and its special values.  The
device runs the same explicitly rounded operations, so the host copy stands for it."""

import math
import os
import platform
import shutil
import subprocess
import sys

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "..", "com-rs_gb300", "csrc")


def test_table_is_its_generator_output():
    out = subprocess.run([sys.executable, os.path.join(CSRC, "gen_logtab.py")], capture_output=True,
                         text=True, check=True).stdout
    assert out == open(os.path.join(CSRC, "logtab.inc")).read()


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    if not shutil.which("g++"):
        pytest.skip("g++ is needed")
    exe = str(tmp_path_factory.mktemp("atanh2") / "atanh2_check")
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-I", CSRC,
                    os.path.join(HERE, "native", "atanh2_check.cpp"), "-o", exe], check=True)
    return exe


def run(exe, n, seed):
    lines = subprocess.run([exe, str(n), str(seed)], capture_output=True, text=True, check=True).stdout.split("\n")
    worst, cr = map(float, lines[0].split())
    # (input, result) pairs in order: 0.0 and -0.0 are one key of a dict
    special = [(float.fromhex(a), float.fromhex(b)) for a, b in (ln.split() for ln in lines[1:] if ln)]
    return worst, cr, special


def test_accuracy_against_long_double(checker):
    if platform.machine() not in ("x86_64", "AMD64", "aarch64", "arm64"):
        pytest.skip("long double must be wider than double")
    worst, cr, _ = run(checker, 2_000_000, 7)
    # within about half an ulp of the exact value, the correctly rounded one nearly always
    assert worst < 0.51, worst
    assert cr > 0.999, cr


def test_special_values(checker):
    _, _, pairs = run(checker, 4, 1)
    (z, zr), (nz, nzr) = pairs[:2]
    assert math.copysign(1, z) == 1 and math.copysign(1, zr) == 1 and zr == 0
    assert math.copysign(1, nz) == -1 and math.copysign(1, nzr) == -1 and nzr == 0
    sp = dict(pairs[2:])
    B = 0.999999999999
    cap = 2 * math.atanh(B)
    # below 2^-27 the result is 2p exactly, subnormals included
    assert sp[5e-324] == 1e-323 and sp[-1e-300] == -2e-300 and sp[1e-20] == 2e-20 and sp[3.7e-9] == 7.4e-9
    assert sp[0.5] == pytest.approx(2 * math.atanh(0.5), rel=2e-16)
    assert sp[-0.25] == pytest.approx(-2 * math.atanh(0.25), rel=2e-16)
    # the clamp: |p| >= B gives the message 2 atanh(B), with p's sign
    for p in (B, 1.0, 2.0):
        assert sp[p] == pytest.approx(cap, rel=2e-16) and sp[p] == sp[B]
    assert sp[-B] == -sp[B] and sp[-1.0] == -sp[B]
