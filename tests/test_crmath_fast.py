"""The fast correctly rounded f64 log and sin/cos of the noise (csrc/crmath_fast.cuh) on
the host: the same bits as the double-double routines (csrc/crmath.cuh) and as binary128
rounded once on every input tried, and the constants file against its generator.  The
device runs the same explicitly rounded operations; the GPU frame tests compare its f64
frames with the oracle's, whose noise is binary128 rounded once."""

import os
import platform
import shutil
import subprocess
import sys

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "..", "com-rs_gb300", "csrc")


def test_constants_are_their_generator_output():
    out = subprocess.run([sys.executable, os.path.join(CSRC, "gen_crmath_consts.py")], capture_output=True,
                         text=True, check=True).stdout
    assert out == open(os.path.join(CSRC, "crmath_consts.inc")).read()


def test_fast_paths_return_the_double_double_bits(tmp_path):
    if not shutil.which("g++"):
        pytest.skip("g++ is needed")
    exe = str(tmp_path / "crfast_check")
    quad = [] if platform.machine() in ("aarch64", "arm64") else ["-lquadmath"]
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-I", CSRC,
                    os.path.join(HERE, "native", "crfast_check.cpp"), "-o", exe] + quad, check=True)
    count, diff, diff_q = map(int, subprocess.run([exe, "1000000", "11"], capture_output=True, text=True,
                                                  check=True).stdout.split())
    assert count > 2_000_000 and diff == 0 and diff_q == 0
