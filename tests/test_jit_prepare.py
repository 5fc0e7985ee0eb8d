"""The run-time compiled decoder of an f32 layered min-sum code, prepared without a GPU:
cb_code_prepare compiles it for the code's base graph and lifting size and stores the
cubin in the on-disk cache, with the toolkit's nvcc or, without one, with NVRTC.  Each
case runs in a child process, since the compiler is looked up once per process."""

import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r"""
import importlib, sys
sys.path.insert(0, sys.argv[1])
cb = importlib.import_module("com-rs_gb300")
g = cb.NrLdpc(520, 1040, base_graph=2, lifting_size=52, precision="f32")
g.prepare()
g.prepare()  # the second call finds the cache
try:
    cb.NrLdpc(520, 1040, base_graph=2, lifting_size=52, precision="f64").prepare()
except cb.ComrsError as e:
    assert e.kind == "Config", e
else:
    raise AssertionError("an f64 code has no run-time compiled decoder")
"""


def have_nvrtc():
    import ctypes

    for name in ("libnvrtc.so.13", "libnvrtc.so", "/usr/local/cuda/lib64/libnvrtc.so.13"):
        try:
            ctypes.CDLL(name)
            return True
        except OSError:
            pass
    return False


@pytest.mark.parametrize("compiler", ["nvcc", "nvrtc"])
def test_prepare_fills_the_disk_cache(compiler, tmp_path):
    env = dict(os.environ, COMRS_JIT_CACHE=str(tmp_path))
    env.pop("COMRS_NO_JIT", None)
    env.pop("COMRS_NVCC", None)
    if compiler == "nvrtc":
        if not have_nvrtc():
            pytest.skip("libnvrtc not found")
        env["COMRS_NVCC"] = ""  # set and empty: no nvcc, NVRTC compiles
    elif not any(os.access(os.path.join(d, "nvcc"), os.X_OK)
                 for d in ["/usr/local/cuda/bin"] + os.environ.get("PATH", "").split(":")):
        pytest.skip("nvcc not found")
    subprocess.run([sys.executable, "-c", CHILD, ROOT], env=env, check=True, timeout=600)
    # the plain decoder's and the learned min-sum's kernels for the code's lifting
    files = [f for f in os.listdir(tmp_path) if f.endswith(".cubin")]
    assert len(files) == 2 and all(f.startswith("nr_bg2_z52_") for f in files), files
    assert all(os.path.getsize(tmp_path / f) > 10000 for f in files)
