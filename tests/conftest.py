import importlib
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run on the GB300 box)")
    config.addinivalue_line("markers", "slow: statistical checks that take tens of seconds")


def load_package():
    """The product package (its directory name has a dash, so it is imported by path)."""
    return importlib.import_module("com-rs_gb300")


@pytest.fixture(scope="session")
def cb():
    return load_package()


@pytest.fixture(scope="session")
def O():
    import oracle

    oracle.build()
    return oracle


def sionna_vectors():
    d = np.load(os.path.join(GOLDEN, "sionna_nr_ldpc.npz"))
    out = {}
    for k in d.files:
        if k.endswith(".shape"):
            continue
        shape = tuple(int(x) for x in d[k + ".shape"])
        out[k] = np.unpackbits(d[k], axis=-1)[..., :shape[-1]].reshape(shape)
    pairs = sorted({tuple(int(x) for x in k.split(".")[1][1:].split("_n")) for k in out})
    return out, pairs


def gpu_available():
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False
