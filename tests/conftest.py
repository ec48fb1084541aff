"""Shared fixtures.  GPU tests carry @pytest.mark.gpu and call the CUDA pass
through its C ABI; everything else runs on the CPU."""
import importlib
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (run with -m gpu)")


@pytest.fixture(scope="session")
def bsm():
    return importlib.import_module("bisemutum-engine_gb300")


@pytest.fixture(scope="session")
def oracle():
    import oracle as o
    return o


@pytest.fixture(scope="session")
def ctx(bsm):
    c = bsm.Context(0)
    yield c
    c.close()


def random_rays(n, lo, hi, seed=0, tmax=100.0):
    rng = np.random.default_rng(seed)
    o = rng.uniform(lo, hi, (n, 3)).astype(np.float32)
    d = rng.normal(size=(n, 3)).astype(np.float32)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    return np.concatenate([o, np.zeros((n, 1), np.float32), d, np.full((n, 1), tmax, np.float32)], 1)


def assert_bits_equal(gpu_img, oracle_img, what=""):
    """Images equal bit for bit (both rendered with fixed-point sums: BSM_PT_DETERMINISTIC on the GPU, the same
    flag bit in the oracle)."""
    g = np.ascontiguousarray(gpu_img).view(np.uint32)
    c = np.ascontiguousarray(oracle_img).view(np.uint32)
    assert g.shape == c.shape
    bad = np.argwhere(g != c)
    assert bad.size == 0, (f"{what}{len(bad)} values differ bit-wise, first {bad[:4].tolist()}: "
                           f"gpu {gpu_img[tuple(bad[0])]!r} oracle {oracle_img[tuple(bad[0])]!r}")
