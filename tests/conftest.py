"""Shared test setup: import paths, the `gpu` marker, and helpers.

CPU tests (-m "not gpu") pin the oracle to the reference's golden vectors and check
host logic and the C ABI's exports; GPU tests (-m gpu) compare the CUDA path, called
through the C ABI, with the oracle on the same seeded inputs.
"""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "oracle"), os.path.join(ROOT, "seismic.jl_gb300")):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built shotwem.so")


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (nb if nb > 0 else 1.0))


def load_golden(name):
    z = np.load(os.path.join(GOLDEN, name))
    out = {k: z[k] for k in z.files}
    out["params"] = eval(str(out["params"]))  # a dict literal written by make_golden.py
    return out


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def gpu_lib():
    import wemgpu
    if not os.path.exists(wemgpu.LIB_PATH):
        wemgpu.build()
    return wemgpu
