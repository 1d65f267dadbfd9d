"""Test configuration: the `gpu` marker, import paths and shared fixtures.

Tests marked `gpu` need a CUDA device and call the CUDA library through its C
ABI; everything else runs on the CPU (oracle against golden vectors, host
logic, ABI surface)."""
import glob
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libhsdl.so")


@pytest.fixture(scope="session")
def built():
    """libhsdl.so and the oracle libraries, built in-tree if missing."""
    from gpu4hophl_code_gb300 import _native
    from oracle import oracle as O

    if not os.path.exists(_native.LIB_PATH):
        from gpu4hophl_code_gb300 import build as B

        B.build()
    if not os.path.exists(O.PORT_LIB):
        O.build()
    return _native.lib()


@pytest.fixture(scope="session")
def orc(built):
    from oracle.oracle import Oracle

    return Oracle()


class GoldenCase:
    def __init__(self, path):
        z = np.load(path)
        self.name = os.path.basename(path)[:-4]
        self.d = {k: z[k] for k in z.files}
        from gpu4hophl_code_gb300 import HostGraph

        self.g = HostGraph(int(self.d["n"]), self.d["row_ptr"], self.d["col"], self.d["w"])
        self.K = int(self.d["K"])

    @property
    def full(self):
        return "labels" in self.d


def golden_cases():
    return sorted(glob.glob(os.path.join(GOLDEN, "*.npz")))


@pytest.fixture(params=golden_cases(), ids=lambda p: os.path.basename(p)[:-4])
def golden(request, built):
    return GoldenCase(request.param)


def www_cases():
    return sorted(glob.glob(os.path.join(GOLDEN, "www", "*.npz")))


@pytest.fixture(params=www_cases(), ids=lambda p: "www_" + os.path.basename(p)[:-4])
def golden_www(request, built):
    """The reference's 2023WWW generation on a seeded graph: raw_off/raw_labels
    before the clean, off/labels after (tests/golden/make_golden.py)."""
    return GoldenCase(request.param)
