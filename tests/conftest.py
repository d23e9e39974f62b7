import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests", "golden")):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(ROOT, "tests", "golden")
# The reference checkout (sources only; never needed on a GPU machine): REF_DIR,
# else a directory named "reference" beside the repository.
REF_DIR = os.environ.get("REF_DIR") or os.path.join(os.path.dirname(ROOT), "reference")
HAVE_REF = os.path.isdir(os.path.join(REF_DIR, "eval"))
SMALL_CASES = ["ref_r10", "ref_r1", "ref_r3_edge"]


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (CUDA device) and the built libidash_gpu.so")
    config.addinivalue_line("markers", "slow: long-running (full-scale) case")


@pytest.fixture(scope="session")
def oracle():
    import pyoracle
    pyoracle.lib()
    return pyoracle
