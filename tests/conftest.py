import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)


# The device-side Tsit5 attempt loop must be the path the tests exercise:
# a failed capture of it is an error here, not a silent host-loop run.
os.environ.setdefault("FI_REQUIRE_TSIT_GRAPH", "1")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
