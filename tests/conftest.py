import os
import sys

import pytest

# Tests choose their engine settings explicitly; the measured tuning table is
# exercised by tests/test_gpu_tuning.py.
os.environ.setdefault("THINDB_GPU_TUNING", "off")

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "tests"), os.path.join(ROOT, "tests", "golden")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session", autouse=True)
def _built_native():
    """Build the in-tree libraries once per session (fast when up to date)."""
    from thindb_gb300 import build

    build.build_datagen()
    try:
        build.build_engine()
    except RuntimeError as e:  # nvcc missing: the GPU tests fail loudly on their own
        print("engine build failed:", e)
    from oracle import build as obuild

    obuild.build()
    yield
