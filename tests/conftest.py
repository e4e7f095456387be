"""Shared test setup: import paths, the `gpu` marker, golden fixtures."""
import glob
import os
import sys

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for sub in ("xfem-amie_gb300", "oracle"):
    p = os.path.join(REPO, sub)
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN_DIR = os.path.join(REPO, "tests", "golden")
# assembly / solve fixtures (one assembled system each); the damage fixtures hold
# load-step histories instead, and the proportional-multiplier fixture needs its
# own multipliers: both have their own tests
GOLDEN_CASES = sorted(n for n in (os.path.splitext(os.path.basename(p))[0]
                                  for p in glob.glob(os.path.join(GOLDEN_DIR, "*.npz")))
                      if not n.startswith("damage") and not n.startswith("prop"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and libamie_gpu.so")


def load_golden(name):
    return dict(np.load(os.path.join(GOLDEN_DIR, name + ".npz")))


@pytest.fixture(scope="session")
def gpu_ctx():
    import amie_gpu
    ctx = amie_gpu.Context(0)
    yield ctx
    ctx.close()
