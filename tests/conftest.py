import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (os.path.join(ROOT, "rust-compress_gb300"), os.path.join(ROOT, "oracle"), ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the rcg kernels)")


@pytest.fixture(scope="session")
def oracle():
    import oracle as O

    O.build()
    return O


@pytest.fixture(scope="session")
def golden():
    import numpy as np

    z = np.load(os.path.join(ROOT, "tests", "golden", "ssim2_pairs.npz"))
    pairs = []
    for n, r, d, s in zip(z["names"], z["refs"], z["dists"], z["scores"]):
        pairs.append((str(n), z["img:" + str(r)], z["img:" + str(d)], float(s)))
    return pairs


@pytest.fixture(scope="session")
def ctx():
    import rcg

    c = rcg.Context(0)
    yield c
    c.close()


def pytest_sessionstart(session):
    # The GPU test modules import the bindings at collection time: make sure librcg.so exists (no-op when current).
    import build as rcg_build  # rust-compress_gb300/build.py

    rcg_build.build()
