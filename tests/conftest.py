import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the native kernels")


@pytest.fixture(scope="session")
def oracle():
    from oracle.oracle import Oracle
    return Oracle()


@pytest.fixture(scope="session")
def reference():
    from oracle.oracle import Reference
    if not Reference.available():
        pytest.skip("reference checkout not present (oracle/_ref cannot be built here)")
    return Reference()


@pytest.fixture(scope="session")
def golden():
    import json
    import numpy as np
    kat = json.loads((ROOT / "tests/golden/kat.json").read_text())
    stamps = dict(np.load(ROOT / "tests/golden/stamps_ref.npz"))
    texture = dict(np.load(ROOT / "tests/golden/texture_ref.npz"))
    render = dict(np.load(ROOT / "tests/golden/render_ref.npz"))
    return {"kat": kat, "stamps": stamps, "texture": texture, "render": render}


@pytest.fixture(scope="session")
def pg():
    import painty_gb300
    return painty_gb300
