import json
import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def built_lib():
    """The device library, built in-tree if missing (host-only use on CPU)."""
    from rstsr_gb300 import build

    build.build()
    from rstsr_gb300 import _lib

    return _lib.lib()


@pytest.fixture(scope="session")
def kats():
    return json.loads((ROOT / "tests" / "golden" / "reference_kats.json").read_text())


@pytest.fixture(scope="session")
def dev(built_lib):
    from rstsr_gb300 import DeviceCuda

    d = DeviceCuda(int(os.environ.get("RSTSR_TEST_DEVICE", "0")))
    yield d
    d.sync()
