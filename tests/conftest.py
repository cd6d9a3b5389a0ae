import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))

from oracle.build_ref import REFERENCE_ROOT as REFERENCE  # noqa: E402


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300); run with -m gpu")


@pytest.fixture(scope="session", autouse=True)
def _built():
    from refraktor_gb300 import build

    build.build()
    from oracle import oracle

    oracle.build()


@pytest.fixture(scope="session")
def db():
    from refraktor_gb300 import librefrakt as lr

    return lr.flamedb()


@pytest.fixture(scope="session")
def ref_config():
    p = REFERENCE / "config"
    if not (p / "variations_new.yml").exists():
        pytest.skip("reference config not present")
    return p
