import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT / "box2d-optimized_gb300"))
sys.path.insert(0, str(ROOT / "tests"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300); runs the engine's kernels")


@pytest.fixture(scope="session")
def lib():
    import b2gpu as G

    return G.Lib()


@pytest.fixture(scope="session")
def orc():
    import oracle_bind as ob

    return ob.Oracle()


@pytest.fixture(scope="session")
def ref():
    import oracle_bind as ob

    if not ob.REF_PATH.exists():
        pytest.skip("reference engine not built here (its sources are not checked out)")
    return ob.Ref()
