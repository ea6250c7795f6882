import os
import subprocess
import sys

import pytest

TESTS = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(TESTS)
for p in (ROOT, TESTS):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(TESTS, "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (runs on the GB300 box)")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Build the oracle (and the product library if it is missing)."""
    import oracle_lib

    if not os.path.exists(oracle_lib.ORACLE_SO):
        oracle_lib.build_oracle()
    from pgd_gb300 import LIB_PATH

    if not os.path.exists(LIB_PATH):
        subprocess.run([sys.executable, "-m", "pgd_gb300.build"], cwd=ROOT, check=True)
    yield


@pytest.fixture(scope="session")
def ctx():
    import pgd_gb300 as pgd

    c = pgd.Context()
    yield c
    c.close()
