import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103) GPU and the built library")


@pytest.fixture(scope="session")
def ctx():
    """One device context for the GPU tests (fails loudly without the CUDA library)."""
    from chrono_photo_gb300 import Context
    c = Context(0)
    yield c
    c.close()


def pytest_collection_modifyitems(config, items):
    # the pure-Python restatement divides by zero where the reference does (inf results)
    for item in items:
        item.add_marker(pytest.mark.filterwarnings("ignore::RuntimeWarning"))
