import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and libpbr.so built for sm_103a")


_MEASURED = []


@pytest.fixture
def measured(request):
    """measured(name, value): records a value the test measured (an error
    against the oracle, a mismatch count) for the end-of-run summary, which
    pytest prints even with -q."""
    def record(name, value):
        _MEASURED.append((request.node.nodeid, name, value))
    return record


def pytest_terminal_summary(terminalreporter, exitstatus, config):
    if _MEASURED:
        terminalreporter.write_sep("-", "measured values")
        for nodeid, name, value in _MEASURED:
            terminalreporter.write_line(f"{nodeid}: {name} = {value}")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as orc
    orc.build()
    return orc


@pytest.fixture(scope="session")
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from pybatchrender_gb300 import _capi
    _capi.load(build_if_missing=True)
    return torch.device("cuda", 0)
