import json
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from tests.parity_log import RECORDS as PARITY_RECORDS  # noqa: E402


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run on the GB300 box)")


def pytest_terminal_summary(terminalreporter):
    if PARITY_RECORDS:
        terminalreporter.write_sep("-", "measured error against the oracle")
        for rec in PARITY_RECORDS:
            terminalreporter.write_line("PARITY " + json.dumps(rec))


@pytest.fixture(scope="session")
def cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch
