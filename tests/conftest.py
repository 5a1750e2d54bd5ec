import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
TESTS = os.path.dirname(os.path.abspath(__file__))
if TESTS not in sys.path:
    sys.path.insert(0, TESTS)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300 / sm_103a)")
    config.addinivalue_line("markers", "slow: long-running (full-size workloads)")
    # A test that stops making progress fails after 10 minutes (stacks of every thread dumped)
    # instead of holding the run: pytest-timeout, where it is installed.
    if config.pluginmanager.hasplugin("timeout") and not config.getoption("timeout", None):
        config.option.timeout = 600
        config.option.timeout_method = "thread"
