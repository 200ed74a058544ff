"""Test configuration: the `gpu` marker and import paths.

`-m "not gpu"` runs on any machine: the oracle against the reference's golden
vectors, host-side logic, and that the C ABI library loads and exports every
symbol include/*.h declares.  `-m gpu` tests need a CUDA device and compare the
GB300 kernels with the oracle through the C ABI.
"""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: long-running CPU check")
