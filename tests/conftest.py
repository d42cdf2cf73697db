"""Test configuration: the repository root on sys.path and the `gpu` marker.

`-m "not gpu"` runs on a machine without a GPU (oracle pins, host logic,
the C ABI's exports and argument errors); `-m gpu` runs the parity tests
through the C ABI on a GB300.
"""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a) and the built library")
