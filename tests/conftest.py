import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import __graft_entry__  # noqa: E402

__graft_entry__.load_package()

# A checkout of the reference (eTraj.jl), read as data by a few CPU tests (its
# molecule database files); those tests skip when ETRAJ_REFERENCE_DIR is unset.
REFERENCE_DIR = os.environ.get("ETRAJ_REFERENCE_DIR", "")
REFERENCE_DB = os.path.join(REFERENCE_DIR, "src", "Targets", "Database") if REFERENCE_DIR else ""


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built library")
    config.addinivalue_line("markers", "slow: long-running CPU test")
