import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def c1():
    from messi_gb300 import synth
    return synth.make_workload("c1", seed=1)


@pytest.fixture(scope="session")
def tiny():
    """6 sequences x 14 columns, every pair allowed."""
    from messi_gb300 import synth
    return synth.make_workload(dict(numseqs=6, numcols=14, W=13, paired=0.3, mean_bl=0.15), seed=7)
