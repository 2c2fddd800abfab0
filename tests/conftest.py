import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle_lib():
    import oracle
    oracle.build()
    return oracle.restatement()


@pytest.fixture(scope="session")
def reference_lib():
    import oracle
    oracle.build()
    lib = oracle.reference()
    if lib is None:
        pytest.skip("reference checker not buildable here (no reference tree or not x86-64)")
    return lib


@pytest.fixture(scope="session")
def cuda_lib():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from softglrender_gb300 import build as b
    b.build()
    import softglrender_gb300 as sg
    return sg.load_library()
