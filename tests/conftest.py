import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line('markers', 'gpu: needs a CUDA GPU (sm_103a) and the built library')


def pytest_collection_modifyitems(config, items):
    # GPU tests need the library built for this machine's architecture.
    pass


@pytest.fixture(scope='session')
def nt():
    import torch
    if not torch.cuda.is_available():
        pytest.skip('no CUDA device')
    import nt_gb300
    nt_gb300._lib = sys.modules['nt_gb300._lib']
    sys.modules['nt_gb300._lib'].load()
    return nt_gb300
