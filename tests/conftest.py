import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
ORACLE = os.path.join(ROOT, 'oracle')
if ORACLE not in sys.path:
    sys.path.insert(0, ORACLE)


def pytest_configure(config):
    config.addinivalue_line('markers', 'gpu: needs a CUDA GPU (GB300) and the built engine library')


@pytest.fixture(scope='session')
def oracle_lib():
    import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope='session')
def engine():
    """The engine package with its CUDA library built (GPU tests only)."""
    import torch
    if not torch.cuda.is_available():
        pytest.skip('no CUDA device')
    from vk_order_independent_transparency_gb300 import _build
    _build.build()
    import vk_order_independent_transparency_gb300 as oit
    return oit
