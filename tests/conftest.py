import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "reference: needs the reference checkout (builds oracle/_ref)")


def _has_gpu() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def pytest_collection_modifyitems(config, items):
    if not _has_gpu():
        skip = pytest.mark.skip(reason="no CUDA GPU")
        for it in items:
            if "gpu" in it.keywords:
                it.add_marker(skip)
    from oracle import ref
    if not ref.available():
        skip = pytest.mark.skip(reason="reference checkout not present")
        for it in items:
            if "reference" in it.keywords:
                it.add_marker(skip)
