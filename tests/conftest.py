"""Test configuration: registers the ``gpu`` marker and makes the package
``elas3d-xtal_gb300/`` importable as ``elas3d_xtal_gb300`` and the oracle as
``oracle`` (test infrastructure)."""
import importlib.util
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG_DIR = os.path.join(ROOT, "elas3d-xtal_gb300")


def load_package():
    if "elas3d_xtal_gb300" in sys.modules:
        return sys.modules["elas3d_xtal_gb300"]
    spec = importlib.util.spec_from_file_location(
        "elas3d_xtal_gb300", os.path.join(PKG_DIR, "__init__.py"), submodule_search_locations=[PKG_DIR])
    mod = importlib.util.module_from_spec(spec)
    sys.modules["elas3d_xtal_gb300"] = mod
    spec.loader.exec_module(mod)
    return mod


load_package()
if os.path.join(ROOT, "oracle") not in sys.path:
    sys.path.insert(0, os.path.join(ROOT, "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def pytest_collection_modifyitems(config, items):
    if _has_gpu():
        return
    skip = pytest.mark.skip(reason="no CUDA device")
    for item in items:
        if "gpu" in item.keywords:
            item.add_marker(skip)
