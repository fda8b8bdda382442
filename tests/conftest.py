"""Test configuration.

Markers: `gpu` tests need a CUDA device (a GB300) and call the product
through its C ABI; everything else runs on the CPU (oracle against the golden
fixtures, host logic, file formats, ABI symbol table).
"""
import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the built sm_103a extension")
    # The extension and the oracle are built once per session (content-stamped).
    # build.py is loaded by path: importing the package itself needs the library.
    import importlib.util

    spec = importlib.util.spec_from_file_location("pm_build", ROOT / "pattenmatching_sharedmemory_gb300" / "build.py")
    pkg_build = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(pkg_build)
    pkg_build.build()
    from oracle import oracle

    oracle.build()


def _have_gpu() -> bool:
    import pattenmatching_sharedmemory_gb300 as pm

    return pm.device_count() > 0


def pytest_collection_modifyitems(config, items):
    if _have_gpu():
        return
    skip = pytest.mark.skip(reason="no CUDA device")
    for item in items:
        if "gpu" in item.keywords:
            item.add_marker(skip)
