"""Shared test set-up: import paths, the ``gpu`` marker and common meshes."""
from __future__ import annotations

import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
PKG = ROOT / "boundaryintegralequations.jl_gb300"
for p in (str(PKG), str(ROOT)):
    if p not in sys.path:
        sys.path.insert(0, p)

# The reference's COMSOL mesh fixtures (its examples/meshes folder) are read in
# place where a checkout of the reference is available (CPU tests only): the
# folder named by BIE_REFERENCE_MESHES, else examples/meshes of a checkout
# named "reference" beside this repository.  Tests that need them skip
# otherwise.
REFERENCE_MESHES = Path(os.environ.get("BIE_REFERENCE_MESHES")
                        or ROOT.parent / "reference" / "examples" / "meshes")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def pytest_collection_modifyitems(config, items):
    # keep files in name order so test_zz_* files run last
    items.sort(key=lambda it: (Path(str(it.fspath)).name, 0))


@pytest.fixture(scope="session")
def reference_meshes():
    if not REFERENCE_MESHES.exists():
        pytest.skip("reference mesh fixtures not mounted")
    return REFERENCE_MESHES


def rel_fro(a, b):
    import numpy as np
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))
