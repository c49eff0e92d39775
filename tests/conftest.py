"""Shared pytest setup: the ``gpu`` marker, import paths and lazily built libraries."""
from __future__ import annotations

import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "fluid-dynamics1_gb300")
for p in (ROOT, PKG, os.path.join(ROOT, "oracle"), os.path.dirname(os.path.abspath(__file__))):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and the built libcnv")


@pytest.fixture(scope="session")
def orc():
    import orc as _orc  # oracle/orc.py

    _orc.build()
    return _orc


@pytest.fixture(scope="session")
def cnv():
    """The product's ctypes binding with libcnv loaded; GPU tests only."""
    import cnvpy

    cnvpy.load()
    return cnvpy
