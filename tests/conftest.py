"""Shared pytest set-up: the ``gpu`` marker and on-demand builds.

CPU-only runs (``-m "not gpu"``) build the oracle and the product library
(cross-compiled for sm_103a; nothing is launched).  GPU runs build the same
on the box they run on.
"""
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "lbm-2d_gb300")
for p in (ROOT, PKG, os.path.join(ROOT, "tests", "golden")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle import oracle as O
    if not os.path.exists(O.LIB_ORACLE):
        O.build()
    return O


@pytest.fixture(scope="session")
def product():
    """The product library, built in-tree if missing."""
    import lbm2d
    lbm2d.build(quiet=True)
    return lbm2d


def has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False
