"""Test configuration: the `gpu` marker and import paths.

Tests marked gpu need a CUDA device and run the library through its C ABI;
everything else runs on the CPU (the oracle, the host-side setup, the ABI
symbol table).
"""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG_DIR = os.path.join(ROOT, "multall-open-18.3_gb300")
ORACLE_DIR = os.path.join(ROOT, "oracle")
for p in (PKG_DIR, ORACLE_DIR, ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a library)")
