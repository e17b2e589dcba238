"""Test configuration: marker registration and import paths.

``-m "not gpu"`` runs the oracle-vs-golden checks, host-side logic and the
C-ABI symbol checks (no GPU needed); ``-m gpu`` runs the parity tests that
call the CUDA path through the C-ABI and compare it with the oracle.
"""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG_DIR = os.path.join(ROOT, "pennylane-lightning-kokkos_gb300")
for p in (ROOT, PKG_DIR, os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests", "golden")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
