"""Test configuration: package loader, marker registration, build on demand.

Tests marked ``gpu`` need a CUDA device (a GB300); the rest run on the CPU:
the oracle against the reference's golden vectors, the case generator, the
host-side logic and the C ABI's exports.
"""
import os
import subprocess
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if REPO not in sys.path:
    sys.path.insert(0, REPO)

import __graft_entry__ as ge  # noqa: E402

ge.load_package()


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs through the C ABI on cuda:0)")


def _ensure_built():
    import importlib
    lib_dir = os.path.join(REPO, "openfoam-dev_gb300", "lib")
    if not (os.path.exists(os.path.join(lib_dir, "libcudaLduSolvers.so"))
            and os.path.exists(os.path.join(lib_dir, "libcfxcase.so"))):
        importlib.import_module("openfoam_dev_gb300.build").build()
    if not all(os.path.exists(os.path.join(REPO, "oracle", "_build", f))
               for f in ("libldu_oracle.so", "libldu_oracle_timed.so")):
        subprocess.run(["make", "-s", "-C", os.path.join(REPO, "oracle")], check=True)


_ensure_built()
