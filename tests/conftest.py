"""Shared fixtures.  GPU tests carry @pytest.mark.gpu; everything else runs on CPU."""
from __future__ import annotations

import ast
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
GOLDEN = Path(__file__).resolve().parent / "golden"
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

import __graft_entry__ as entry  # noqa: E402


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on the GB300 box)")


@pytest.fixture(scope="session")
def pkg():
    return entry.load_package()


@pytest.fixture(scope="session")
def abi(pkg):
    return pkg.abi


@pytest.fixture(scope="session")
def workloads(pkg):
    return entry.load_submodule("workloads")


@pytest.fixture(scope="session")
def oracle():
    from oracle import build_oracle
    build_oracle.build_oracle()
    from oracle.oracle import Oracle
    return Oracle()


def load_golden(name: str) -> dict:
    """Loads tests/golden/<name>.npz, restoring structured arrays."""
    z = np.load(GOLDEN / f"{name}.npz")
    out = {}
    for k in z.files:
        if k.endswith("__dtype"):
            continue
        if k + "__dtype" in z.files:
            dt = np.dtype(ast.literal_eval(str(z[k + "__dtype"])))
            out[k] = np.ascontiguousarray(z[k]).view(dt).reshape(-1)
        else:
            out[k] = z[k]
    return out


@pytest.fixture(scope="session")
def golden():
    return load_golden


@pytest.fixture(scope="session")
def cuda(pkg):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    entry.build()
    torch.cuda.set_device(0)
    return torch
