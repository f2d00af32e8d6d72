"""The C-ABI library loads on CPU and exports every function include/*.h declares."""
from __future__ import annotations

import ctypes
import re
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[1]


def declared_functions():
    names = set()
    for h in sorted((ROOT / "include").glob("*.h")):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        for m in re.finditer(r"^\s*(?:[A-Za-z_][\w\s\*]*?)\b(pg\w+)\s*\(", text, flags=re.M):
            names.add(m.group(1))
    return sorted(names)


def test_header_declares_entry_points():
    names = declared_functions()
    assert "pg_fit_regions" in names and "pg_ctx_create" in names
    assert len(names) >= 15


def test_library_exports_every_declared_symbol(pkg):
    lib = pkg.library()
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, f"not exported: {missing}"


def test_bindings_cover_every_declared_symbol(pkg):
    missing = [n for n in declared_functions() if n not in pkg.SIGNATURES]
    assert not missing, f"no ctypes signature for: {missing}"


def test_host_only_entry_points(pkg, abi):
    lib = pkg.library()
    cfg = abi.FitConfig()
    lib.pg_default_fit_config(ctypes.byref(cfg))
    # VMMFactoryProperties defaults with PathGuiding's overrides
    assert cfg.num_initial_components == 8 and cfg.max_itr == 100 and cfg.max_kappa == 50000.0
    assert abs(cfg.rel_ll_threshold - 0.005) < 1e-9 and cfg.min_itr == 1
    assert lib.pg_status_string(abi.PG_ERR_TIMEOUT) == b"PG_ERR_TIMEOUT"
    # argument errors are reported without touching a device
    assert lib.pg_ctx_create(None, 1, 0, ctypes.byref(ctypes.c_void_p())) == abi.PG_ERR_ARG
    bad = abi.default_fit_config(num_initial_components=17)
    assert lib.pg_ctx_create(ctypes.byref(bad), 1, 0, ctypes.byref(ctypes.c_void_p())) == abi.PG_ERR_ARG
    assert b"num_initial_components" in lib.pg_last_error(None)
    assert lib.pg_ctx_destroy(None) == abi.PG_OK


def test_struct_layouts(abi):
    assert abi.STATE_DTYPE.itemsize == 704
    assert abi.VMM_THETA_DTYPE.itemsize == 720
    assert ctypes.sizeof(abi.FitConfig) == 40
    rec = np.zeros(1, dtype=np.dtype([("position", "<f4", (3,)), ("direction", "<f4", (3,)),
                                      ("weight", "<f4"), ("pdf", "<f4"), ("distance", "<f4"),
                                      ("flags", "<u4")]))
    assert rec.itemsize == 40
