"""The C-ABI library loads on CPU and exports every function include/*.h declares."""
from __future__ import annotations

import ctypes
import re
from pathlib import Path

import numpy as np
import pytest

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


def _c_layout(pairs):
    """sizeof / offsetof of header structs, compiled from include/pathguide.h with gcc."""
    import shutil
    import subprocess
    import tempfile
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "pathguide.h"', "int main(void) {"]
    for struct, fields in pairs:
        lines.append(f'printf("{struct} %zu\\n", sizeof({struct}));')
        for f in fields:
            lines.append(f'printf("{struct}.{f} %zu\\n", offsetof({struct}, {f}));')
    lines.append("return 0; }")
    with tempfile.TemporaryDirectory() as d:
        src, exe = Path(d) / "layout.c", Path(d) / "layout"
        src.write_text("\n".join(lines))
        subprocess.run([cc, "-std=c11", "-I", str(ROOT / "include"), str(src), "-o", str(exe)], check=True)
        out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    return {k: int(v) for k, v in (ln.split() for ln in out.splitlines())}


def test_ctypes_mirrors_match_the_header(abi):
    structs = [("pg_fit_config", abi.FitConfig), ("pg_fit_tuning", abi.FitTuning), ("pg_camera", abi.Camera),
               ("pg_cornell_params", abi.CornellParams), ("pg_plates_params", abi.PlatesParams),
               ("pg_scene_info", abi.SceneInfo), ("pg_render_params", abi.RenderParams),
               ("pg_render_stats", abi.RenderStats), ("pg_mlp_config", abi.MlpConfig),
               ("pg_split_merge_config", abi.SplitMergeConfig), ("pg_region_split_config", abi.RegionSplitConfig)]
    dtypes = [("pg_region_state", abi.STATE_DTYPE), ("pg_vmm_theta", abi.VMM_THETA_DTYPE),
              ("pg_vmf_theta", abi.VMF_THETA_DTYPE), ("pg_material", abi.MATERIAL_DTYPE),
              ("pg_sphere", abi.SPHERE_DTYPE), ("pg_ray", abi.RAY_DTYPE), ("pg_hit", abi.HIT_DTYPE),
              ("pg_region_extra", abi.EXTRA_DTYPE)]
    pairs = [(n, [f[0] for f in t._fields_]) for n, t in structs] + [(n, list(dt.names)) for n, dt in dtypes]
    got = _c_layout(pairs)
    for n, t in structs:
        assert got[n] == ctypes.sizeof(t), n
        for f in t._fields_:
            assert got[f"{n}.{f[0]}"] == getattr(t, f[0]).offset, f"{n}.{f[0]}"
    for n, dt in dtypes:
        assert got[n] == dt.itemsize, n
        for f in dt.names:
            assert got[f"{n}.{f}"] == dt.fields[f][1], f"{n}.{f}"
