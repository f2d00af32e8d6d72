"""Build recipe for the oracle libraries (TEST INFRASTRUCTURE).

* ``oracle/liboracle.so`` - the plain-C restatement (pg_oracle.c, and the
  tracer restatement pg_oracle_trace.cpp), built on whichever machine runs it.
* ``oracle/_ref/liblightpmm_ref.so`` - the reference's own vendored lightpmm fit
  compiled from its sources where they lie (REFERENCE_ROOT), through
  lightpmm_harness.cpp and a project-written glm stand-in (glm_shim/).  It is
  built only when the reference tree is present and the host is x86-64 (the
  vendored vectorclass library has no other SIMD back end); its flags are the
  reference's own (CMakeLists.txt: C++20, -O4, no -march).
"""
from __future__ import annotations

import os
import platform
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent
REFERENCE_ROOT = Path(os.environ.get("PG_REFERENCE_ROOT", "/root/reference"))


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        sys.stderr.write(" ".join(map(str, cmd)) + "\n" + r.stdout + r.stderr)
        raise RuntimeError(f"oracle build failed: {cmd[0]}")


def _stale(out: Path, srcs) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(Path(s).stat().st_mtime > t for s in srcs)


def build_oracle(force: bool = False) -> Path:
    out = HERE / "liboracle.so"
    srcs = [HERE / "pg_oracle.c", HERE / "pg_oracle.h", ROOT / "include" / "pathguide.h"]
    trace_src = HERE / "pg_oracle_trace.cpp"
    objs = []
    if trace_src.exists():
        srcs += [trace_src, HERE / "pg_oracle_trace.h"]
    if force or _stale(out, srcs):
        build = HERE / "_build"
        build.mkdir(exist_ok=True)
        c_obj = build / "pg_oracle.o"
        _run(["gcc", "-std=gnu11", "-O2", "-ffp-contract=off", "-fPIC", "-pthread",
              f"-I{ROOT / 'include'}", "-c", str(HERE / "pg_oracle.c"), "-o", str(c_obj)])
        objs.append(c_obj)
        if trace_src.exists():
            t_obj = build / "pg_oracle_trace.o"
            _run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fPIC", "-pthread",
                  f"-I{ROOT / 'include'}", f"-I{HERE}", "-c", str(trace_src), "-o", str(t_obj)])
            objs.append(t_obj)
        _run(["g++", "-shared", "-pthread", "-o", str(out)] + [str(o) for o in objs] + ["-lm"])
    return out


def build_reference(force: bool = False):
    """Compile the reference's lightpmm fit into oracle/_ref (x86-64 hosts with the tree only)."""
    inc = REFERENCE_ROOT / "external" / "lightpmm" / "include"
    if not inc.exists() or platform.machine() not in ("x86_64", "AMD64"):
        return None
    out_dir = HERE / "_ref"
    out_dir.mkdir(exist_ok=True)
    out = out_dir / "liblightpmm_ref.so"
    srcs = [HERE / "lightpmm_harness.cpp", ROOT / "include" / "pathguide.h"]
    if force or _stale(out, srcs):
        _run(["g++", "-std=c++20", "-O3", "-fPIC", "-shared", "-w",
              f"-I{HERE / 'glm_shim'}", f"-I{inc}", f"-I{REFERENCE_ROOT / 'external'}",
              f"-I{ROOT / 'include'}", str(HERE / "lightpmm_harness.cpp"), "-o", str(out)])
    return out


if __name__ == "__main__":
    print(build_oracle(force=True))
    print(build_reference(force=True))
