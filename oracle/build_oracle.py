"""Build recipe for the oracle libraries (TEST INFRASTRUCTURE).

* ``oracle/liboracle.so`` - the plain-C restatement (pg_oracle.c, and the
  tracer restatement pg_oracle_trace.cpp), built on whichever machine runs it.
* ``oracle/_ref/liblightpmm_ref.so`` - the reference's own vendored lightpmm fit
  compiled through lightpmm_harness.cpp and a project-written glm stand-in
  (glm_shim/), with the reference's flags (CMakeLists.txt: C++20, -O4, no
  -march).  Where the reference tree is present its lightpmm and guiding
  headers are read where they lie, and also staged (copied, not committed:
  oracle/_ref is git-ignored) into oracle/_ref/src so that a host without the
  tree - the Arm GPU host - can build the same fit.  On x86-64 with the tree
  the build uses the vendored vectorclass library (SSE); elsewhere it uses the
  project-written portable stand-in for that library (vcl_shim/: lane loops,
  and SSE type stand-ins on hosts without x86 intrinsics), which
  ``oracle/_ref/liblightpmm_ref_portable.so`` also builds on x86-64 so the two
  can be compared.
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


STAGED = HERE / "_ref" / "src"
X86 = platform.machine() in ("x86_64", "AMD64")


def stage_reference_sources():
    """Copies the reference's lightpmm and guiding headers into oracle/_ref/src
    (where the tree is present); returns the staged directory, or None."""
    pmm = REFERENCE_ROOT / "external" / "lightpmm" / "include" / "pmm"
    guiding = REFERENCE_ROOT / "external" / "guiding"
    if pmm.exists() and guiding.exists():
        for src_dir, name in ((pmm, "pmm"), (guiding, "guiding")):
            dst = STAGED / name
            dst.mkdir(parents=True, exist_ok=True)
            for f in sorted(src_dir.glob("*.h")):
                t = dst / f.name
                data = f.read_bytes()
                if not t.exists() or t.read_bytes() != data:
                    t.write_bytes(data)
    return STAGED if (STAGED / "pmm" / "VMMFactory.h").exists() else None


def _build_lightpmm(out: Path, include_dirs, force: bool):
    srcs = [HERE / "lightpmm_harness.cpp", ROOT / "include" / "pathguide.h"]
    if force or _stale(out, srcs + sorted((HERE / "vcl_shim").rglob("*.h"))):
        _run(["g++", "-std=c++20", "-O3", "-ffp-contract=off", "-fPIC", "-shared", "-pthread", "-w"] +
             [f"-I{d}" for d in include_dirs] +
             [f"-I{ROOT / 'include'}", str(HERE / "lightpmm_harness.cpp"), "-o", str(out)])
    return out


def build_reference(force: bool = False):
    """Compile the reference's lightpmm fit into oracle/_ref: from the tree
    with its vectorclass on x86-64, else from the staged headers with the
    portable vectorclass stand-in (the Arm host).  None if neither source is
    there."""
    staged = stage_reference_sources()
    inc = REFERENCE_ROOT / "external" / "lightpmm" / "include"
    out_dir = HERE / "_ref"
    out_dir.mkdir(exist_ok=True)
    shim = [HERE / "vcl_shim"] + ([] if X86 else [HERE / "vcl_shim" / "noarch"])
    if inc.exists() and X86:
        out = _build_lightpmm(out_dir / "liblightpmm_ref.so",
                              [HERE / "glm_shim", inc, REFERENCE_ROOT / "external"], force)
        _build_lightpmm(out_dir / "liblightpmm_ref_portable.so", shim + [HERE / "glm_shim", staged], force)
        return out
    if staged is not None:
        return _build_lightpmm(out_dir / "liblightpmm_ref.so", shim + [HERE / "glm_shim", staged], force)
    return None


if __name__ == "__main__":
    print(build_oracle(force=True))
    print(build_reference(force=True))
