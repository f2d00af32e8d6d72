"""In-tree build of libpathguide.so (CUDA kernels + C ABI + C++ host code)
and of the C++ programs in app/.

Every CUDA translation unit is compiled for sm_103a only, in parallel, then
linked into one shared library next to this file.  The host scene code
(host/*.cpp) is compiled with g++ and linked into the same library; app/*.cpp
(drivers over include/pathguiding.hpp) become executables next to it.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent
CSRC = HERE / "csrc"
HOST = HERE / "host"
APP = HERE / "app"
BUILD = HERE / "_build"
LIB = HERE / "libpathguide.so"

NVCC = os.environ.get("NVCC", shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
              f"-I{ROOT / 'include'}", f"-I{CSRC}"]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", f"-I{ROOT / 'include'}", f"-I{HOST}"]
# Per-file extras.  The split/merge control arithmetic follows the reference's
# SSE2 build, which rounds every product and sum: no FMA contraction there.
FILE_FLAGS = {"pg_splitmerge.cu": ["-fmad=false"]}


def _sources():
    cu = sorted(CSRC.glob("*.cu"))
    cpp = sorted(HOST.glob("*.cpp")) if HOST.exists() else []
    headers = sorted(CSRC.glob("*.cuh")) + sorted(CSRC.glob("*.h")) + \
        (sorted(HOST.glob("*.h")) if HOST.exists() else []) + [ROOT / "include" / "pathguide.h"] + \
        sorted((ROOT / "include").glob("*.h"))
    return cu, cpp, headers


def _compile(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    return cmd, r.returncode, r.stdout + r.stderr


def build(force: bool = False, verbose: bool = False) -> Path:
    cu, cpp, headers = _sources()
    BUILD.mkdir(exist_ok=True)
    newest_header = max((h.stat().st_mtime for h in headers if h.exists()), default=0.0)
    jobs, objs = [], []
    for src in cu + cpp:
        obj = BUILD / (src.stem + (".cu.o" if src.suffix == ".cu" else ".cpp.o"))
        objs.append(obj)
        stale = force or not obj.exists() or obj.stat().st_mtime < max(src.stat().st_mtime, newest_header)
        if not stale:
            continue
        if src.suffix == ".cu":
            cmd = [NVCC] + ARCH + NVCC_FLAGS + FILE_FLAGS.get(src.name, []) + ["-c", str(src), "-o", str(obj)]
        else:
            cmd = ["g++"] + CXX_FLAGS + ["-c", str(src), "-o", str(obj)]
        jobs.append(cmd)
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            for cmd, rc, out in ex.map(_compile, jobs):
                if verbose or rc != 0:
                    sys.stderr.write(" ".join(cmd) + "\n" + out)
                if rc != 0:
                    raise RuntimeError(f"compile failed: {cmd[-3]}")
    relinked = False
    if force or jobs or not LIB.exists():
        cmd = [NVCC] + ARCH + ["-shared", "-o", str(LIB)] + [str(o) for o in objs] + \
            ["-lcudart", "-lstdc++"]
        cmd, rc, out = _compile(cmd)
        if rc != 0:
            sys.stderr.write(" ".join(cmd) + "\n" + out)
            raise RuntimeError("link of libpathguide.so failed")
        relinked = True
    build_apps(force or relinked, newest_header)
    return LIB


def build_apps(force: bool, newest_header: float) -> list[Path]:
    """C++ programs over the facades (app/*.cpp), linked against the library
    with an $ORIGIN run path so they run from the package directory."""
    bins = []
    for src in sorted(APP.glob("*.cpp")) if APP.exists() else []:
        exe = HERE / src.stem
        bins.append(exe)
        hpp = ROOT / "include" / "pathguiding.hpp"
        deps = max(src.stat().st_mtime, newest_header, hpp.stat().st_mtime if hpp.exists() else 0.0)
        if not force and exe.exists() and exe.stat().st_mtime >= deps:
            continue
        cmd = [NVCC, "-O2", "-std=c++17", f"-I{ROOT / 'include'}", str(src), "-o", str(exe), f"-L{HERE}",
               "-lpathguide", "-Xlinker", "-rpath", "-Xlinker", "$ORIGIN"]
        cmd, rc, out = _compile(cmd)
        if rc != 0:
            sys.stderr.write(" ".join(cmd) + "\n" + out)
            raise RuntimeError(f"build of {src.name} failed")
    return bins


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
