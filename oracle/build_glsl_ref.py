"""Build recipe: the reference's shader functions compiled as host C++
(TEST INFRASTRUCTURE).

The reference's tracer is GLSL run through Vulkan ray tracing; its shading,
sampling, guiding and recording functions are plain arithmetic and compile as
C++ once a few GLSL spellings are mapped (oracle/glsl_shim.hpp gives the types
and built-ins).  This recipe reads the shader files where they lie
(REFERENCE_ROOT/shaders), takes the cited line ranges, applies mechanical
rewrites only -

  * ``in`` parameter qualifiers dropped, ``out``/``inout T x`` become ``T &x``;
  * unsuffixed floating literals get an ``f`` suffix (GLSL literals are float);
  * a scalar swizzle ``(expr).xxx`` becomes ``xxx(expr)``;
  * ``T f = f(...)`` (a variable named after the function that initialises
    it, legal in GLSL) calls ``glsl::f`` by its qualified name;
  * each switch case's statements are put in braces (GLSL allows
    declarations between case labels);
  * ``#include`` / ``#version`` / ``#extension`` lines are dropped;

and writes oracle/_ref/glsl_ref_gen.cpp, which wraps the text in namespace
glsl between the shim and the project-written harness (glsl_ref_stubs.inc for
the globals the functions read, glsl_ref_harness.inc for the C exports).  The
result, oracle/_ref/libglslref.so, is the pinned oracle for the tracer's
shader math; it is built only where the reference tree is present.  No
reference file is modified and nothing of it is committed.
"""
from __future__ import annotations

import os
import re
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
REFERENCE_ROOT = Path(os.environ.get("PG_REFERENCE_ROOT", "/root/reference"))
SHADERS = REFERENCE_ROOT / "shaders"
OUT_DIR = HERE / "_ref"

# (file, first line, last line), 1-based inclusive, in compilation order.
PART_A = [
    ("limits.glsl", 1, 7),            # SIZE_LIGHT_RANDOM, MAX_DISTRIBUTIONS, MAX_DIRECTIONAL_DATA_PER_PIXEL
    ("raycommon.glsl", 1, 76),        # hitInfo, shadowCheck, pushConstant, sphere
    ("raycommon.glsl", 83, 103),      # cacheHeader, cacheData, cacheHits
    ("wavefront.glsl", 9, 45),        # Material, InstanceInfo, Light, FaceSample
    ("random_fwd.glsl", 1, 40),       # forward declarations of random.glsl
    ("transform_fwd.glsl", 1, 11),    # forward declarations of transform.glsl
    ("guiding.glsl", 5, 113),         # VMF_Theta, vMF, VMM_Theta, VMM, sampleVMF, sampleVMM, DirectionalData
    ("random.glsl", 3, 136),          # tea, lcg, rnd, the warps
    ("transform.glsl", 3, 42),        # coordinateAxis, toLocal, toWorld
    ("raytrace.rgen", 15, 53),        # material / light constants, tMin, tMax
    ("raytrace.rgen", 86, 93),        # ADRRS estimate, guiding sample sums
    ("raytrace.rgen", 144, 348),      # fresnel .. balanceHeuristic (BSDFs, pdfs, MIS heuristics)
    ("raytrace.rgen", 483, 599),      # sampleBSDF, evalBsdf
    ("raytrace.rgen", 733, 742),      # hasDiscreteDirection
]
PART_B = [
    ("raytrace.rgen", 806, 869),      # isICCapable, approxDiffuse, applyWeightWindow
    ("raytrace.rgen", 923, 990),      # getNewDirection, isMatAlmostDiscrete, getBaseIndex, updateSamples, commitSamples
]

_QUAL_OUT = re.compile(r"\b(?:out|inout)\s+(\w+)\s+(\w+)")
_QUAL_IN = re.compile(r"\bin\s+(\w+)\s+(\w+)")
_SIGNATURE = re.compile(r"^\s*\w+\s+\w+\s*\(.*\)\s*[{;]?\s*$")
_LABEL = re.compile(r"^\s*(case\s+[^:]+|default\s*):\s*$")
_SELF_INIT = re.compile(r"\b(\w+)\s+(\w+)\s*=\s*\2\s*\(")
_FLOAT_LIT = re.compile(r"(?<![\w.])((?:\d+\.\d*|\.\d+)(?:[eE][+-]?\d+)?|\d+[eE][+-]?\d+)(?![\w.])")


def _swizzle_xxx(line: str) -> str:
    """(expr).xxx -> xxx((expr)); name(args).xxx -> xxx(name(args))."""
    while ").xxx" in line:
        end = line.index(").xxx")
        depth, i = 0, end
        while i >= 0:
            if line[i] == ")":
                depth += 1
            elif line[i] == "(":
                depth -= 1
                if depth == 0:
                    break
            i -= 1
        start = i
        while start > 0 and (line[start - 1].isalnum() or line[start - 1] == "_"):
            start -= 1
        line = line[:start] + "xxx(" + line[start:end + 1] + ")" + line[end + 5:]
    return line


def _scope_cases(lines):
    """Braces around the statements of each switch case, so that C++ accepts
    the declarations GLSL allows between case labels."""
    out, depth, switches, open_case = [], 0, [], []
    for line in lines:
        code, sep, comment = line.partition("//")
        if _LABEL.match(code):
            if open_case and open_case[-1]:
                out.append("}")
            out.append(code.rstrip() + " {" + (" " + sep + comment if sep else ""))
            if open_case:
                open_case[-1] = True
            continue
        opens, closes = code.count("{"), code.count("}")
        if switches and closes and depth - closes <= switches[-1] and open_case[-1]:
            out.append("}")
            open_case[-1] = False
        if re.match(r"^\s*switch\s*\(", code):
            switches.append(depth)
            open_case.append(False)
        depth += opens - closes
        if switches and depth <= switches[-1] and closes:
            switches.pop()
            open_case.pop()
        out.append(line)
    return out


def transform(text: str) -> str:
    out = []
    for line in _scope_cases(text.splitlines()):
        s = line.strip()
        if s.startswith("#include") or s.startswith("#version") or s.startswith("#extension"):
            out.append("")
            continue
        if _SIGNATURE.match(line):
            line = _QUAL_OUT.sub(r"\1 &\2", line)
            line = _QUAL_IN.sub(r"\1 \2", line)
        if not s.startswith("//"):
            code, sep, comment = line.partition("//")
            code = _FLOAT_LIT.sub(lambda m: m.group(1) + "f", code)
            code = _swizzle_xxx(code)
            code = _SELF_INIT.sub(lambda m: f"{m.group(1)} {m.group(2)} = glsl::{m.group(2)}(", code)
            line = code + sep + comment
        out.append(line)
    return "\n".join(out)


def _excerpt(parts) -> str:
    chunks = []
    for name, a, b in parts:
        lines = (SHADERS / name).read_text().splitlines()
        chunks.append(f"#line {a} \"{name}\"\n" + transform("\n".join(lines[a - 1:b])))
    return "\n".join(chunks)


def generate() -> Path:
    OUT_DIR.mkdir(exist_ok=True)
    src = "\n".join([
        "// Generated by oracle/build_glsl_ref.py from the reference's shaders; not committed.",
        '#include "glsl_shim.hpp"',
        "namespace glsl {",
        "int textureSamplers[64];",
        _excerpt(PART_A),
        '#line 1 "glsl_ref_stubs.inc"',
        '#include "glsl_ref_stubs.inc"',
        _excerpt(PART_B),
        "}  // namespace glsl",
        '#include "glsl_ref_harness.inc"',
        "",
    ])
    out = OUT_DIR / "glsl_ref_gen.cpp"
    if not out.exists() or out.read_text() != src:
        out.write_text(src)
    return out


def build_glsl_ref(force: bool = False):
    if not (SHADERS / "raytrace.rgen").exists():
        return None
    gen = generate()
    lib = OUT_DIR / "libglslref.so"
    deps = [gen, HERE / "glsl_shim.hpp", HERE / "glsl_ref_stubs.inc", HERE / "glsl_ref_harness.inc",
            Path(__file__)]
    if force or not lib.exists() or any(d.stat().st_mtime > lib.stat().st_mtime for d in deps):
        cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-fpermissive", "-w",
               f"-I{HERE}", f"-I{HERE.parent / 'include'}", str(gen), "-o", str(lib)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
            raise RuntimeError("build of the reference shader functions failed")
    return lib


if __name__ == "__main__":
    print(build_glsl_ref(force=True))
