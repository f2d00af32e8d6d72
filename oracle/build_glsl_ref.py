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
  * a scalar swizzle ``(expr).xxx`` becomes ``xxx(expr)``, and the identity
    swizzle ``origin.xyz`` / ``direction.xyz`` / ``normal.xyz`` of a vec3 the
    vec3 itself;
  * ``T f = f(...)`` (a variable named after the function that initialises
    it, legal in GLSL) calls ``glsl::f`` by its qualified name;
  * each switch case's statements are put in braces (GLSL allows
    declarations between case labels);
  * variables declared at file scope become ``thread_local`` (each shader
    invocation has its own), and a shader's ``main()`` body becomes a named
    function;
  * an identifier swizzle ``name.xxx`` becomes ``xxx(name)`` too;
  * in the irradiance cache's intersection shader its buffer name
    ``spheres`` becomes ``cacheSpheres`` (the name raytrace.rgen binds the
    same buffer under), and in its any-hit shader the local ``E`` becomes
    ``E_`` (raytrace.rgen defines a macro ``E``, which the separately
    compiled shader does not see);
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
    ("raycommon.glsl", 78, 81),       # aabb
    ("raycommon.glsl", 83, 103),      # cacheHeader, cacheData, cacheHits
    ("wavefront.glsl", 1, 45),        # Vertex, Material, InstanceInfo, Light, FaceSample
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
# the estimator: the per-invocation state of the ray-generation shader, the
# hit / miss shaders (their main() bodies become the named functions) and the
# path loop with next-event estimation
PART_C_STATE = [
    ("raytrace.rgen", 56, 84),        # ray flags, new irradiance-cache entries, the split queue
]
# the irradiance cache's any-hit helpers, after the cache buffers (glsl_ref_scene.inc)
PART_IC_HELPERS = [
    ("raytrace.irradiance.rahit", 18, 25),  # irradianceWeight, visibilityCheck
]
# (file, first, last, function name[, renames]): a renamed identifier is a
# buffer the shader binds under another name than raytrace.rgen does (binding
# 12 is `spheres` in the cache's intersection shader, `cacheSpheres` in
# raytrace.rgen:118), or a local variable named like a macro of
# raytrace.rgen (`E`, :19), which a separate shader does not see
SHADERS_AS_FUNCTIONS = [
    ("raytrace.rchit", 17, 58, "closestHitTriangle"),
    ("raytrace.sphere.rchit", 14, 35, "closestHitSphere"),
    ("raytrace.rmiss", 16, 30, "missShader"),
    ("raytrace.shadow.rmiss", 8, 10, "shadowMissShader"),
    ("raytrace.irradiance.rint", 13, 20, "icIntersectionShader", {"spheres": "cacheSpheres"}),
    ("raytrace.irradiance.rahit", 28, 50, "icAnyHitShader", {"E": "E_"}),
]
PART_C = [
    ("raytrace.rgen", 358, 473),      # sampleLights
    ("raytrace.rgen", 601, 731),      # nextEventEstimation
    ("raytrace.rgen", 745, 804),      # queryIrradianceCache(Gradients)
    ("raytrace.rgen", 871, 902),      # multipleNEE, split
    ("raytrace.rgen", 992, 1226),     # raytrace: the path loop, NEE, guiding, sample recording
    ("raytrace.rgen", 1231, 1421),    # calculateCacheData, clampGradients, update- / createIrradianceCache
]

_QUAL_OUT = re.compile(r"\b(?:out|inout)\s+(\w+)\s+(\w+)")
_QUAL_IN = re.compile(r"\bin\s+(\w+)\s+(\w+)")
_SIGNATURE = re.compile(r"^\s*\w+\s+\w+\s*\(.*\)\s*[{;]?\s*$")
_LABEL = re.compile(r"^\s*(case\s+[^:]+|default\s*):\s*$")
_NAME_XXX = re.compile(r"\b([A-Za-z_]\w*)\.xxx\b")
_VEC3_XYZ = re.compile(r"\b(origin|direction|normal)\.xyz\b")
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


_GLOBAL_VAR = re.compile(r"^(?!\s*(?:const|struct|return|#|typedef)\b)(\w+\s+\w+\s*(?:\[[^\]]*\])?\s*(?:=[^;]*)?;)\s*$")


def _thread_local_globals(lines):
    out, depth = [], 0
    for line in lines:
        code = line.partition("//")[0]
        if depth == 0 and _GLOBAL_VAR.match(code) and "(" not in code:
            line = "thread_local " + line
        depth += code.count("{") - code.count("}")
        out.append(line)
    return out


def transform(text: str) -> str:
    out = []
    for line in _thread_local_globals(_scope_cases(text.splitlines())):
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
            code = _NAME_XXX.sub(r"xxx(\1)", code)
            code = _VEC3_XYZ.sub(r"\1", code)
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


def _shaders_as_functions() -> str:
    chunks = []
    for name, a, b, fn, *rest in SHADERS_AS_FUNCTIONS:
        lines = (SHADERS / name).read_text().splitlines()
        body = "\n".join(lines[a - 1:b])
        for old, new in (rest[0] if rest else {}).items():
            body = re.sub(rf"\b{old}\b", new, body)
        chunks.append(f"void {fn}() {{\n#line {a} \"{name}\"\n" + transform(body) + "\n}")
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
        _excerpt(PART_C_STATE),
        '#line 1 "glsl_ref_scene.inc"',
        '#include "glsl_ref_scene.inc"',
        _excerpt(PART_IC_HELPERS),
        _shaders_as_functions(),
        _excerpt(PART_C),
        "}  // namespace glsl",
        '#include "glsl_ref_harness.inc"',
        '#include "glsl_ref_render.inc"',
        "",
    ])
    out = OUT_DIR / "glsl_ref_gen.cpp"
    if not out.exists() or out.read_text() != src:
        out.write_text(src)
    return out


def build_glsl_ref(force: bool = False):
    if not (SHADERS / "raytrace.rgen").exists():
        return None
    import importlib.util
    spec = importlib.util.spec_from_file_location("_pg_oracle_build", HERE / "build_oracle.py")
    ob = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(ob)
    ob.build_oracle()  # the traversal twin the estimator's ray queries run on
    gen = generate()
    lib = OUT_DIR / "libglslref.so"
    deps = [gen, HERE / "glsl_shim.hpp", HERE / "glsl_ref_stubs.inc", HERE / "glsl_ref_harness.inc",
            HERE / "glsl_ref_scene.inc", HERE / "glsl_ref_render.inc", HERE / "liboracle.so", Path(__file__)]
    if force or not lib.exists() or any(d.stat().st_mtime > lib.stat().st_mtime for d in deps):
        cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-fpermissive", "-w", "-pthread",
               f"-I{HERE}", f"-I{HERE.parent / 'include'}", str(gen), "-o", str(lib),
               f"-L{HERE}", "-loracle", "-Wl,-rpath,$ORIGIN/.."]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
            raise RuntimeError("build of the reference shader functions failed")
    return lib


if __name__ == "__main__":
    print(build_glsl_ref(force=True))
