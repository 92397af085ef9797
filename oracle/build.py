"""Build recipe for the CPU oracle and for the reference shaders compiled as C++.

TEST INFRASTRUCTURE ONLY: the tests, the smoke check and the benchmark's CPU
baseline leg load what this builds; the CUDA library never does.

* ``build_oracle()`` compiles ``oracle/cf_oracle.cpp`` (the restatement) into
  ``oracle/_build/libcf_oracle.so`` with ``g++ -O2 -ffp-contract=off -fopenmp``.
* ``generate_ref(shader_root)`` reads the reference's shaders where they lie
  and rewrites them mechanically into ``oracle/_ref/ref_shaders_gen.cpp``
  (git-ignored):

  - the three compute shaders ``ClusteredForward/AABBGenerator.comp``,
    ``ClusteredForward/LightCulling.comp`` and ``FrustumCulling.comp``, whole:
    ``#include`` lines are expanded, ``#version`` and the ``local_size`` layout
    are dropped, each interface block becomes a namespace-scope variable,
    unsuffixed float literals get an ``f`` (GLSL literals are single
    precision) and ``.xyz`` becomes a call;
  - from ``ClusteredForward/Scene.frag``, the declarations and statements of
    the clustered lookup and the direct lighting: the includes they need
    (``Radiance.glsl``, ``PBR/PBRHeader.glsl`` and the record headers; the
    texture, normal-map and IBL headers are left out), the interface blocks
    they read, the ``worldPos`` input, ``LinearDepth``, and main's statements
    from ``float linDepth`` to ``lightIndexOffset`` (the lookup) and from
    ``alphaRoughness`` through the light loop (the lighting), each found by
    its pattern and wrapped in a function of its own.  A pattern that no
    longer matches exactly once is an error, so a changed shader fails loudly.

  Everything else is the shaders' own text, compiled against
  ``oracle/glsl_compat.h`` and driven by ``oracle/ref_driver.inc``.
* ``build_ref()`` compiles that generated file into ``oracle/_ref/libcf_ref.so``.
  It needs only the generated file, so it also runs where the reference
  checkout is absent, as long as the file was generated beforehand.

The shader root is the ``--shaders`` argument, else the ``CF_REF_SHADERS``
environment variable, else ``HelloVulkan/Shaders`` of a ``reference`` checkout
beside this repository.
"""
from __future__ import annotations

import os
import re
import subprocess
import sys
from pathlib import Path

ORACLE_DIR = Path(__file__).resolve().parent
REPO = ORACLE_DIR.parent
BUILD_DIR = ORACLE_DIR / "_build"
REF_DIR = ORACLE_DIR / "_ref"
ORACLE_SO = BUILD_DIR / "libcf_oracle.so"
REF_SRC = REF_DIR / "ref_shaders_gen.cpp"
REF_SO = REF_DIR / "libcf_ref.so"


def default_shader_root() -> Path:
    """The reference's shader directory: $CF_REF_SHADERS, else a checkout named
    ``reference`` beside this repository."""
    env = os.environ.get("CF_REF_SHADERS")
    if env:
        return Path(env)
    return REPO.parent / "reference" / "HelloVulkan" / "Shaders"


CXXFLAGS = ["-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math", "-fopenmp"]

SHADERS = (
    ("aabbgen", "ClusteredForward/AABBGenerator.comp"),
    ("lightcull", "ClusteredForward/LightCulling.comp"),
    ("frustum", "FrustumCulling.comp"),
)
SCENE_FRAG = "ClusteredForward/Scene.frag"
# Scene.frag's includes that the lookup and the direct lighting do not use:
# bindless texture records, Hammersley sampling, normal mapping (screen-space
# derivatives) and the IBL ambient term (cube-map sampling).
SCENE_SKIPPED_INCLUDES = ("Bindless/", "PBR/Hammersley.glsl", "PBR/NormalTBN.glsl", "PBR/Ambient.glsl")
# the interface blocks the lookup and the lighting read
SCENE_BLOCKS = ("pc", "camUBO", "cfUBO", "lights", "lightCells", "lightIndices")


def _stale(target: Path, sources) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(Path(s).stat().st_mtime > t for s in sources)


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: %s\n%s%s" % (" ".join(map(str, cmd)), r.stdout, r.stderr))


def build_oracle(force: bool = False) -> Path:
    src = ORACLE_DIR / "cf_oracle.cpp"
    deps = [src, REPO / "include" / "cf_types.h", REPO / "include" / "cf_pinned_math.h"]
    if force or _stale(ORACLE_SO, deps):
        BUILD_DIR.mkdir(parents=True, exist_ok=True)
        tmp = ORACLE_SO.with_suffix(".so.tmp%d" % os.getpid())
        _run(["g++", *CXXFLAGS, "-I", str(REPO / "include"), str(src), "-o", str(tmp)])
        os.replace(tmp, ORACLE_SO)
    return ORACLE_SO


_INCLUDE = re.compile(r'^\s*#\s*include\s*[<"]([^>"]+)[>"]\s*$', re.M)
_VERSION = re.compile(r"^\s*#\s*version[^\n]*$", re.M)
_EXTENSION = re.compile(r"^\s*#\s*extension[^\n]*$", re.M)
_LOCAL_SIZE = re.compile(r"layout\s*\([^)]*\)\s*in\s*;")
_BLOCK = re.compile(
    r"layout\s*\([^)]*\)\s*((?:readonly|writeonly|coherent|restrict)\s+)*(buffer|uniform)\s+\w+\s*"
    r"\{\s*(\w+)\s+(\w+)\s*(\[\s*\])?\s*;\s*\}\s*;")
_FLOAT_LIT = re.compile(r"(?<![\w.])(\d+\.\d*|\.\d+)(?![\w.])")
_SWIZZLE_XYZ = re.compile(r"\.xyz\b(?!\s*\()")


def _expand_includes(text: str, root: Path, seen=None) -> str:
    seen = set() if seen is None else seen

    def sub(m):
        p = (root / m.group(1)).resolve()
        if p in seen:
            return ""
        seen.add(p)
        return _expand_includes(p.read_text(), root, seen) + "\n"

    return _INCLUDE.sub(sub, text)


def _block(m) -> str:
    type_, name, arr = m.group(3), m.group(4), m.group(5)
    return ("static Buffer<%s> %s;" % (type_, name)) if arr else ("static %s %s;" % (type_, name))


def _literals(text: str) -> str:
    text = _FLOAT_LIT.sub(lambda m: m.group(1) + "f", text)
    return _SWIZZLE_XYZ.sub(".xyz()", text)


def transform_shader(text: str, root: Path) -> str:
    text = _expand_includes(text, root)
    text = _VERSION.sub("", text)
    text = _EXTENSION.sub("", text)
    text = _LOCAL_SIZE.sub("", text)
    text = _BLOCK.sub(_block, text)
    return _literals(text)


_FRAG_INPUT = re.compile(r"layout\s*\([^)]*\)\s*in\s+(vec2|vec3|vec4|float)\s+(\w+)\s*;")
_LAYOUT_LINE = re.compile(r"^[ \t]*layout\s*\(.*?;[^\n]*$", re.M)
_MAIN = re.compile(r"\bvoid\s+main\s*\(\s*\)")


def _once(pattern: str, text: str, what: str, flags=0) -> str:
    found = re.findall(pattern, text, flags)
    if len(found) != 1:
        raise RuntimeError("Scene.frag: %d matches for %s (expected 1)" % (len(found), what))
    return found[0]


def _balanced(text: str, start: int) -> int:
    """Index just past the brace block opening at or after `start`."""
    i = text.index("{", start)
    depth = 0
    for j in range(i, len(text)):
        if text[j] == "{":
            depth += 1
        elif text[j] == "}":
            depth -= 1
            if depth == 0:
                return j + 1
    raise RuntimeError("Scene.frag: unbalanced braces")


def scene_fragment_source(text: str, root: Path) -> str:
    """The clustered lookup and direct lighting of Scene.frag as C++ (see the
    module docstring): declarations in file order, then two functions."""
    m = _MAIN.search(text)
    if not m:
        raise RuntimeError("Scene.frag: no main()")
    head, body = text[:m.start()], text[m.start():]

    def include(mi):
        name = mi.group(1)
        if name.startswith(SCENE_SKIPPED_INCLUDES):
            return ""
        return _expand_includes(mi.group(0), root)

    head = _INCLUDE.sub(include, head)
    head = _VERSION.sub("", head)
    head = _EXTENSION.sub("", head)
    head = _BLOCK.sub(lambda mb: _block(mb) if mb.group(4) in SCENE_BLOCKS else "", head)
    head = _FRAG_INPUT.sub(lambda mi: "static thread_local %s %s;" % (mi.group(1), mi.group(2)), head)
    head = _LAYOUT_LINE.sub("", head)
    lookup = _once(r"(float\s+linDepth\s*=.*?uint\s+lightIndexOffset\s*=[^;]*;)", body, "the lookup", re.S)
    prologue = [
        _once(r"float\s+alphaRoughness\s*=[^;]*;", body, "alphaRoughness"),
        _once(r"vec3\s+V\s*=[^;]*;", body, "V"),
        _once(r"float\s+NoV\s*=[^;]*;", body, "NoV"),
        _once(r"vec3\s+F0\s*=[^;]*;", body, "F0"),
        _once(r"F0\s*=\s*mix\s*\([^;]*;", body, "F0 = mix"),
        _once(r"vec3\s+Lo\s*=\s*albedo[^;]*;", body, "Lo"),
    ]
    loop_m = re.search(r"for\s*\(\s*int\s+i\s*=\s*0\s*;\s*i\s*<\s*lightCount\s*;[^)]*\)", body)
    if not loop_m:
        raise RuntimeError("Scene.frag: no light loop")
    loop = body[loop_m.start():_balanced(body, loop_m.end())]
    funcs = (
        "struct FragmentLookup { float linDepth; uint zIndex; uint clusterIdx; uint lightCount; "
        "uint lightIndexOffset; };\n"
        "inline FragmentLookup fragment_lookup()\n{\n%s\n"
        "    return FragmentLookup{linDepth, zIndex, clusterIdx, lightCount, lightIndexOffset};\n}\n"
        "inline vec3 fragment_direct_lighting(vec3 albedo, vec3 N, float metallic, float roughness, "
        "uint lightCount, uint lightIndexOffset)\n{\n%s\n%s\n    return Lo;\n}\n"
    ) % (lookup, "\n".join(prologue), loop)
    return _literals(head) + "\n" + _literals(funcs)


def generate_ref(shader_root: Path | None = None) -> Path:
    shader_root = Path(shader_root) if shader_root else default_shader_root()
    parts = [
        "// Generated by oracle/build.py from the reference's shader sources; not part of the repository.\n",
        '#include "glsl_compat.h"\n',
    ]
    for ns, rel in SHADERS:
        body = transform_shader((shader_root / rel).read_text(), shader_root)
        parts.append("namespace %s {\nusing namespace glsl;\n// ---- %s ----\n%s\n}  // namespace %s\n" % (ns, rel, body, ns))
    frag = scene_fragment_source((shader_root / SCENE_FRAG).read_text(), shader_root)
    parts.append("namespace scene {\nusing namespace glsl;\n// ---- %s (lookup and direct lighting) ----\n%s\n"
                 "}  // namespace scene\n" % (SCENE_FRAG, frag))
    parts.append('#include "ref_driver.inc"\n')
    REF_DIR.mkdir(parents=True, exist_ok=True)
    out = "".join(parts)
    if not REF_SRC.exists() or REF_SRC.read_text() != out:
        REF_SRC.write_text(out)
    return REF_SRC


def build_ref(force: bool = False, shader_root: Path | None = None) -> Path | None:
    """Build oracle/_ref/libcf_ref.so; returns None when it cannot be built here."""
    root = Path(shader_root) if shader_root else default_shader_root()
    if root.is_dir():
        generate_ref(root)
    if not REF_SRC.exists():
        return None
    deps = [REF_SRC, ORACLE_DIR / "glsl_compat.h", ORACLE_DIR / "ref_driver.inc", REPO / "include" / "cf_pinned_math.h"]
    if force or _stale(REF_SO, deps):
        tmp = REF_SO.with_suffix(".so.tmp%d" % os.getpid())
        _run(["g++", *CXXFLAGS, "-w", "-I", str(ORACLE_DIR), "-I", str(REPO / "include"), str(REF_SRC), "-o", str(tmp)])
        os.replace(tmp, REF_SO)
    return REF_SO


if __name__ == "__main__":
    import argparse
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--force", action="store_true")
    ap.add_argument("--shaders", type=Path, default=None, help="the reference's HelloVulkan/Shaders directory")
    a = ap.parse_args()
    print(build_oracle(force=a.force))
    print(build_ref(force=a.force, shader_root=a.shaders))
