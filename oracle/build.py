"""Build recipe for the CPU oracle and for the reference shaders compiled as C++.

TEST INFRASTRUCTURE ONLY: the tests, the smoke check and the benchmark's CPU
baseline leg load what this builds; the CUDA library never does.

* ``build_oracle()`` compiles ``oracle/cf_oracle.cpp`` (the restatement) into
  ``oracle/_build/libcf_oracle.so`` with ``g++ -O2 -ffp-contract=off -fopenmp``.
* ``generate_ref(shader_root)`` reads the reference's two compute shaders
  (``HelloVulkan/Shaders/ClusteredForward/AABBGenerator.comp`` and
  ``LightCulling.comp``) where they lie and rewrites them mechanically into
  ``oracle/_ref/ref_shaders_gen.cpp`` (git-ignored): ``#include`` lines are
  expanded, ``#version`` and the ``local_size`` layout are dropped, each
  interface block becomes a namespace-scope variable, unsuffixed float
  literals get an ``f`` (GLSL literals are single precision) and ``.xyz``
  becomes a call.  Everything else is the shaders' own text, compiled against
  ``oracle/glsl_compat.h`` and driven by ``oracle/ref_driver.inc``.
* ``build_ref()`` compiles that generated file into ``oracle/_ref/libcf_ref.so``.
  It needs only the generated file, so it also runs where the reference
  checkout is absent, as long as the file was generated beforehand.
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
DEFAULT_SHADER_ROOT = Path("/root/reference/HelloVulkan/Shaders")

CXXFLAGS = ["-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math", "-fopenmp"]

SHADERS = (
    ("aabbgen", "ClusteredForward/AABBGenerator.comp"),
    ("lightcull", "ClusteredForward/LightCulling.comp"),
)


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


def transform_shader(text: str, root: Path) -> str:
    text = _expand_includes(text, root)
    text = _VERSION.sub("", text)
    text = _EXTENSION.sub("", text)
    text = _LOCAL_SIZE.sub("", text)
    text = _BLOCK.sub(_block, text)
    text = _FLOAT_LIT.sub(lambda m: m.group(1) + "f", text)
    text = _SWIZZLE_XYZ.sub(".xyz()", text)
    return text


def generate_ref(shader_root: Path = DEFAULT_SHADER_ROOT) -> Path:
    shader_root = Path(shader_root)
    parts = [
        "// Generated by oracle/build.py from the reference's shader sources; not part of the repository.\n",
        '#include "glsl_compat.h"\n',
    ]
    for ns, rel in SHADERS:
        body = transform_shader((shader_root / rel).read_text(), shader_root)
        parts.append("namespace %s {\nusing namespace glsl;\n// ---- %s ----\n%s\n}  // namespace %s\n" % (ns, rel, body, ns))
    parts.append('#include "ref_driver.inc"\n')
    REF_DIR.mkdir(parents=True, exist_ok=True)
    out = "".join(parts)
    if not REF_SRC.exists() or REF_SRC.read_text() != out:
        REF_SRC.write_text(out)
    return REF_SRC


def build_ref(force: bool = False) -> Path | None:
    """Build oracle/_ref/libcf_ref.so; returns None when it cannot be built here."""
    if DEFAULT_SHADER_ROOT.is_dir():
        generate_ref(DEFAULT_SHADER_ROOT)
    if not REF_SRC.exists():
        return None
    deps = [REF_SRC, ORACLE_DIR / "glsl_compat.h", ORACLE_DIR / "ref_driver.inc", REPO / "include" / "cf_pinned_math.h"]
    if force or _stale(REF_SO, deps):
        tmp = REF_SO.with_suffix(".so.tmp%d" % os.getpid())
        _run(["g++", *CXXFLAGS, "-w", "-I", str(ORACLE_DIR), "-I", str(REPO / "include"), str(REF_SRC), "-o", str(tmp)])
        os.replace(tmp, REF_SO)
    return REF_SO


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv))
    print(build_ref(force="--force" in sys.argv))
