"""The drop-in boundary from C++: tests/cpp/app_cluster_forward.cpp drives
the two pipelines through include/cfcull.h as the reference application
does, and checks every frame against the oracle library.  Compiled here;
run on the GPU."""
import shutil
import subprocess
from pathlib import Path

import pytest

REPO = Path(__file__).resolve().parents[1]
SRC = REPO / "tests" / "cpp" / "app_cluster_forward.cpp"
LIB_DIR = REPO / "hellovulkan_gb300"
ORACLE_DIR = REPO / "oracle" / "_build"


def _compile(out: Path) -> Path:
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    from hellovulkan_gb300 import build as cuda_build
    from oracle import build as oracle_build
    cuda_build.build()
    oracle_build.build_oracle()
    cmd = ["g++", "-std=c++20", "-O2", "-Wall", "-Wextra", "-Werror", "-I", str(REPO / "include"), str(SRC),
           "-L", str(LIB_DIR), "-lcfcull", "-L", str(ORACLE_DIR), "-lcf_oracle",
           "-Wl,-rpath," + str(LIB_DIR) + ":" + str(ORACLE_DIR), "-o", str(out)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return out


def test_cpp_host_compiles_and_links(tmp_path):
    assert _compile(tmp_path / "app").exists()


@pytest.mark.gpu
def test_cpp_host_frames_match_the_oracle(tmp_path):
    app = _compile(tmp_path / "app")
    r = subprocess.run([str(app)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.strip().endswith("ok") and r.stdout.count("bit-exact") == 4, r.stdout
