"""Host code under AddressSanitizer and UndefinedBehaviorSanitizer (CPU).

Builds tests/cpp/sanitize_main.cpp with the oracle and the library's host
translation units (C ABI, batches, server, load driver) instrumented with
-fsanitize=address,undefined, linked against the library's ordinary kernel
objects and the static CUDA runtime, and runs it on the golden views: the
oracle's culling, lookup, shading and frustum culling, the server arena under
a randomised allocation sequence, and the C ABI's argument checks without a
device.  Any sanitizer report fails the run (-fno-sanitize-recover)."""
import os
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

REPO = Path(__file__).resolve().parents[1]
CSRC = REPO / "hellovulkan_gb300" / "csrc"
HOST_SOURCES = ["cf_runtime.cpp", "cf_batch.cpp", "cf_server.cpp", "cf_serve_load.cpp"]


def kernel_objects():
    """The library's ordinary (not instrumented) objects of every .cu file."""
    return [REPO / "hellovulkan_gb300" / "_build" / (src.name + ".o") for src in sorted(CSRC.glob("*.cu"))]


def cuda_home() -> Path:
    nvcc = shutil.which("nvcc")
    return Path(nvcc).resolve().parents[1] if nvcc else Path("/usr/local/cuda")


def write_views(path: Path, golden) -> int:
    from hellovulkan_gb300.camera import ubo_from_bytes
    n = 0
    with open(path, "wb") as f:
        for name in [str(x) for x in golden["names"]]:
            ubo = ubo_from_bytes(golden[name + "/ubo"])
            lights = np.ascontiguousarray(golden[name + "/lights"], np.float32)
            f.write(bytes(ubo))
            f.write(np.array([int(golden[name + "/cap"][0]), lights.shape[0]], np.uint32).tobytes())
            f.write(lights.tobytes())
            n += 1
    return n


def test_host_code_is_clean_under_address_and_undefined_behaviour_sanitizers(tmp_path, cflib, golden):
    cuda = cuda_home()
    objs = kernel_objects()
    if not all(o.exists() for o in objs) or not (cuda / "lib64" / "libcudart_static.a").exists():
        pytest.skip("kernel objects or the static CUDA runtime are not available")
    exe = tmp_path / "sanitize_main"
    flags = ["-std=c++20", "-O1", "-g", "-fsanitize=address,undefined", "-fno-sanitize-recover=all",
             "-fno-omit-frame-pointer", "-ffp-contract=off", "-fopenmp"]
    inc = ["-I", str(REPO / "include"), "-I", str(CSRC), "-I", str(REPO / "oracle"), "-I", str(cuda / "include")]
    srcs = [str(REPO / "tests" / "cpp" / "sanitize_main.cpp"), str(REPO / "oracle" / "cf_oracle.cpp")] + [
        str(CSRC / s) for s in HOST_SOURCES]
    cmd = ["g++", *flags, *inc, *srcs, *map(str, objs), "-L", str(cuda / "lib64"), "-lcudart_static", "-ldl",
           "-lrt", "-lpthread", "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
    views = tmp_path / "views.bin"
    n = write_views(views, golden)
    env = dict(os.environ, ASAN_OPTIONS="detect_leaks=0:abort_on_error=0", UBSAN_OPTIONS="print_stacktrace=1",
               OMP_NUM_THREADS="2")
    r = subprocess.run([str(exe), str(views)], capture_output=True, text=True, env=env, timeout=600)
    assert r.returncode == 0, (r.stdout[-2000:], r.stderr[-6000:])
    assert ("views %d, failures 0" % n) in r.stdout
