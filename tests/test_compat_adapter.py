"""The drop-in adapter of INTEGRATION.md, compiled and run as a user would.

The `gpuheap_compat.hpp` block is taken from INTEGRATION.md itself, so the
document is what is tested.  tests/compat/app.cu keeps the reference's host
class and calls the device API from its own kernels (test/heap_test.cu:13-77
does the same with the reference's Heap<K>*).  On the CPU it is compiled for
sm_103a; on a GPU it is linked against libgpuheap_gb300.so and run: the keys
its kernels delete must be the sorted inputs."""
import os
import re
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
NVCC = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _compat_header():
    text = open(os.path.join(REPO, "INTEGRATION.md")).read()
    blocks = re.findall(r"```cpp\n(.*?)```", text, re.S)
    hdr = [b for b in blocks if b.startswith("// gpuheap_compat.hpp")]
    assert len(hdr) == 1, "INTEGRATION.md holds one gpuheap_compat.hpp block"
    return "#pragma once\n" + hdr[0]


def _stage(tmp_path):
    (tmp_path / "gpuheap_compat.hpp").write_text(_compat_header())
    shutil.copy(os.path.join(HERE, "compat", "app.cu"), tmp_path / "app.cu")
    return ["-std=c++17", "-I" + str(tmp_path), "-I" + os.path.join(REPO, "include")]


def _nvcc():
    if not os.path.exists(NVCC) and not shutil.which("nvcc"):
        pytest.skip("no nvcc")
    return NVCC if os.path.exists(NVCC) else "nvcc"


def test_adapter_compiles(tmp_path):
    flags = _stage(tmp_path)
    r = subprocess.run([_nvcc()] + ARCH + flags + ["-c", str(tmp_path / "app.cu"), "-o", str(tmp_path / "app.o")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


@pytest.mark.gpu
def test_adapter_runs(tmp_path, ghlib):
    flags = _stage(tmp_path)
    libdir = os.path.join(REPO, "gpuheap_gb300")
    exe = str(tmp_path / "app")
    r = subprocess.run([_nvcc()] + ARCH + flags + [str(tmp_path / "app.cu"), "-o", exe, "-L" + libdir,
                        "-lgpuheap_gb300", "-Xlinker", "-rpath=" + libdir], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    run = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert run.returncode == 0 and "compat ok" in run.stdout, run.stdout + run.stderr
