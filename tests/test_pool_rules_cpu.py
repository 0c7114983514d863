"""The committed code keeps to the rules of a shared GPU: it never faults a
GPU on purpose, never changes a GPU's settings and uses none of the batched
copy calls that faulted GPUs of this generation.  Checked on the sources
(documentation excluded), on CPU."""
import glob
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SKIP_DIRS = {".git", "_work", "gpurun_out", "__pycache__", "_build", "_ref", "baseline"}
EXTS = (".cu", ".cuh", ".h", ".hpp", ".c", ".cpp", ".py", ".sh", "Makefile")


def _files():
    for dirpath, dirs, files in os.walk(ROOT):
        dirs[:] = [d for d in dirs if d not in SKIP_DIRS]
        for f in files:
            if f.endswith(EXTS):
                yield os.path.join(dirpath, f)


def _device_sources():
    return sorted(glob.glob(os.path.join(ROOT, "gpuheap_gb300", "csrc", "*.cu*")) +
                  glob.glob(os.path.join(ROOT, "include", "*.cuh")))


def test_no_batched_copy_calls():
    # the names are assembled here so that this file does not name them
    names = ["cuda" + "Memcpy" + "BatchAsync", "cuda" + "Memcpy3D" + "BatchAsync",
             "cu" + "Memcpy" + "BatchAsync", "cu" + "Memcpy3D" + "BatchAsync"]
    hits = []
    for path in _files():
        text = open(path, errors="replace").read()
        hits += [f"{os.path.relpath(path, ROOT)}: {n}" for n in names if n in text]
    assert not hits, hits


def test_no_trap_or_device_assert():
    """Failures are error words the host reads, never a trap or a failing
    device assert (either would end the context, or hang the GPU)."""
    bad = []
    for path in _device_sources():
        for i, line in enumerate(open(path).read().split("\n"), 1):
            code = line.split("//", 1)[0]
            if "__trap" in code or re.search(r"\btrap\s*;", code) or re.search(r"(?<![_\w])assert\s*\(", code):
                bad.append(f"{os.path.relpath(path, ROOT)}:{i}: {line.strip()}")
    assert not bad, bad


def test_gpu_settings_are_only_read():
    """nvidia-smi is used to sample clocks (queries), never to set clocks,
    power limits, persistence, compute or ECC mode, or to reset a GPU."""
    setters = re.compile(r"(-lgc|--lock-gpu-clocks|-rgc|-ac\b|--applications-clocks|-pl\b|--power-limit|-pm\b|"
                         r"--persistence-mode|-c\b|--compute-mode|-e\b|--ecc-config|-r\b|--gpu-reset|-mig)")
    bad = []
    for path in _files():
        text = open(path, errors="replace").read()
        for m in re.finditer(r"nvidia-smi[^\n]*", text):
            frag = m.group(0)
            if setters.search(frag.replace("--query-gpu", "").replace("--format", "")):
                bad.append(f"{os.path.relpath(path, ROOT)}: {frag[:100]}")
    assert not bad, bad


def test_ncu_commands_leave_clocks_alone():
    """Any ncu command line in committed scripts passes --clock-control none."""
    bad = []
    for path in _files():
        if path.endswith(".py") and os.path.basename(path).startswith("test_"):
            continue
        for i, line in enumerate(open(path, errors="replace").read().split("\n"), 1):
            if re.search(r"\bncu\s+--", line) and "--clock-control none" not in line:
                bad.append(f"{os.path.relpath(path, ROOT)}:{i}: {line.strip()[:100]}")
    assert not bad, bad
