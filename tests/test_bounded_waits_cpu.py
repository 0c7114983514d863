"""Every spin-wait in the device code is bounded.  A loop whose condition
polls a shared word (an mbarrier try-wait, an acquire or relaxed load, a
CAS, an atomicMax) must give up: through the heap's `keep_waiting`
(globaltimer against the heap's time limit, which raises a sticky error),
a deadline of its own on the globaltimer (the FIFO's and the served
loop's time limits), or an iteration cap.  A GPU kernel
that can spin forever on a word nobody will write hangs the GPU for
everyone after it, so this is checked on the sources, on CPU."""
import glob
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SOURCES = sorted(glob.glob(os.path.join(ROOT, "gpuheap_gb300", "csrc", "*.cu")) +
                 glob.glob(os.path.join(ROOT, "gpuheap_gb300", "csrc", "*.cuh")) +
                 glob.glob(os.path.join(ROOT, "include", "*.cuh")))
POLLS = ("mbar_try_wait", "ld_acquire", "ld_relaxed", "lds(", "atomicCAS", "cas_acquire", "max_acquire")
BOUNDS = ("keep_waiting", "globaltimer", "timeoutNs", "(1u << 22)", "tries <", "waitNs", "stallNs")


def _loops(text):
    """(line, header condition, loop text) of every for/while loop."""
    for m in re.finditer(r"\b(for|while)\s*\(", text):
        i = m.end()
        depth = 1
        while depth and i < len(text):
            depth += {"(": 1, ")": -1}.get(text[i], 0)
            i += 1
        cond = text[m.end():i - 1]
        rest = text[i:]
        body = rest.lstrip()
        if body.startswith("{"):
            depth, k = 0, 0
            for k, ch in enumerate(body):
                depth += {"{": 1, "}": -1}.get(ch, 0)
                if depth == 0:
                    break
            body = body[:k + 1]
        else:
            body = body.split(";", 1)[0]
        yield text.count("\n", 0, m.start()) + 1, cond, cond + body


def test_sources_found():
    assert len(SOURCES) >= 10


def test_every_polling_loop_is_bounded():
    unbounded = []
    polling = 0
    for path in SOURCES:
        text = open(path).read()
        for line, cond, loop in _loops(text):
            if not any(p in cond for p in POLLS):
                continue
            polling += 1
            if not any(b in loop for b in BOUNDS):
                unbounded.append(f"{os.path.relpath(path, ROOT)}:{line}: ({cond.strip()[:80]})")
    assert polling >= 20, polling  # the scan sees the device code's polls
    assert not unbounded, "spin-waits without a bound:\n" + "\n".join(unbounded)


def test_every_sleeping_loop_is_bounded():
    """Open loops (for (;;), while (true)) that back off with __nanosleep
    are waits too: each gives up the same ways."""
    unbounded = []
    sleeping = 0
    for path in SOURCES:
        for line, cond, loop in _loops(open(path).read()):
            if cond.strip() not in (";;", "true", "1") or "__nanosleep" not in loop:
                continue
            sleeping += 1
            if not any(b in loop for b in BOUNDS):
                unbounded.append(f"{os.path.relpath(path, ROOT)}:{line}")
    assert sleeping >= 5, sleeping
    assert not unbounded, "sleeping waits without a bound:\n" + "\n".join(unbounded)
