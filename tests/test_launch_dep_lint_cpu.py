"""Every kernel launched with programmatic dependent launch (launch_dep in
csrc/sevc_internal.h) may start while the previous kernel of its stream is
still running, so its first statement must be griddep_wait(): the wait
returns only once that kernel has completed and its writes are visible.
A kernel launched this way without the wait would race with its
predecessor, which a parity run need not catch; this check reads the
sources."""
import os
import re

CSRC = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "se-grain-growth-gpu_gb300", "csrc")


def _sources():
    out = {}
    for f in sorted(os.listdir(CSRC)):
        if f.endswith((".cu", ".cuh", ".h")):
            out[f] = open(os.path.join(CSRC, f)).read()
    return out


def test_kernels_launched_with_launch_dep_wait_first():
    src = _sources()
    launched = set()
    for f, text in src.items():
        if not f.endswith(".cu"):
            continue                      # the helper's own definition lives in a header
        for mo in re.finditer(r"launch_dep\(\s*([A-Za-z_]\w*)", text):
            launched.add(mo.group(1))
    assert launched, "no launch_dep call found"
    missing = []
    for name in sorted(launched):
        body = None
        for text in src.values():
            mo = re.search(r"__global__ void (?:__launch_bounds__\([^)]*\)\s*)?" + re.escape(name) + r"\([^)]*\)\s*\{", text)
            if mo:
                body = text[mo.end():]
                break
        assert body is not None, "kernel %s not found" % name
        first = body.lstrip().split(";", 1)[0].strip()
        if first != "griddep_wait()":
            missing.append((name, first))
    assert not missing, missing


def _kernel_bodies(text):
    """(name, body) of every __global__ function in text, body by brace matching"""
    for mo in re.finditer(r"__global__ void (?:__launch_bounds__\([^)]*\)\s*)?(\w+)\([^)]*\)\s*\{", text):
        depth, i = 1, mo.end()
        while depth:
            depth += {"{": 1, "}": -1}.get(text[i], 0)
            i += 1
        yield mo.group(1), text[mo.end():i - 1]


def test_kernels_with_last_block_never_return_early():
    """last_block counts the blocks that reach it: a thread that returns
    before it would leave the count short and the list counts it resets
    would never be reset."""
    found = 0
    for f, text in _sources().items():
        for name, body in _kernel_bodies(text):
            if "last_block(" in body:
                found += 1
                assert not re.search(r"\breturn\b", body), name
    assert found >= 2
