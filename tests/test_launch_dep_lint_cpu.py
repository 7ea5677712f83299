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
    """last_block counts the blocks that reach it and holds a block
    barrier: every thread must call it.  So a kernel that uses it returns
    nowhere early, and the call sits at the top level of the kernel body
    (no enclosing block that could depend on the thread) as the first
    operand of its expression (no short-circuit operator or conditional
    before it that some threads could stop at)."""
    found = 0
    for f, text in _sources().items():
        for name, body in _kernel_bodies(text):
            if "last_block(" not in body:
                continue
            assert not re.search(r"\breturn\b", body), name
            for mo in re.finditer(r"last_block\(", body):
                found += 1
                head = body[:mo.start()]
                depth = head.count("{") - head.count("}")
                assert depth == 0, "%s: last_block inside a nested block" % name
                stmt = re.split(r"[;{}]", head)[-1]
                assert not re.search(r"&&|\|\||\?", stmt), "%s: last_block after a short-circuit operand" % name
    assert found >= 2
