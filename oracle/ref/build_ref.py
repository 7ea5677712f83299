#!/usr/bin/env python3
"""Build the reference's own sources for the CPU (test infrastructure only).

Recipe: read the reference sources where they lie (``<checkout>/src``, the
checkout being $SEVC_REFERENCE or a directory named ``reference`` next to
this repository), rewrite each CUDA launch ``k<<<g, b>>>(args)`` into
``SEVC_LAUNCH(k, g, b, args)`` and the constant of ``src/main.cu:49``
(``min_grains = 5000;``) into a call that reads SEVC_REF_MIN_GRAINS (default
5000), write the rewritten files to a temporary directory, compile them with
g++ against ``shim.h`` (CUDA runtime stand-ins) and ``fake_include/`` (cuRAND
stand-in), and link the runtime ``harness_rt.cpp``.  Only the executable
``oracle/_ref/sevc_ref`` is kept; the rewritten sources are deleted.

The executable is ``sevc_ref -c file.ini``: the reference program itself,
running its main loop on one CPU core.  The reference has no tests or golden
vectors; the outputs of this compiled reference pin the oracle
(tests/golden).
"""
import os
import re
import shutil
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE = os.path.dirname(HERE)
OUT_DIR = os.path.join(ORACLE, "_ref")
# the reference checkout: $SEVC_REFERENCE, else a directory named "reference"
# next to this repository
DEFAULT_SRC = os.path.join(os.environ.get("SEVC_REFERENCE") or
                           os.path.join(os.path.dirname(os.path.dirname(ORACLE)), "reference"), "src")


def _comment_mask(text):
    """Boolean per character: True inside // or /* */ comments."""
    mask = bytearray(len(text))
    i, n = 0, len(text)
    while i < n:
        if text.startswith("//", i):
            j = text.find("\n", i)
            j = n if j < 0 else j
            mask[i:j] = b"\x01" * (j - i)
            i = j
        elif text.startswith("/*", i):
            j = text.find("*/", i + 2)
            j = n if j < 0 else j + 2
            mask[i:j] = b"\x01" * (j - i)
            i = j
        elif text[i] == '"':
            j = i + 1
            while j < n and text[j] != '"':
                j += 2 if text[j] == "\\" else 1
            i = j + 1
        else:
            i += 1
    return mask


def _split_top(s):
    parts, depth, cur = [], 0, []
    for ch in s:
        if ch in "([{":
            depth += 1
        elif ch in ")]}":
            depth -= 1
        if ch == "," and depth == 0:
            parts.append("".join(cur))
            cur = []
        else:
            cur.append(ch)
    parts.append("".join(cur))
    return parts


def rewrite_launches(text):
    out, pos, count = [], 0, 0
    mask = _comment_mask(text)
    for m in re.finditer(r"([A-Za-z_][A-Za-z0-9_]*)\s*<<<", text):
        if m.start() < pos or mask[m.start()]:
            continue
        cfg_end = text.find(">>>", m.end())
        cfg = text[m.end():cfg_end]
        k = cfg_end + 3
        while text[k].isspace():
            k += 1
        if text[k] != "(":
            raise SystemExit("unexpected launch syntax near: " + text[m.start():m.start() + 80])
        depth, j = 0, k
        while True:
            if text[j] == "(":
                depth += 1
            elif text[j] == ")":
                depth -= 1
                if depth == 0:
                    break
            j += 1
        args = text[k + 1:j]
        g, b = _split_top(cfg)
        call = "SEVC_LAUNCH(%s, %s, %s%s)" % (m.group(1), g.strip(), b.strip(),
                                              (", " + args) if args.strip() else "")
        out.append(text[pos:m.start()])
        out.append(call)
        pos = j + 1
        count += 1
    out.append(text[pos:])
    return "".join(out), count


def build(src_dir=DEFAULT_SRC, out_dir=OUT_DIR, verbose=False):
    if not os.path.isdir(src_dir):
        if verbose:
            print("reference sources not found at %s: sevc_ref not built" % src_dir)
        return None
    os.makedirs(out_dir, exist_ok=True)
    tmp = tempfile.mkdtemp(prefix="sevc_ref_")
    try:
        total = 0
        for name in sorted(os.listdir(src_dir)):
            if not (name.endswith(".h") or name.endswith(".cu")):
                continue
            with open(os.path.join(src_dir, name)) as f:
                text = f.read()
            text, c = rewrite_launches(text)
            total += c
            if name == "main.cu":
                if "min_grains = 5000;" not in text:
                    raise SystemExit("src/main.cu:49 constant not found")
                text = text.replace("min_grains = 5000;", "min_grains = sevc_ref_min_grains();", 1)
            with open(os.path.join(tmp, name), "w") as f:
                f.write(text)
        flags = ["-std=c++17", "-O2", "-ffp-contract=off", "-fno-fast-math", "-w", "-U_FORTIFY_SOURCE", "-D_FORTIFY_SOURCE=0"]
        obj_main = os.path.join(tmp, "ref_main.o")
        obj_rt = os.path.join(tmp, "rt.o")
        subprocess.check_call(["g++"] + flags + ["-include", os.path.join(HERE, "shim.h"),
                               "-I", os.path.join(HERE, "fake_include"), "-I", tmp,
                               "-Dmain=sevc_ref_main", "-x", "c++", "-c", os.path.join(tmp, "main.cu"),
                               "-o", obj_main])
        subprocess.check_call(["g++"] + flags + ["-c", os.path.join(HERE, "harness_rt.cpp"), "-o", obj_rt])
        exe = os.path.join(out_dir, "sevc_ref")
        subprocess.check_call(["g++", obj_main, obj_rt, "-o", exe, "-lm"])
        if verbose:
            print("built %s (%d launch sites rewritten)" % (exe, total))
        return exe
    finally:
        shutil.rmtree(tmp, ignore_errors=True)


if __name__ == "__main__":
    build(sys.argv[1] if len(sys.argv) > 1 else DEFAULT_SRC, verbose=True)
