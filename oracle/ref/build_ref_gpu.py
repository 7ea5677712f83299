#!/usr/bin/env python3
"""The reference's own CUDA program, built for the GB300 (test infrastructure).

Two steps, because the reference's sources are only where its checkout is
and binaries built on one machine do not run on the other:

  stage   (where the checkout is: $SEVC_REFERENCE, --reference DIR, or a
          directory named "reference" next to this repository) copies
          <checkout>/src/*.cu, *.h into oracle/_ref/gpu_src/ (git-ignored,
          never committed) with the edits listed below;
  build   (on the GPU machine) compiles the staged copy with nvcc into
          oracle/_ref/:
            sevc_ref_gpu         nvcc main.cu                 (as shipped:
                                 src/Makefile:7, no -arch, nvcc's default
                                 contraction of a*b+c into fma)
            sevc_ref_gpu_sm103a  nvcc -arch=sm_103a main.cu
            sevc_ref_gpu_nofma   nvcc -arch=sm_103a --fmad=false main.cu

Edits (each keeps the step's arithmetic and event logic as written):
  H1  src/topological.h:598,601 pass an int where printf's "%s" expects a
      string (device printf would read it as an address): __func__ is
      passed for the %s, as in the reference's other messages;
  H2  src/main.cu:74-75,102: dev_vrt_id_candidate and candidate_buffer are
      used before anything writes them: both are zeroed after cudaMalloc;
      src/nucleation2.cu:411 indexes dev_vertices with a candidate that can
      be -1 or stale when no block picked a vertex: such a candidate is
      reported and rejected (set to -1) instead of dereferenced;
  H3  src/geometry.h:615-619 writes past a grain's 100 vertex slots after
      its warning: the write is skipped;
  H5  src/topological.h:555 polls without a bound: after 100000
      iterations the program prints a message and exits with status 4;
  M1  src/main.cu:49 hard-codes min_grains = 5000: SEVC_REF_MIN_GRAINS
      (default 5000) replaces the constant;
  T1  instrumentation: the start of every loop iteration and the end of
      the loop print "SEVC_T <n> <seconds>" on stderr (CLOCK_MONOTONIC);
  S1  SEVC_REF_SNAPSHOTS=0 skips the snapshot block (src/main.cu:328-348;
      only for timing runs: it reads the state and frees and re-allocates
      the device arrays, it changes nothing the steps compute).
"""
import argparse
import os
import re
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE = os.path.dirname(HERE)
OUT_DIR = os.path.join(ORACLE, "_ref")
STAGE = os.path.join(OUT_DIR, "gpu_src")
VARIANTS = {
    "sevc_ref_gpu": [],
    "sevc_ref_gpu_sm103a": ["-arch=sm_103a"],
    "sevc_ref_gpu_nofma": ["-arch=sm_103a", "--fmad=false"],
}

PATCH_HEADER = r'''/* edits of the staging recipe (oracle/ref/build_ref_gpu.py) */
#include <stdlib.h>
#include <stdio.h>
#include <time.h>
static inline int sevc_ref_min_grains(int dflt)
{
    const char *s = getenv("SEVC_REF_MIN_GRAINS");
    return s ? atoi(s) : dflt;
}
static inline int sevc_ref_snapshots(void)
{
    const char *s = getenv("SEVC_REF_SNAPSHOTS");
    return !(s && s[0] == '0');
}
static inline void sevc_ref_mark(int n)
{
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    fprintf(stderr, "SEVC_T %d %.9f\n", n, ts.tv_sec + 1e-9 * ts.tv_nsec);
}
'''


def reference_dir(arg=None):
    return arg or os.environ.get("SEVC_REFERENCE") or \
        os.path.join(os.path.dirname(os.path.dirname(ORACLE)), "reference")


def _sub(text, old, new, what, count=1):
    if text.count(old) < count:
        raise SystemExit("staging: %s: expected text not found" % what)
    return text.replace(old, new, count)


def _edit(name, text):
    if name == "topological.h":
        # H1
        text = _sub(text, 'printf("In %s: 3 sided grain about to flip before flipping (%d and %d)\\n", gic[0]->id',
                    'printf("In %s: 3 sided grain about to flip before flipping (%d and %d)\\n", __func__, gic[0]->id',
                    "H1 topological.h:598")
        text = _sub(text, 'printf("In %s: Error: 3 Sided grains will flip  (%d and %d)\\n", gic[0]->id',
                    'printf("In %s: Error: 3 Sided grains will flip  (%d and %d)\\n", __func__, gic[0]->id',
                    "H1 topological.h:601")
        # H5
        text = _sub(text, "    bool convergence = false;\n    while(!convergence) {",
                    "    bool convergence = false;\n    long sevc_iters = 0;\n    while(!convergence) {\n"
                    "        if(++sevc_iters > 100000) { printf(\"polling did not converge\\n\"); exit(4); }",
                    "H5 topological.h:555")
    elif name == "geometry.h":
        # H3
        text = _sub(text, 'printf("In %s: Maximum number of vertices reached for grain %d.\\n", __func__, grn->id);\n'
                          '    }',
                    'printf("In %s: Maximum number of vertices reached for grain %d.\\n", __func__, grn->id);\n'
                    '        return;\n    }', "H3 geometry.h:615-619")
    elif name == "nucleation2.cu":
        # H2 (reading side)
        text = _sub(text, "        vertex *vrt = &dev_vertices[dev_vrt_id_candidate[0]];",
                    "        if(dev_vrt_id_candidate[0] < 0 || dev_vrt_id_candidate[0] >= n_vertices) {\n"
                    "            printf(\"no valid nucleation candidate\\n\");\n"
                    "            dev_vrt_id_candidate[0] = -1;\n"
                    "            state[tid] = localState;\n"
                    "            return;\n"
                    "        }\n"
                    "        vertex *vrt = &dev_vertices[dev_vrt_id_candidate[0]];", "H2 nucleation2.cu:411")
    elif name == "main.cu":
        text = PATCH_HEADER + text
        # M1
        text = _sub(text, "    min_grains = 5000;", "    min_grains = sevc_ref_min_grains(5000);", "M1 main.cu:49")
        # H2 (allocation side)
        text = _sub(text, "    HERR(cudaMalloc(&dev_vrt_id_candidate, sizeof(int) * opt.n_blocks));",
                    "    HERR(cudaMalloc(&dev_vrt_id_candidate, sizeof(int) * opt.n_blocks));\n"
                    "    HERR(cudaMemset(dev_vrt_id_candidate, 0, sizeof(int) * opt.n_blocks));", "H2 main.cu:74")
        text = _sub(text, "    HERR(cudaMalloc((void **) &candidate_buffer, sizeof(bool) * n_boundaries));",
                    "    HERR(cudaMalloc((void **) &candidate_buffer, sizeof(bool) * n_boundaries));\n"
                    "    HERR(cudaMemset(candidate_buffer, 0, sizeof(bool) * n_boundaries));", "H2 main.cu:102")
        # T1
        text = _sub(text, '        printf("n = %d, t = %f\\n", n, t);',
                    '        sevc_ref_mark(n);\n        printf("n = %d, t = %f\\n", n, t);', "T1 main.cu:122")
        # S1
        text = _sub(text, "        if(n % opt.snap_gap == 0 || (curr_n_grains <= min_grains && min_grains > 0)) {",
                    "        if(sevc_ref_snapshots() && "
                    "(n % opt.snap_gap == 0 || (curr_n_grains <= min_grains && min_grains > 0))) {", "S1 main.cu:328")
        m = re.search(r"\n(\s*)return 0;\s*\n\}\s*$", text)
        if not m:
            raise SystemExit("staging: T1: end of main not found")
        text = text[:m.start()] + "\n    sevc_ref_mark(n);" + text[m.start():]
    return text


def stage(ref_dir):
    src = os.path.join(ref_dir, "src")
    if not os.path.isdir(src):
        raise SystemExit("reference sources not found at %s" % src)
    if os.path.isdir(STAGE):
        shutil.rmtree(STAGE)
    os.makedirs(STAGE)
    for name in sorted(os.listdir(src)):
        if name.endswith(".cu") or name.endswith(".h"):
            with open(os.path.join(src, name)) as f:
                text = f.read()
            with open(os.path.join(STAGE, name), "w") as f:
                f.write(_edit(name, text))
    return STAGE


def build(variants=None, verbose=False):
    if not os.path.exists(os.path.join(STAGE, "main.cu")):
        raise SystemExit("stage the reference first (python oracle/ref/build_ref_gpu.py stage)")
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    procs = {}
    for exe in variants or VARIANTS:
        cmd = [nvcc] + VARIANTS[exe] + ["-w", "main.cu", "-o", os.path.join(OUT_DIR, exe)]
        procs[exe] = subprocess.Popen(cmd, cwd=STAGE, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    for exe, p in procs.items():
        out = p.communicate()[0]
        if p.returncode:
            raise SystemExit("nvcc failed for %s:\n%s" % (exe, out))
        if verbose:
            print("built", os.path.join(OUT_DIR, exe))
    return [os.path.join(OUT_DIR, e) for e in procs]


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("what", choices=["stage", "build"])
    ap.add_argument("--reference", default=None)
    ap.add_argument("--variants", nargs="*", default=None)
    a = ap.parse_args()
    if a.what == "stage":
        print("staged", stage(reference_dir(a.reference)))
    else:
        build(a.variants, verbose=True)
