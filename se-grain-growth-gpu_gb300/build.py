"""Build the engine: libsevc.so (CUDA kernels + C ABI + host C), the sevc CLI
and the sevc-voronoi input generator.

Every .cu file is compiled for sm_103a only, with -fmad=false (no fused
multiply-add, the arithmetic contract of the kernels) and -lineinfo; host C
is compiled with -ffp-contract=off.  Objects go to _build/, the library and
the CLI next to this file.  Translation units compile in parallel.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OBJ = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libsevc.so")
CLI = os.path.join(PKG, "sevc")
VORONOI_CLI = os.path.join(PKG, "sevc-voronoi")

NVCC = os.environ.get("NVCC", shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-O3", "-std=c++17", "-lineinfo", "-fmad=false", "-Xcompiler", "-fPIC,-ffp-contract=off",
           "-I", os.path.join(ROOT, "include")]
CFLAGS = ["-O2", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-fopenmp", "-Wall", "-I",
          os.path.join(ROOT, "include")]

CU = ["sevc_geometry.cu", "sevc_topology.cu", "sevc_nucleation.cu", "sevc_adjoint.cu", "sevc_check.cu",
      "sevc_engine.cu"]
C = ["sevc_host.c", "sevc_voronoi.c"]
HDRS = ["sevc_device.cuh", "sevc_internal.h", "sevc_host.h"]


def _stale(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode:
        raise RuntimeError("build failed:\n%s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return r.stdout + r.stderr


def build(force=False, verbose=False, ptxas_info=False):
    os.makedirs(OBJ, exist_ok=True)
    hdrs = [os.path.join(CSRC, h) for h in HDRS] + [os.path.join(ROOT, "include", "sevc.h")]
    jobs, objs = [], []
    for f in CU:
        src, obj = os.path.join(CSRC, f), os.path.join(OBJ, f + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + hdrs):
            extra = ["-Xptxas", "-v"] if ptxas_info else []
            jobs.append([NVCC] + ARCH + NVFLAGS + extra + ["-c", src, "-o", obj])
    for f in C:
        src, obj = os.path.join(CSRC, f), os.path.join(OBJ, f + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + hdrs):
            jobs.append(["gcc"] + CFLAGS + ["-c", src, "-o", obj])
    logs = []
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for out in ex.map(_run, jobs):
            logs.append(out)
    if force or jobs or _stale(LIB, objs):
        tmp = LIB + ".tmp%d" % os.getpid()
        _run([NVCC] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart", "-lgomp"])
        os.replace(tmp, LIB)
    for src, exe in ((os.path.join(PKG, "cli", "sevc_main.c"), CLI),
                     (os.path.join(PKG, "cli", "sevc_voronoi_main.c"), VORONOI_CLI)):
        if force or _stale(exe, [src, LIB]):
            _run(["gcc"] + CFLAGS + [src, "-o", exe, "-L", PKG, "-lsevc", "-lm", "-Wl,-rpath,$ORIGIN"])
    if verbose:
        print("".join(logs))
    return LIB


if __name__ == "__main__":
    import sys
    build(force="--force" in sys.argv, verbose=True, ptxas_info="--ptxas" in sys.argv)
    print("built", LIB)
