#!/usr/bin/env python3
"""Regenerate the golden fixtures (run where a checkout of the reference is).

    python tests/golden/make_golden.py [--reference DIR] [--only NAME ...]

DIR is the reference checkout (default: $SEVC_REFERENCE, else a directory
named "reference" next to this repository).

1. Meshes: the reference's own generator, voronoi/voronoi.py, run with
   fixed seeds (m300: N=300 seed 11, m1000: N=1000 seed 12, m2000: N=2000
   seed 1), with both its uniform and triangular stored-energy files; and
   ref2k, a copy of the reference's shipped 2,000-grain input
   (voronoi/2K/{vertices,ridges,oris}.txt, SE/uniform.txt, SE/triangular.txt).
2. Runs: each configuration of configs.py executed by the reference's own
   sources built for the CPU (oracle/_ref/sevc_ref, see oracle/ref), with the
   synthetic random stream seeded as listed.  For every snapshot the full and
   integer-only digests are stored, plus the per-step numbers of the
   reference's log (2x3 counts, grain count, nucleated area, nucleation
   site); for the long runs (configs.LONG_CONFIGS) the same for their first
   configs.FIRST_STEPS steps.

Output: tests/golden/meshes/*, tests/golden/golden.json.
"""
import json
import os
import re
import shutil
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.join(ROOT, "oracle", "ref"))

import configs  # noqa: E402
import snapshot  # noqa: E402

MESHES = {"m300": (300, 11), "m1000": (1000, 12), "m2000": (2000, 1)}
REF_MESHES = {"ref2k": "2K"}   # copies of the reference's shipped inputs (voronoi/<dir>)


def reference_dir(arg=None):
    return arg or os.environ.get("SEVC_REFERENCE") or os.path.join(os.path.dirname(ROOT), "reference")


def copy_reference_meshes(ref):
    for name, sub in REF_MESHES.items():
        src, d = os.path.join(ref, "voronoi", sub), os.path.join(configs.MESH_DIR, name)
        os.makedirs(d, exist_ok=True)
        for a, b in (("vertices.txt", "vertices.txt"), ("ridges.txt", "ridges.txt"), ("oris.txt", "oris.txt"),
                     (os.path.join("SE", "uniform.txt"), "se_uniform.txt"),
                     (os.path.join("SE", "triangular.txt"), "se_triangular.txt")):
            shutil.copyfile(os.path.join(src, a), os.path.join(d, b))


def make_meshes(ref):
    copy_reference_meshes(ref)
    gen = os.path.join(ref, "voronoi", "voronoi.py")
    for name, (n, seed) in MESHES.items():
        d = os.path.join(configs.MESH_DIR, name)
        os.makedirs(d, exist_ok=True)
        base = [sys.executable, gen, str(n), str(seed), os.path.join(d, "vertices.txt"), os.path.join(d, "ridges.txt"),
                os.path.join(d, "oris.txt")]
        subprocess.check_call(base + [os.path.join(d, "se_uniform.txt")], stdout=subprocess.DEVNULL)
        tmp = tempfile.mkdtemp()
        try:
            subprocess.check_call([sys.executable, gen, str(n), str(seed), os.path.join(tmp, "v"), os.path.join(tmp, "r"),
                                   os.path.join(tmp, "o"), os.path.join(d, "se_triangular.txt"), "--sedist", "triangular"],
                                  stdout=subprocess.DEVNULL)
        finally:
            shutil.rmtree(tmp)


def parse_log(text):
    steps, cur = [], None
    for line in text.splitlines():
        m = re.match(r"n = (\d+), t = ", line)
        if m:
            cur = {"n": int(m.group(1)), "two_three": [], "n_grains": None, "nucl_area": None, "nucleated_at": -1}
            steps.append(cur)
            continue
        if cur is None:
            continue
        m = re.match(r"(\d+) configurations of two three sided grains", line)
        if m:
            cur["two_three"].append(int(m.group(1)))
        m = re.match(r"Number of grains: (\d+)", line)
        if m and cur["n_grains"] is None:
            cur["n_grains"] = int(m.group(1))
        m = re.match(r"Nucleated area %: (\S+)", line)
        if m:
            cur["nucl_area"] = m.group(1)
        m = re.match(r"Nucleating at vertex (\d+)", line)
        if m:
            cur["nucleated_at"] = int(m.group(1))
    return steps


def run_config(name, exe):
    _, _, _, seed, min_grains = configs.ALL_CONFIGS[name]
    tmp = tempfile.mkdtemp(prefix="golden_")
    try:
        folder = os.path.join(tmp, "out")
        nmax = configs.golden_nmax(name)
        ini = configs.write_ini(os.path.join(tmp, "run.ini"), name, folder, nmax=nmax)
        env = dict(os.environ, SEVC_REF_MIN_GRAINS=str(min_grains), SEVC_REF_RNG_SEED=str(seed))
        r = subprocess.run([exe, "-c", ini], capture_output=True, text=True, env=env, check=True)
        data = os.path.join(folder, "DATA")
        snaps = [list(snapshot.digests(os.path.join(data, f))) for f in sorted(os.listdir(data))]
        return {"snapshots": snaps, "steps": parse_log(r.stdout), "rng_seed": seed, "min_grains": min_grains,
                "nmax": nmax}
    finally:
        shutil.rmtree(tmp)


def main():
    import argparse
    import build_ref
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=None, help="reference checkout (default $SEVC_REFERENCE or ../reference)")
    ap.add_argument("--only", nargs="*", default=None, help="regenerate these configurations only (meshes are kept)")
    args = ap.parse_args()
    ref = reference_dir(args.reference)
    exe = build_ref.build(os.path.join(ref, "src"), verbose=True)
    if exe is None:
        raise SystemExit("the reference sources are needed to regenerate the fixtures (%s)" % ref)
    path = os.path.join(HERE, "golden.json")
    out = {}
    if args.only:
        out = json.load(open(path))
    else:
        make_meshes(ref)
    for name in (args.only or configs.ALL_CONFIGS):
        out[name] = run_config(name, exe)
        g = out[name]
        s = g["steps"]
        print("%-14s %4d steps, %3d snapshots, grains %d -> %s, nucleations %d, 2x3 steps %d" % (
            name, len(s), len(g["snapshots"]), s[0]["n_grains"], s[-1]["n_grains"],
            sum(1 for x in s if x["nucleated_at"] >= 0), sum(1 for x in s if any(x["two_three"]))), flush=True)
    with open(path, "w") as f:
        json.dump(out, f, indent=0)


if __name__ == "__main__":
    main()
