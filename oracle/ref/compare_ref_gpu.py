#!/usr/bin/env python3
"""Run the reference's own CUDA program (oracle/ref/build_ref_gpu.py) and
this repository's engine on the same configuration on the GB300, and
compare what they print and write (test infrastructure).

  compare_ref_gpu.py events  --exe sevc_ref_gpu_nofma --config example_ref2k [--nmax N] --json out.json
      both programs run the configuration of tests/golden/configs.py from
      the same .ini (min_grains = leave_percent * n_grains on both sides);
      compared: every step's log numbers (grain count, 2x3 counts,
      nucleated area) and every snapshot, byte for byte and by its integer
      columns (snapshot.digests); the first difference is reported.
  compare_ref_gpu.py timing  --exe sevc_ref_gpu_sm103a --grains 1000000 --nmax 5 --json out.json
      the benchmark's 1M-grain workload written as input files; both run
      nmax steps with snapshots off; per-step wall times of the reference
      from its SEVC_T marks, the engine's from the same loop in-process.
"""
import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
for p in (ROOT, os.path.join(ROOT, "se-grain-growth-gpu_gb300"), os.path.join(ROOT, "tests", "golden")):
    sys.path.insert(0, p)
OUT = os.path.join(ROOT, "oracle", "_ref")


def run(cmd, env=None, timeout=None):
    t0 = time.time()
    r = subprocess.run(cmd, capture_output=True, text=True, env=env, timeout=timeout)
    return r, time.time() - t0


def marks(stderr):
    t = {}
    for line in stderr.splitlines():
        if line.startswith("SEVC_T "):
            _, n, s = line.split()
            t[int(n)] = float(s)
    return t


def events(args):
    import configs
    import make_golden
    import snapshot
    name = args.config
    mesh, se, keys, _, mg = configs.ALL_CONFIGS[name]
    tmp = tempfile.mkdtemp(prefix="cmp_")
    n_grains = int(keys["n_grains"])
    out = {"config": name, "exe": args.exe, "min_grains": mg}
    dirs = {}
    for side in ("ref", "eng"):
        ini = configs.write_ini(os.path.join(tmp, side + ".ini"), name, os.path.join(tmp, side), nmax=args.nmax)
        if "leave_percent" not in keys:
            with open(ini, "a") as f:
                f.write("[Temporal]\nleave_percent=%r\n" % (mg / n_grains))
        dirs[side] = (ini, os.path.join(tmp, side, "DATA"))
    env = dict(os.environ, SEVC_REF_MIN_GRAINS=str(mg))
    r, ref_s = run([os.path.join(OUT, args.exe), "-c", dirs["ref"][0]], env=env, timeout=args.timeout)
    out["ref_rc"], out["ref_wall_s"] = r.returncode, ref_s
    t = marks(r.stderr)
    if len(t) > 2:
        ks = sorted(t)
        out["ref_ms_per_step"] = 1e3 * (t[ks[-1]] - t[ks[0]]) / (ks[-1] - ks[0])
    ref_log = make_golden.parse_log(r.stdout)
    out["ref_tail"] = r.stdout[-400:]
    e, eng_s = run([os.path.join(ROOT, "se-grain-growth-gpu_gb300", "sevc"), "-c", dirs["eng"][0],
                    "--honor-leave-percent"], timeout=args.timeout)
    out["eng_rc"], out["eng_wall_s"] = e.returncode, eng_s
    eng_log = make_golden.parse_log(e.stdout)
    out["steps"] = [len(ref_log), len(eng_log)]
    first = None
    for a, b in zip(ref_log, eng_log):
        if a != b:
            first = {"step": a["n"], "ref": a, "eng": b}
            break
    if first is None and len(ref_log) != len(eng_log):
        first = {"step": min(len(ref_log), len(eng_log)), "note": "runs of different length"}
    out["first_log_difference"] = first
    out["log_steps_differing"] = sum(1 for a, b in zip(ref_log, eng_log) if a != b)
    out["two_three_steps"] = sum(1 for s in ref_log if any(s["two_three"]))
    fr = sorted(os.listdir(dirs["ref"][1])) if os.path.isdir(dirs["ref"][1]) else []
    fe = sorted(os.listdir(dirs["eng"][1])) if os.path.isdir(dirs["eng"][1]) else []
    out["snapshots"] = [len(fr), len(fe)]
    nbytes = ntopo = 0
    first_bytes = first_topo = None
    for a, b in zip(fr, fe):
        pa, pb = os.path.join(dirs["ref"][1], a), os.path.join(dirs["eng"][1], b)
        da, db = snapshot.digests(pa), snapshot.digests(pb)
        if da[0] == db[0]:
            nbytes += 1
        elif first_bytes is None:
            first_bytes = a
        if da[1] == db[1]:
            ntopo += 1
        elif first_topo is None:
            first_topo = a
    out.update({"snapshots_identical_bytes": nbytes, "snapshots_identical_integers": ntopo,
                "first_snapshot_text_difference": first_bytes, "first_snapshot_integer_difference": first_topo})
    if first_bytes is not None:
        out["text_difference_detail"] = text_difference(os.path.join(dirs["ref"][1], first_bytes),
                                                        os.path.join(dirs["eng"][1], first_bytes))
    subprocess.run(["rm", "-rf", tmp])
    return out


def text_difference(a, b):
    """first differing line of two snapshots and the largest relative
    difference of each float column of the tables"""
    import numpy as np
    import snapshot
    la, lb = open(a).read().splitlines(), open(b).read().splitlines()
    first = next((i for i, (x, y) in enumerate(zip(la, lb)) if x != y), None)
    pa, pb = snapshot.parse(a), snapshot.parse(b)
    rel = {}
    for k in ("v_float", "b_float", "g_float"):
        x, y = pa[k], pb[k]
        if x.shape != y.shape:
            rel[k] = "shape"
            continue
        d = np.abs(x - y) / np.maximum(np.maximum(np.abs(x), np.abs(y)), 1e-300)
        d[x == y] = 0
        rel[k] = [float(v) for v in d.max(axis=0)]
    return {"line": first, "ref": la[first] if first is not None else None,
            "eng": lb[first] if first is not None else None, "max_rel_by_column": rel}


def timing(args):
    import numpy as np
    import meshgen
    import sevc
    sys.path.insert(0, ROOT)
    import bench
    n = args.grains
    tmp = tempfile.mkdtemp(prefix="cmpt_")
    mesh = bench.make_mesh(n, 2024)
    paths = meshgen.write_files(tmp, mesh)
    opt = bench.workload_options(sevc, n, args.nmax)
    ini = os.path.join(tmp, "run.ini")
    with open(ini, "w") as f:
        f.write("[Temporal]\ndt=%r\ndtau=%r\nnmax=%d\nsnap_gap=100000000\n[Grains]\nn_grains=%d\n"
                "vertex_fname=%s\nboundary_fname=%s\norientation_fname=%s\nSE_fname=%s\n"
                "GB_eps=0.0\nGB_scaling=1.0\nSE_eps=1\ndomain_bound=%r\ndo_nucleation=true\nMC_k=1.0\n"
                "[System]\nn_blocks=32\nn_threads=256\ndebug_lvl=0\n[Output]\nfolder=%s\n"
                % (opt.dt, opt.dtau, args.nmax, n, paths["vertices"], paths["ridges"], paths["oris"], paths["se"],
                   opt.domain_bound, os.path.join(tmp, "out")))
    # the loop runs only while min_grains > 0 (src/main.cu:120): 1 never stops it here
    env = dict(os.environ, SEVC_REF_MIN_GRAINS="1", SEVC_REF_SNAPSHOTS="0")
    r, ref_s = run([os.path.join(OUT, args.exe), "-c", ini], env=env, timeout=args.timeout)
    t = marks(r.stderr)
    ks = sorted(t)
    per = [t[ks[i + 1]] - t[ks[i]] for i in range(len(ks) - 1)]
    out = {"exe": args.exe, "grains": n, "ref_rc": r.returncode, "ref_wall_s": ref_s,
           "ref_step_s": per, "ref_tail": r.stdout[-300:]}
    opt2 = sevc.load_ini(ini)
    opt2.min_grains = -1
    eng = sevc.Engine.from_files(opt2)
    eng.step()
    sec = []
    for _ in range(args.nmax):
        w0 = time.time()
        eng.step()
        sec.append(time.time() - w0)
    eng.close()
    out["eng_step_s"] = sec
    if per:
        out["ref_vertex_steps_per_s"] = 2 * n / float(np.median(per))
        out["eng_vertex_steps_per_s"] = 2 * n / float(np.median(sec))
    subprocess.run(["rm", "-rf", tmp])
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("mode", choices=["events", "timing"])
    ap.add_argument("--exe", default="sevc_ref_gpu_nofma")
    ap.add_argument("--config", default="example_ref2k")
    ap.add_argument("--nmax", type=int, default=None)
    ap.add_argument("--grains", type=int, default=1000000)
    ap.add_argument("--timeout", type=float, default=900)
    ap.add_argument("--json", default=None)
    a = ap.parse_args()
    res = events(a) if a.mode == "events" else timing(a)
    s = json.dumps(res, indent=1)
    print(s)
    if a.json:
        with open(a.json, "w") as f:
            f.write(s)


if __name__ == "__main__":
    main()
