#!/usr/bin/env python3
"""Benchmark: vertex-steps/s of the vertex-model time step on one GB300.

Workload ("1M-grain stored-energy + nucleation"): periodic Voronoi
microstructure from 1,000,000 uniform seeds (V = 2M triple junctions,
B = 3M boundaries), FP64, isotropic boundaries (GB_eps = 0, gamma = 1),
per-grain stored energy lognormal(mu=-1, sigma=0.5), Monte-Carlo nucleation
on (one attempt every nucleation_gap = 10 steps once 1/6 of the grains are
gone, the reference's rule), domain [0, 1000)^2 so that grains are about one
unit across as in the reference's example.ini, dt = 1e-4 (example.ini).
Inputs are synthetic (seeded generator); there is no dataset.

A "step" is one iteration of the reference's main loop (src/main.cu:121-389).
metric = sum over timed steps of the enabled vertices / time.

  value    device time (CUDA events on the engine's stream), mesh resident
           in HBM, K steps after W warm-up steps;
  e2e      the same through the C ABI from host buffers: upload of the mesh,
           K steps with the per-step summary read back, download of the
           final state - all inside the timed region;
  roofline per-kernel CUDA-event times from a profiling pass of the same
           workload; algorithmic bytes per launch are stated in the design doc.

--impl reference times the reference's algorithm on the host cores: the
oracle restatement (the reference's CUDA program cannot run on the GPU machine:
its sources are not there and binaries built elsewhere are x86).
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "se-grain-growth-gpu_gb300")
sys.path.insert(0, PKG)
sys.path.insert(0, ROOT)

METRIC = "vertex-steps/s at 1M grains"
UNIT = "vertex-steps/s"


def workload_options(mod, n, steps):
    kw = dict(n_grains=n, dt=1e-4, dtau=1e-3, nucleation_gap=10, domain_bound=1000.0, GB_eps=0.0, GB_scaling=1.0,
              SE_eps=1.0, SE_min=999.0, SE_max=999.0, do_nucleation=1, MC_k=1.0, nmax=10 ** 8, tmax=-1,
              snap_gap=10 ** 8, min_grains=-1, n_blocks=32, n_threads=256)
    o = mod.default_options(**kw)
    o.min_grains = -1
    return o


class Clocks:
    """nvidia-smi samples during the timed region."""

    def __init__(self):
        self.samples, self.proc = [], None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "--query-gpu=clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
                 "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
                 "clocks_event_reasons.sw_power_cap", "--format=csv,noheader,nounits", "-lms", "200", "-i", "0"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.samples.append([x.strip() for x in line.split(",")])

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        sm = sorted(float(s[0]) for s in self.samples if s and s[0].replace(".", "").isdigit())
        mx = [float(s[1]) for s in self.samples if len(s) > 1 and s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4) if len(s) > 3 + i and s[3 + i] == "Active"})
        return {"sm_mhz": sm[len(sm) // 2] if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def make_mesh(n, seed, cache=None):
    import numpy as np
    if cache and os.path.exists(cache):
        z = np.load(cache)
        if int(z["n_grains"]) == n:
            return {k: z[k] for k in z.files}
    import meshgen
    mesh = meshgen.make_inputs(n, seed, se="lognormal", se_params=(-1.0, 0.5))
    if cache:
        np.savez(cache, **mesh)
    return mesh


def algorithmic_bytes_per_step(nv):
    """Compulsory traffic of one step per vertex (131.5 B per vertex-step:
    72*V + 25*B + 20*G + 4*sum(vlen) with B = 1.5V, G = V/2, sum(vlen) = 3V)."""
    return 131.5 * nv


# algorithmic bytes per unit for each kernel (kernel table)
KERNEL_BYTES = {
    # per grain: list 4*vlen + vlen/SE/area/gq/enabled 29 + positions 16*V/G + grain
    # slots of the listed vertices 16*V/G + stored-energy terms 48*V/G
    "grain_fd": ("grains", 24 + 29 + 32 + 32 + 96),
    # per vertex: pos 16 + slots 32 + 3 boundary ends 24 + 3 neighbour positions 48 (shared) +
    # gamma/length 48 + terms in 48 + grain q 24 + vel/terms/energy out 56
    "vertex_fd": ("vertices", 16 + 32 + 24 + 24 + 48 + 48 + 24 + 56),
    # per boundary: ends 8 + positions 32 + velocities 32 + t_ext 8 + flags 2
    "text_label": ("boundaries", 8 + 32 + 32 + 8 + 2),
}


def run_engine(args):
    import sevc
    n = args.grains
    t0 = time.time()
    mesh = make_mesh(n, args.seed, args.mesh_cache)
    gen_s = time.time() - t0
    opt = workload_options(sevc, n, args.steps)
    host_bytes = mesh["xy"].nbytes + mesh["ridges"].nbytes + mesh["oris"].nbytes + mesh["se"].nbytes

    # ---------------- device-resident leg ----------------
    eng = sevc.Engine.from_arrays(opt, mesh["xy"], mesh["ridges"], mesh["oris"], mesh["se"])
    g = n
    for _ in range(args.warmup):
        g = eng.step().curr_n_grains
    clocks = Clocks()
    clocks.start()
    ms, vsteps, infos = 0.0, 0, []
    w0 = time.time()
    for _ in range(args.steps):
        vsteps += 2 * g          # enabled vertices at the start of the step (V = 2G)
        info = eng.step()
        infos.append(info)
        ms += info.gpu_ms
        g = info.curr_n_grains
    wall = time.time() - w0
    ck = clocks.stop()
    value = vsteps / (ms / 1e3)

    # ---------------- profiling pass (per-kernel event times) ----------------
    eng.set_profiling(True)
    for _ in range(max(1, args.prof_steps)):
        eng.step()
    prof = eng.profile()
    eng.close()
    tot = sum(v[0] for v in prof.values())
    dom = max((k for k in prof if k in KERNEL_BYTES), key=lambda k: prof[k][0])
    unit, per_unit = KERNEL_BYTES[dom]
    units = {"grains": g, "vertices": 2 * g, "boundaries": 3 * g}[unit]
    avg_ms = prof[dom][0] / prof[dom][1]
    achieved = per_unit * units / (avg_ms / 1e3) / 1e9
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except OSError:
        pass
    peak = peaks.get("hbm_gbs", 6800.0)

    # ---------------- end-to-end leg through the C ABI ----------------
    e0 = time.time()
    eng = sevc.Engine.from_arrays(opt, mesh["xy"], mesh["ridges"], mesh["oris"], mesh["se"])
    e_vsteps = 0
    g = n
    for _ in range(args.steps):
        info = eng.step()
        e_vsteps += 2 * g
        g = info.curr_n_grains
    st = eng.get_state()
    e_wall = time.time() - e0
    eng.close()
    state_bytes = sum(a.nbytes for a in st.values())
    step_info_bytes = 8 * 4 * 3  # counters read back per step

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic (seeded periodic Voronoi, lognormal stored energy)",
        "config": {"workload": "1M-grain stored-energy + nucleation vertex model", "grains": n,
                   "vertices": 2 * n, "boundaries": 3 * n, "dt": 1e-4, "nucleation_gap": 10,
                   "domain_bound": 1000.0, "GB_eps": 0.0, "se": "lognormal(-1,0.5)",
                   "l2": "working set > L2 (129 MB): ~1 GB of mesh state per step",
                   "removals_per_step": sum(i.n_removals for i in infos) / len(infos),
                   "flips_per_step": sum(i.n_flips for i in infos) / len(infos),
                   "nucleation_attempts": sum(i.nucleation_attempted for i in infos),
                   "mesh_generation_s": round(gen_s, 1), "wall_s": round(wall, 3)},
        "e2e": {"value": e_vsteps / e_wall, "unit": UNIT, "h2d_bytes_per_step": host_bytes / args.steps,
                "d2h_bytes_per_step": step_info_bytes + state_bytes / args.steps},
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": None, "peak_source": "MEASURED_PEAKS.json hbm_gbs",
                     "note": "FP64-pipe bound on GB300; see DESIGN.md"},
        "kernel_ms_share": {k: round(v[0] / tot, 4) for k, v in sorted(prof.items(), key=lambda kv: -kv[1][0])},
        "step_bytes_rate_gbs": algorithmic_bytes_per_step(2 * n) * args.steps / (ms / 1e3) / 1e9,
        "gpu_launches": sum(i.kernel_launches for i in infos),
        "kernel_ms_per_step": {k: round(v[0] / v[1] if v[1] else 0, 4) for k, v in prof.items()},
        "clocks": ck,
    }
    if args.cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(mesh, n, args.cpu_steps)
    print(json.dumps(line))


def cpu_baseline(mesh, n, steps):
    from oracle import oracle as O
    O.build()
    opt = workload_options(O, n, steps)
    O.finish_options(opt)
    opt.min_grains = -1
    orc = O.Oracle.from_arrays(opt, mesh["xy"], mesh["ridges"], mesh["oris"], mesh["se"])
    cores = os.cpu_count() or 1
    orc.set_threads(cores)
    vs, t0 = 0, time.time()
    for _ in range(steps):
        g = orc.s.curr_n_grains
        orc.step()
        orc.finish_step()
        vs += 2 * g
    dt = time.time() - t0
    return {"value": vs / dt, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": "%d steps of the same 1M-grain workload (oracle restatement, OpenMP)" % steps}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    mesh = make_mesh(args.grains, args.seed, args.mesh_cache)
    from oracle import oracle as O
    O.build()
    opt = workload_options(O, args.grains, args.steps)
    O.finish_options(opt)
    opt.min_grains = -1
    orc = O.Oracle.from_arrays(opt, mesh["xy"], mesh["ridges"], mesh["oris"], mesh["se"])
    cores = os.cpu_count() or 1
    orc.set_threads(cores)
    for _ in range(args.warmup):
        orc.step()
        orc.finish_step()
    vs, t0 = 0, time.time()
    for _ in range(args.steps):
        g = orc.s.curr_n_grains
        orc.step()
        orc.finish_step()
        vs += 2 * g
    dt = time.time() - t0
    v = vs / dt
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": dt * 1e3 / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "1M-grain stored-energy + nucleation vertex model", "grains": args.grains},
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": "%d steps of the 1M-grain workload on the host cores" % args.steps},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="engine", choices=["engine", "reference"])
    ap.add_argument("--grains", type=int, default=1000000)
    ap.add_argument("--seed", type=int, default=2024)
    ap.add_argument("--prof-steps", type=int, default=5)
    ap.add_argument("--cpu-steps", type=int, default=2)
    ap.add_argument("--mesh-cache", default=None, help="npz file to reuse the generated mesh")
    ap.add_argument("--no-cpu-baseline", dest="cpu_baseline", action="store_false")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
        return
    if int(os.environ.get("RANK", "0")) != 0 and args.gpus > 1:
        return
    import __graft_entry__
    __graft_entry__.build()
    run_engine(args)


if __name__ == "__main__":
    main()
