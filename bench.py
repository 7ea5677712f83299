#!/usr/bin/env python3
"""Benchmark: vertex-steps/s of the vertex-model time step on one GB300.

Workload ("1M-grain stored-energy + nucleation"): periodic Voronoi
microstructure from 1,000,000 uniform seeds (V = 2M triple junctions,
B = 3M boundaries), FP64, isotropic boundaries (GB_eps = 0, gamma = 1),
per-grain stored energy lognormal(mu=-1, sigma=0.5), Monte-Carlo nucleation
on (one attempt every nucleation_gap = 10 steps once 1/6 of the grains are
gone, the reference's rule), domain [0, 1000)^2 so that grains are about one
unit across as in the reference's example.ini, dt = 2e-4.  The run is the
configuration's: 10,000 steps or until 20% of the grains remain; the 5/6
gate is passed after about 7,000 steps, so the last ~3,000 steps carry
nucleation attempts and tens of removals and flips per step.
Inputs are synthetic (seeded generator); there is no dataset.

A "step" is one iteration of the reference's main loop (src/main.cu:121-389).
metric = sum over timed steps of the enabled vertices / time.

  value     device time (CUDA events on the engine's stream), mesh resident
            in HBM, of K steps starting W steps past the nucleation gate
            (from a checkpoint; the event-heavy phase of the run);
  e2e       the configuration's whole run through the C ABI from host
            buffers: mesh build and upload, every step with its summary
            read back, download of the final state - all inside the timed
            region;
  t0_window the first K steps after W of the same run (hardly any events);
  roofline  per-kernel CUDA-event times from a profiling pass of the same
            window; algorithmic bytes per launch are KERNEL_BYTES below.

--impl reference times the reference's algorithm on the host cores: the
oracle restatement (the reference's CUDA program is not part of this
benchmark: its sources do not travel with the repository), on the t = 0
window of the same configuration (a CPU cannot reach the gate in a bounded
sample; the oracle's cost per step hardly depends on the phase).
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


FULL_STEPS = 10000     # the configuration's run: 10,000 steps ...
LEAVE = 0.2            # ... or until 20% of the grains remain


def workload_options(mod, n, steps):
    kw = dict(n_grains=n, dt=2e-4, dtau=2e-3, nucleation_gap=10, domain_bound=1000.0, GB_eps=0.0, GB_scaling=1.0,
              SE_eps=1.0, SE_min=999.0, SE_max=999.0, do_nucleation=1, MC_k=1.0, nmax=10 ** 8, tmax=-1,
              snap_gap=10 ** 8, min_grains=-1, n_blocks=32, n_threads=256)
    o = mod.default_options(**kw)
    o.min_grains = -1
    return o


def current_gpu_bus_id():
    """PCI bus id of this process's CUDA device 0 (the first one visible
    under CUDA_VISIBLE_DEVICES), the id nvidia-smi -i takes; None if the
    runtime cannot say."""
    import ctypes
    import glob
    for name in ["libcudart.so"] + sorted(glob.glob("/usr/local/cuda/lib64/libcudart.so*")):
        try:
            rt = ctypes.CDLL(name)
        except OSError:
            continue
        buf = ctypes.create_string_buffer(64)
        if rt.cudaDeviceGetPCIBusId(buf, 64, 0) == 0:
            return buf.value.decode()
        return None
    return None


class Clocks:
    """nvidia-smi samples of this process's GPU during the timed region."""

    def __init__(self):
        self.samples, self.proc = [], None
        self.gpu = current_gpu_bus_id()

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "--query-gpu=clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
                 "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
                 "clocks_event_reasons.sw_power_cap", "--format=csv,noheader,nounits", "-lms", "50",
                 "-i", self.gpu or "0"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
            t0 = time.time()                 # the timed region starts once sampling runs
            while not self.samples and time.time() - t0 < 3.0:
                time.sleep(0.01)
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
                "reasons": reasons, "samples": len(self.samples), "gpu": self.gpu or "index 0"}


def make_mesh(n, seed, cache=None):
    import numpy as np
    if cache and os.path.exists(cache):
        z = np.load(cache)
        if int(z["n_grains"]) == n:
            return {k: z[k] for k in z.files}
    import meshgen
    mesh = meshgen.make_inputs(n, seed, se="lognormal", se_params=(-1.0, 0.5), generator="c")
    if cache:
        np.savez(cache, **mesh)
    return mesh


def make_ensemble(n_inst, lo, hi, seed, cache=None):
    """n_inst periodic Voronoi meshes, grain counts uniform in [lo, hi],
    per-instance seeds, stored energy U[0,1) (rescaled to [0, 0.5] by
    SE_min/SE_max in the options)."""
    import numpy as np
    key = "%d_%d_%d_%d" % (n_inst, lo, hi, seed)
    if cache and os.path.exists(cache):
        z = np.load(cache)
        if str(z["key"]) == key:
            return [{f: z["%s%d" % (f, i)] for f in ("xy", "ridges", "oris", "se")} for i in range(n_inst)]
    import meshgen
    rng = np.random.default_rng(seed)
    sizes = rng.integers(lo, hi + 1, n_inst)
    meshes = [meshgen.make_inputs(int(n), seed * 100003 + i, generator="c") for i, n in enumerate(sizes)]
    if cache:
        np.savez(cache, key=key, **{"%s%d" % (f, i): m[f] for i, m in enumerate(meshes)
                                    for f in ("xy", "ridges", "oris", "se")})
    return meshes


def ensemble_options(mod, n):
    """Unit square, gamma = 1, SE U[0, 0.5], dt = 1e-6; nucleation on with
    dtau = 0.1 (a rate of 1e-3 per grain per unit time at 10,000 grains, one
    Metropolis attempt per dtau as the reference does)."""
    kw = dict(n_grains=n, dt=1e-6, dtau=0.1, nucleation_gap=100000, domain_bound=1.0, GB_eps=0.0, GB_scaling=1.0,
              SE_eps=1.0, SE_min=0.0, SE_max=0.5, do_nucleation=1, MC_k=1.0, nmax=10 ** 8, tmax=-1,
              snap_gap=10 ** 8, min_grains=-1, n_blocks=32, n_threads=256)
    o = mod.default_options(**kw)
    o.min_grains = -1
    return o


def run_ensemble(n_inst, lo, hi, steps, warmup, seed=7, cache=None):
    """Batched handle against the same instances run one after another as
    plain handles (same output rule as the batch).  Times are
    wall clock around the steps (the host round trips of every step are
    part of what batching removes)."""
    import sevc
    t0 = time.time()
    meshes = make_ensemble(n_inst, lo, hi, seed, cache)
    gen_s = time.time() - t0
    grains = [len(m["oris"]) for m in meshes]
    opt = ensemble_options(sevc, grains[0])
    batch = sevc.Engine.from_batch(opt, meshes)
    g = sum(grains)
    for _ in range(warmup):
        g = batch.step().curr_n_grains
    shapes = batch.autotune(2)
    vs, ms = 0, 0.0
    w0 = time.time()
    for _ in range(steps):
        vs += 2 * g
        info = batch.step()
        ms += info.gpu_ms
        g = info.curr_n_grains
    batch_wall = time.time() - w0
    batch.close()
    seq_wall, seq_vs = 0.0, 0
    for m in meshes:
        o = ensemble_options(sevc, len(m["oris"]))
        e = sevc.Engine.from_arrays(o, m["xy"], m["ridges"], m["oris"], m["se"])
        gi = len(m["oris"])
        for _ in range(warmup):
            gi = e.step().curr_n_grains
        w0 = time.time()
        for _ in range(steps):
            seq_vs += 2 * gi
            gi = e.step().curr_n_grains
        seq_wall += time.time() - w0
        e.close()
    return {"instances": n_inst, "grains_range": [lo, hi], "total_grains": int(sum(grains)), "steps": steps,
            "warmup": warmup, "batch_ms_per_step": 1e3 * batch_wall / steps,
            "batch_device_ms_per_step": ms / steps, "sequential_ms_per_step": 1e3 * seq_wall / steps,
            "batch_vertex_steps_per_s": vs / batch_wall, "sequential_vertex_steps_per_s": seq_vs / seq_wall,
            "speedup": seq_wall / batch_wall, "mesh_generation_s": round(gen_s, 1),
            "batch_launch_shapes": list(shapes),
            "timing": "wall clock around the steps, inputs resident on the device"}


def run_adjoint(n=10000, steps=2000, every=100, dt=4e-6, seed=17, nbins=20, amax=3.0):
    """Forward + adjoint of the 10,000-grain differentiable workload: unit
    square, SE U[0, 0.5], gamma = mu = 1, histogram loss after `steps`
    steps, checkpoints every `every` steps; dt = 4e-6 so that the window
    holds flips and removals (about 190 of each).  Wall-clock times of the
    steps (forward, with the tape) and of the adjoint call (replay +
    backward)."""
    import numpy as np
    import sevc
    import meshgen
    mesh = meshgen.make_inputs(n, seed)
    se = np.random.default_rng(seed).uniform(0.0, 0.5, n)
    o = sevc.default_options(n_grains=n, dt=dt, dtau=1.0, domain_bound=1.0, GB_eps=0.0, GB_scaling=1.0, SE_eps=1.0,
                             SE_min=999.0, SE_max=999.0, do_nucleation=0, nmax=10 ** 8, tmax=-1, snap_gap=10 ** 8,
                             n_blocks=32, n_threads=256)
    o.min_grains = -1
    eng = sevc.Engine.from_arrays(o, mesh["xy"], mesh["ridges"], mesh["oris"], mesh["se"])
    eng.set_stored_energy(se)
    eng.tape_start(every)
    ev = np.zeros(3, np.int64)
    t0 = time.time()
    for _ in range(steps):
        i = eng.step()
        ev += (i.n_flips, i.n_removals, i.n_two_three)
    fwd = time.time() - t0
    h = eng.area_histogram(nbins, amax)
    target = np.full(nbins, 1.0 / nbins)
    t0 = time.time()
    gse, ggam, gmu = eng.adjoint_histogram(nbins, amax, 2.0 * (h - target) / nbins)
    bwd = time.time() - t0
    eng.close()
    return {"grains": n, "steps": steps, "checkpoint_every": every, "dt": dt, "forward_s": fwd, "backward_s": bwd,
            "backward_forward_ratio": bwd / fwd, "events": {"flips": int(ev[0]), "removals": int(ev[1]),
                                                           "two_three": int(ev[2])},
            "grad_gb_scaling": ggam, "grad_mu": gmu,
            "timing": "wall clock; forward = the taped steps, backward = sevc_adjoint_histogram"}


def run_calibration(n_inst=16, lo=2000, hi=5000, steps=200, iters=30, dt=2e-3, seed=5, nucleation=None):
    """Batched calibration of (gamma, mu, stored-energy scale) by Adam steps
    through the adjoint, against the histogram of the same batch run with
    the generating values (1, 1, 1); grains about one unit across (domain
    sqrt of the mean grain count), SE U[0,1).  nucleation (gap, MC_k): the
    window starts once every instance has passed its 5/6 gate, with stored
    energies triangular(3, 6, 6) (voronoi.py's, where the Metropolis test
    accepts nucleations at this grain size; the motion is then ~10x faster
    than with U[0,1), so dt is smaller to keep the window's removals to a
    few per thousand grains, where the loss is smooth enough between
    discrete events for gradient steps)."""
    import numpy as np
    import meshgen
    import calibrate
    rng = np.random.default_rng(seed)
    sizes = rng.integers(lo, hi + 1, n_inst)
    se = "triangular" if nucleation else "uniform"
    meshes = [meshgen.make_inputs(int(n), 100 + i, se=se, generator="c") for i, n in enumerate(sizes)]
    return calibrate.run(meshes, dt=dt, steps=steps, iters=iters, checkpoint_every=50,
                         domain=float(np.sqrt(sizes.mean())), nucleation=nucleation)


LAUNCH_MODES = {"graph": 1, "hostloops": 2, "direct": 0}


def run_window(args):
    """The main workload's mesh at --grains, run to W steps past the 5/6
    nucleation gate and saved to --ckpt (or loaded from it when it exists),
    then K steps: a short launch sequence from the event-heavy phase, for
    profilers (the first call makes the checkpoint, the profiled call only
    loads it and steps)."""
    import sevc
    n = args.grains
    mesh = make_mesh(n, args.seed, args.mesh_cache)
    opt = workload_options(sevc, n, args.steps)
    opt.domain_bound = float(n) ** 0.5
    eng = sevc.Engine.from_arrays(opt, mesh["xy"], mesh["ridges"], mesh["oris"], mesh["se"])
    made = False
    eng.set_graphs(LAUNCH_MODES[args.launch])
    if args.ckpt and os.path.exists(args.ckpt):
        eng.checkpoint_load(args.ckpt)
    else:
        g, k, gate = n, 0, None
        while gate is None or k < gate + args.warmup:
            g = eng.step().curr_n_grains
            k += 1
            if gate is None and g <= 5 * n // 6:
                gate = k
            if k > FULL_STEPS:
                raise RuntimeError("no gate within %d steps" % FULL_STEPS)
        if args.ckpt:
            eng.checkpoint_save(args.ckpt)
        made = True
    if args.ckpt:
        # three untimed steps (first launches load kernel code, graphs are
        # captured), then the checkpoint again: the window is the same steps
        for _ in range(3):
            eng.step()
        eng.checkpoint_load(args.ckpt)
    g0 = eng.grain_stats(-1)["n_grains"]
    ms, vs, g, ev = 0.0, 0, g0, [0, 0, 0]
    for _ in range(args.steps):
        vs += 2 * g
        i = eng.step()
        ms += i.gpu_ms
        g = i.curr_n_grains
        ev = [ev[0] + i.n_flips, ev[1] + i.n_removals, ev[2] + i.nucleation_attempted]
    eng.close()
    return {"grains": n, "value": vs / (ms / 1e3), "ms_per_step": ms / args.steps, "checkpoint_made": made,
            "grains_at_window": g0, "flips": ev[0], "removals": ev[1], "nucleation_attempts": ev[2]}


def run_small(steps, seed=1, n=2000):
    """The small plain configuration: 2,000 grains on the unit square, SE
    U[0, 0.5], dt = 1e-6, no nucleation.  The engine and the oracle (serial
    and with every host core) run the same steps; the per-step event counts
    and grain counts are compared."""
    import numpy as np
    import sevc
    import meshgen
    from oracle import oracle as O
    O.build()
    mesh = meshgen.make_inputs(n, seed)
    kw = dict(n_grains=n, dt=1e-6, dtau=1.0, domain_bound=1.0, GB_eps=0.0, GB_scaling=1.0, SE_eps=1.0,
              SE_min=0.0, SE_max=0.5, do_nucleation=0, nmax=10 ** 8, tmax=-1, snap_gap=10 ** 8,
              n_blocks=32, n_threads=256)
    o = sevc.default_options(**kw)
    o.min_grains = -1
    e = sevc.Engine.from_arrays(o, mesh["xy"], mesh["ridges"], mesh["oris"], mesh["se"])
    ev_gpu, vs = [], 0
    g = n
    t0 = time.time()
    for _ in range(steps):
        vs += 2 * g
        i = e.step()
        g = i.curr_n_grains
        ev_gpu.append((i.curr_n_grains, i.n_flips, i.n_removals, i.n_two_three))
    gpu_s = time.time() - t0
    e.close()
    out = {"grains": n, "steps": steps, "grains_left": g, "gpu_vertex_steps_per_s": vs / gpu_s,
           "gpu_ms_per_step": 1e3 * gpu_s / steps}
    for threads in (1, os.cpu_count() or 1):
        opt = O.default_options(**kw)
        O.finish_options(opt)
        opt.min_grains = -1
        orc = O.Oracle.from_arrays(opt, mesh["xy"], mesh["ridges"], mesh["oris"], mesh["se"])
        orc.set_threads(threads)
        ev, vs_c, g = [], 0, n
        t0 = time.time()
        for _ in range(steps):
            vs_c += 2 * g
            orc.step()
            orc.finish_step()
            s = orc.s
            g = s.curr_n_grains
            ev.append((s.curr_n_grains, s.ev_flips, s.ev_removals, s.ev_two_three))
        cpu_s = time.time() - t0
        out["cpu_%d_threads_vertex_steps_per_s" % threads] = vs_c / cpu_s
        out["events_identical_%d" % threads] = ev == ev_gpu
    out["events"] = [int(x) for x in np.array(ev_gpu)[:, 1:].sum(0)]
    return out


def algorithmic_bytes_per_step(nv):
    """Compulsory traffic of one step per vertex (131.5 B per vertex-step:
    72*V + 25*B + 20*G + 4*sum(vlen) with B = 1.5V, G = V/2, sum(vlen) = 3V)."""
    return 131.5 * nv


# algorithmic bytes per unit for each kernel phase (compulsory traffic, each datum once)
KERNEL_BYTES = {
    # per grain: list 4*vlen + vlen/SE/area/gq/enabled 29 + positions 16*V/G + grain
    # slots of the listed vertices 16*V/G + stored-energy terms 48*V/G
    "grain_fd": ("grains", 24 + 29 + 32 + 32 + 96),
    # per vertex: pos 16 + slots 32 + 3 boundary ends 24 + 3 neighbour positions 48 (shared) +
    # gamma/length 48 + terms in 48 + grain q 24 + vel/terms/energy out 56
    "vertex_fd": ("vertices", 16 + 32 + 24 + 24 + 48 + 48 + 24 + 56),
    # per boundary decided by the speed bound (nearly all): enabled 1 + ends 8 + arclength 8 +
    # the ends' speed bounds 8, then t_ext 8, exact flag 1, candidate 1, conflict 4 written
    # (the few others also read both ends' positions and velocities, 64)
    "text_label": ("boundaries", 1 + 8 + 8 + 8 + 8 + 1 + 1 + 4),
}

# DRAM bytes (read + write) per unit measured by ncu for each kernel phase on
# the 200K-grain mesh (the ncu summaries of k_grain_fd_sorted and
# k_vertex_fd under profiles/); traffic grows with the units processed, so
# a full launch is scaled by its units.
NCU_TRAFFIC_PER_UNIT = {
    "grain_fd": (52.807e6 + 11.475e6) / 200000,
    "vertex_fd": (50.061e6 + 0.945e6) / 400000,
}
# FP64 pipe activity of the same captures (of elapsed cycles)
NCU_FP64_ACTIVE = {"grain_fd": 0.557, "vertex_fd": 0.650}
# DADD + DMUL + DFMA thread instructions per unit, ncu counters on the
# 200K-grain mesh (the FP64 instruction summary kept with the profiles)
NCU_FP64_INST_PER_UNIT = {"grain_fd": (46.032e6 + 0.702e6) / 200000, "vertex_fd": 24.405e6 / 400000}


def run_engine(args):
    """The 1M-grain workload in three legs.

    full run  the configuration's whole run (10,000 steps or until 20% of
              the grains remain) through the C ABI from host buffers:
              host mesh build and upload, every step with its summary
              read back, the final state downloaded -> e2e.  On the way it
              saves a checkpoint W steps after the 5/6 nucleation gate.
    window    from that checkpoint: K steps timed with CUDA events on the
              engine's stream (mesh resident) -> value; then the same K
              steps again with per-kernel events -> roofline.
    cpu       the oracle built from the window's starting state, on every
              host core -> cpu_baseline (same window).
    """
    import tempfile

    import numpy as np
    import sevc
    n = args.grains
    t0 = time.time()
    mesh = make_mesh(n, args.seed, args.mesh_cache)
    gen_s = time.time() - t0
    opt = workload_options(sevc, n, args.steps)
    host_bytes = mesh["xy"].nbytes + mesh["ridges"].nbytes + mesh["oris"].nbytes + mesh["se"].nbytes
    tmpdir = tempfile.mkdtemp(prefix="sevc_bench_")
    ckpt = os.path.join(tmpdir, "window.ckpt")
    W, K = args.warmup, args.steps

    # ---------------- full run, end to end through the C ABI ----------------
    e0 = time.time()
    eng = sevc.Engine.from_arrays(opt, mesh["xy"], mesh["ridges"], mesh["oris"], mesh["se"])
    eng.set_graphs(LAUNCH_MODES[args.launch])
    g, vs, ms_full, k = n, 0, 0.0, 0
    gate, ck_s, win_state, t0_ms, t0_vs = None, 0.0, None, 0.0, 0
    ev_full = np.zeros(5, np.int64)
    lost = 64                                  # most grains one step has removed so far, and a margin
    while k < FULL_STEPS and g > LEAVE * n:
        if gate is not None and k == gate + W and win_state is None:
            c0 = time.time()                     # excluded from the e2e time
            eng.checkpoint_save(ckpt)
            win_state = (eng.get_state(), k)
            ck_s += time.time() - c0
        # sevc_run keeps two steps in flight; a chunk ends before the stop
        # threshold, the 5/6 gate or the checkpoint step could fall inside it
        # (single steps near them), so the run takes the configuration's
        # steps exactly
        chunk = min(100, FULL_STEPS - k)
        if g - LEAVE * n <= 2 * chunk * lost or (gate is None and g - 5 * n // 6 <= 2 * chunk * lost):
            chunk = 1
        if gate is not None and win_state is None:
            chunk = min(chunk, gate + W - k)
        for info in eng.run(chunk):
            vs += 2 * g
            ms_full += info.gpu_ms
            if W <= k < W + K:                 # the first K steps after W: the t = 0 window
                t0_ms += info.gpu_ms
                t0_vs += 2 * g
            lost = max(lost, g - info.curr_n_grains + 64)
            g = info.curr_n_grains
            ev_full += (info.n_flips, info.n_removals, info.n_two_three, info.nucleation_attempted, info.n_nucleations)
            k += 1
            if gate is None and g <= 5 * n // 6:
                gate = k
    st_final = eng.get_state()
    e_wall = time.time() - e0 - ck_s
    eng.close()
    state_bytes = sum(a.nbytes for a in st_final.values())
    del st_final
    if win_state is None:
        raise RuntimeError("the run did not pass the nucleation gate (gate %s, %d steps)" % (gate, k))

    # ---------------- the window past the gate, device-timed ----------------
    eng = sevc.Engine.from_arrays(opt, mesh["xy"], mesh["ridges"], mesh["oris"], mesh["se"])
    eng.set_graphs(LAUNCH_MODES[args.launch])
    eng.checkpoint_load(ckpt)
    shapes = eng.autotune(10)         # launch shapes for this state (10 steps per candidate); the state is left as it was
    for _ in range(W):                # graphs captured, caches warm
        eng.step()
    eng.checkpoint_load(ckpt)
    g0 = int(win_state[0]["gen"].sum())
    clocks = Clocks()
    clocks.start()
    ms, vsteps, infos, g = 0.0, 0, [], g0
    w0 = time.time()
    for _ in range(K):
        vsteps += 2 * g          # enabled vertices at the start of the step (V = 2G)
        info = eng.step()
        infos.append(info)
        ms += info.gpu_ms
        g = info.curr_n_grains
    wall = time.time() - w0
    ck = clocks.stop()
    value = vsteps / (ms / 1e3)

    # ---------------- profiling pass of the same window ----------------
    eng.checkpoint_load(ckpt)
    eng.set_profiling(True)
    for _ in range(K):
        eng.step()
    prof = eng.profile()
    eng.close()
    tot = sum(v[0] for v in prof.values())
    dom = max((kk for kk in prof if kk in KERNEL_BYTES), key=lambda kk: prof[kk][0])
    unit, per_unit = KERNEL_BYTES[dom]
    units = {"grains": g0, "vertices": 2 * g0, "boundaries": 3 * g0}[unit]
    avg_ms = prof[dom][0] / prof[dom][1]
    achieved = per_unit * units / (avg_ms / 1e3) / 1e9
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except OSError:
        pass
    peak = peaks.get("hbm_gbs", 6800.0)
    fp64_peak = sevc.measure_fp64_rate()
    fp64 = {}
    for kk in ("grain_fd", "vertex_fd"):
        if kk in prof and prof[kk][1]:
            u = {"grains": g0, "vertices": 2 * g0, "boundaries": 3 * g0}[KERNEL_BYTES[kk][0]]
            ach = NCU_FP64_INST_PER_UNIT[kk] * u / (prof[kk][0] / prof[kk][1] / 1e3)
            fp64[kk] = {"achieved": ach, "frac": ach / fp64_peak}
    step_bytes = algorithmic_bytes_per_step(1) * vsteps / K     # per step, at the window's sizes
    ev_win = {"flips_per_step": sum(i.n_flips for i in infos) / K,
              "removals_per_step": sum(i.n_removals for i in infos) / K,
              "two_three_per_step": sum(i.n_two_three for i in infos) / K,
              "conflicts_per_step": sum(i.n_conflicts for i in infos) / K,
              "nucleation_attempts": sum(i.nucleation_attempted for i in infos),
              "nucleations": sum(i.n_nucleations for i in infos)}
    step_info_bytes = 8 * 4 * 3  # counters read back per step
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 1, "steps": K, "warmup": W,
        "ms_per_step": ms / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic (seeded periodic Voronoi, lognormal stored energy)",
        "config": {"workload": "1M-grain stored-energy + nucleation vertex model", "grains": n,
                   "vertices": 2 * n, "boundaries": 3 * n, "dt": opt.dt, "nucleation_gap": opt.nucleation_gap,
                   "domain_bound": opt.domain_bound, "GB_eps": 0.0, "se": "lognormal(-1,0.5)",
                   "window": "K steps from %d steps past the 5/6 nucleation gate (step %d of the run, %d grains)"
                             % (W, win_state[1], g0),
                   "l2": "working set > L2 (129 MB): ~1.4 GB of mesh state per step", **ev_win,
                   "mesh_generation_s": round(gen_s, 1), "wall_s": round(wall, 3),
                   "launch_shapes": {"tpb_vertex": shapes[0], "tpb_boundary": shapes[1], "wide_sides": shapes[2],
                                     "grain_blocks_per_sm": shapes[3],
                                     "picked_by": "sevc_autotune, 10 steps per candidate"},
                   "launch_mode": {"graph": "one CUDA graph per step (device-driven loops)",
                                   "hostloops": "CUDA graphs of the step's fixed sequences, loops on the host",
                                   "direct": "direct launches"}[args.launch]},
        "e2e": {"value": vs / e_wall, "unit": UNIT, "h2d_bytes_per_step": host_bytes / k,
                "d2h_bytes_per_step": step_info_bytes + state_bytes / k,
                "run": "the configuration's whole run through the C ABI: sevc_create_from_arrays from host arrays, "
                       "%d steps (stop: 10,000 steps or 20%% of the grains left) by sevc_run (two steps in flight) "
                       "with every step's summary read back, sevc_get_state of the final mesh" % k,
                "steps": k, "wall_s": round(e_wall, 3), "device_vertex_steps_per_s": vs / (ms_full / 1e3),
                "gate_step": gate, "events": {"flips": int(ev_full[0]), "removals": int(ev_full[1]),
                                              "two_three": int(ev_full[2]), "nucleation_attempts": int(ev_full[3]),
                                              "nucleations": int(ev_full[4])}},
        "t0_window": {"value": t0_vs / (t0_ms / 1e3), "unit": UNIT, "ms_per_step": t0_ms / K,
                      "note": "steps %d..%d of the same run (before the gate: hardly any events)" % (W, W + K - 1)},
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak,
                     "traffic": NCU_TRAFFIC_PER_UNIT[dom] * units if dom in NCU_TRAFFIC_PER_UNIT else None,
                     "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum on the 200K-grain mesh, "
                                       "scaled by units per launch",
                     "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)",
                     "step_frac": step_bytes / (ms / K / 1e3) / 1e9 / peak,
                     "step_bytes": step_bytes,
                     "fp64_pipe_active_ncu": NCU_FP64_ACTIVE.get(dom),
                     "note": "FP64-issue bound on GB300 (DRAM idle); step_frac is the whole step's compulsory "
                             "bytes (131.5 per vertex) over its time"},
        "roofline_fp64": {"bound": "fp64", "unit": "FP64 thread-instructions/s", "peak": fp64_peak,
                          "peak_source": "sevc_measure_fp64_rate (independent DFMA chains, this GPU, now)",
                          "kernels": fp64,
                          "inst_per_unit_source": "ncu DADD+DMUL+DFMA thread instructions per grain / vertex "
                                                  "on the 200K-grain mesh"},
        "kernel_ms_share": {kk: round(v[0] / tot, 4) for kk, v in sorted(prof.items(), key=lambda kv: -kv[1][0])},
        "gpu_launches": sum(i.kernel_launches for i in infos),
        "kernel_ms_per_step": {kk: round(v[0] / v[1] if v[1] else 0, 4) for kk, v in prof.items()},
        "clocks": ck,
    }
    if args.cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(win_state[0], n, args.cpu_steps, win_state[1], opt)
    import shutil
    shutil.rmtree(tmpdir, ignore_errors=True)
    if args.ensemble_sample > 0:
        line["ensemble"] = run_ensemble(args.ensemble_sample, args.ensemble_grains[0], args.ensemble_grains[1],
                                        10, 3, cache=args.ensemble_cache)
    if args.adjoint_sample:
        line["adjoint"] = run_adjoint()
        line["calibration"] = run_calibration(n_inst=64, lo=20000, hi=20000, steps=40, iters=50, dt=1e-4,
                                              nucleation=(5, 3.0))
    print(json.dumps(line))


def cpu_baseline(state, n, steps, step_index, eopt):
    """The oracle (the reference's step logic restated in C, OpenMP) on the
    same window: built from the engine's state at the window's start."""
    from oracle import oracle as O
    O.build()
    opt = workload_options(O, n, steps)
    O.finish_options(opt)
    opt.min_grains = -1
    orc = O.Oracle.from_state(opt, state, n=step_index, allow_nucleation=1)
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
            "sample": "%d steps of the same window (the oracle built from the engine's state at its start, "
                      "OpenMP on every host core)" % steps}


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
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="engine", choices=["engine", "reference"])
    ap.add_argument("--grains", type=int, default=1000000)
    ap.add_argument("--seed", type=int, default=2024)
    ap.add_argument("--prof-steps", type=int, default=5)
    ap.add_argument("--cpu-steps", type=int, default=2)
    ap.add_argument("--mesh-cache", default=None, help="npz file to reuse the generated mesh")
    ap.add_argument("--no-cpu-baseline", dest="cpu_baseline", action="store_false")
    ap.add_argument("--launch", default="graph", choices=["graph", "hostloops", "direct"],
                    help="one graph per step (default), graphs with the loops on the host, or every kernel "
                         "launched directly (for profilers)")
    ap.add_argument("--cal-dt", type=float, default=1e-4, help="--workload calibrate: time step")
    ap.add_argument("--ckpt", default=None, help="--workload window: checkpoint file past the gate (made if absent)")
    ap.add_argument("--workload", default="single", choices=["single", "ensemble", "calibrate", "small", "window"],
                    help="ensemble: batched ensemble against sequential plain runs; calibrate: 64 x 20,000-grain "
                         "batched calibration with nucleation, 50 iterations of a --steps window past the "
                         "gate; each prints its own JSON line")
    ap.add_argument("--instances", type=int, default=512)
    ap.add_argument("--ensemble-grains", type=int, nargs=2, default=[500, 20000])
    ap.add_argument("--ensemble-sample", type=int, default=512,
                    help="instances of the ensemble measurement added to the single-run line (0: none)")
    ap.add_argument("--ensemble-cache", default=None, help="npz file to reuse the generated ensemble")
    ap.add_argument("--no-adjoint-sample", dest="adjoint_sample", action="store_false",
                    help="skip the forward/adjoint timing added to the single-run line")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
        return
    if int(os.environ.get("RANK", "0")) != 0 and args.gpus > 1:
        return
    import __graft_entry__
    __graft_entry__.build()
    if args.workload == "ensemble":
        r = run_ensemble(args.instances, args.ensemble_grains[0], args.ensemble_grains[1], args.steps, args.warmup,
                         cache=args.ensemble_cache)
        print(json.dumps({"metric": "ensemble speedup vs sequential plain runs", "value": r["speedup"],
                          "unit": "x", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
                          "ms_per_step": r["batch_ms_per_step"], "higher_is_better": True, "scaling": "weak",
                          "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded periodic Voronoi)",
                          "config": {"workload": "batched ensemble", **r}}))
        return
    if args.workload == "window":
        r = run_window(args)
        print(json.dumps({"metric": METRIC.replace("1M", "%d" % args.grains), "value": r["value"], "unit": UNIT,
                          "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": r["ms_per_step"],
                          "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                          "data": "synthetic (seeded periodic Voronoi, lognormal stored energy)",
                          "config": {"workload": "steps past the nucleation gate", **r}}))
        return
    if args.workload == "small":
        r = run_small(args.steps)
        print(json.dumps({"metric": "vertex-steps/s at 2K grains", "value": r["gpu_vertex_steps_per_s"],
                          "unit": UNIT, "n_gpus": 1, "steps": args.steps, "warmup": 0,
                          "ms_per_step": r["gpu_ms_per_step"], "higher_is_better": True, "scaling": "weak",
                          "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded periodic Voronoi)",
                          "config": {"workload": "2,000-grain plain run, SE U[0,0.5], dt 1e-6", **r}}))
        return
    if args.workload == "calibrate":
        r = run_calibration(n_inst=64, lo=20000, hi=20000, steps=args.steps, iters=50, dt=args.cal_dt,
                            nucleation=(5, 3.0))
        print(json.dumps({"metric": "backward/forward time ratio of batched calibration",
                          "value": r["backward_forward_ratio"], "unit": "x", "n_gpus": 1, "steps": args.steps,
                          "warmup": 0, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
                          "dtype": "f64", "data": "synthetic (seeded periodic Voronoi)",
                          "config": {"workload": "batched stored-energy calibration", **r}}))
        return
    run_engine(args)


if __name__ == "__main__":
    main()
