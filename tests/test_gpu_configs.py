"""The GPU engine on the benchmark specification's configurations, through
the C ABI, against the oracle at every step and against the reference's
own run.

Configurations (tests/golden/configs.py, LONG_CONFIGS):
  example_ref2k  the reference's shipped 2,000-grain input (voronoi/2K) with
                 its config/example.ini, to 100 grains: flips, removals,
                 2x3 pairs and conflicts all occur;
  c1_ref2k       2,000 grains, SE U[0, 0.5], dt = 1e-6, unit square, no
  c1_m2000       nucleation, until 50% of the grains are removed, on the
                 reference's input and on a voronoi.py mesh;
  events_m1000   dense events (tens of removals and flips per step).
and a nucleation-phase window of a 100,000-grain lognormal-SE mesh.

Every step: the step summary (grain count, flips, removals, 2x3 passes and
counts, conflicts, polling iterations, nucleation attempt and site) equals
the oracle's, and the state digests (sevc_state_digest, one per field,
computed on the device) equal the oracle's digests of its own state: every
position, velocity, connectivity entry, flag, list slot, area, arclength
and energy bit-identical.  Every FULL_EVERY steps and at the end the whole
state is downloaded and compared field by field (to locate a difference).
Against the reference's own sources run on the CPU (tests/golden/
golden.json): the grain count at every step, every nonzero 2x3 count and
the integer digest of every snapshot.

The oracle runs on the host while a second thread steps the engine (the C
calls release the interpreter lock), so a run takes about as long as the
slower of the two.
"""
import json
import os
import queue
import threading

import numpy as np
import pytest

import configs
import digest
import snapshot
from test_gpu_parity import compare

pytestmark = pytest.mark.gpu

GOLDEN = json.load(open(os.path.join(configs.HERE, "golden.json")))
FULL_EVERY = 2000


def step_summary_equal(info, s, where):
    assert info.curr_n_grains == s.curr_n_grains, where
    assert info.polling_iters == s.polling_iters, where
    assert list(info.two_three_counts)[:info.n_two_three_iters] == \
        [s.last_two_three[i] for i in range(s.n_two_three_iters)], where
    assert (info.n_flips, info.n_removals, info.n_two_three, info.n_nucleations, info.n_conflicts) == \
        (s.ev_flips, s.ev_removals, s.ev_two_three, s.ev_nucleations, s.ev_conflicts), where
    assert bool(info.nucleation_attempted) == (s.allow_nucleation and s.opt.do_nucleation and
                                               s.opt.nucleation_gap > 0 and s.n % s.opt.nucleation_gap == 0), where
    if info.nucleation_attempted:
        assert info.nucleation_candidate == s.vrt_id_candidate, where


def lockstep(eng, orc, where, max_steps=None, full_every=FULL_EVERY, on_step=None):
    """Step the engine (in a thread) and the oracle side by side until the
    run ends; compare summaries and digests every step and the full state
    every full_every steps.  Returns per-step records (info dicts)."""
    q = queue.Queue(maxsize=256)
    stop = threading.Event()

    def producer():
        k = 0
        try:
            while not stop.is_set():
                info = eng.step()
                dg = eng.state_digest()
                last = not info.keep_going or (max_steps is not None and k + 1 >= max_steps)
                st = eng.get_state() if (k % full_every == 0 or last) else None
                extra = on_step(eng, info) if on_step else None
                q.put((info, dg, st, extra))
                k += 1
                if last:
                    break
        except Exception as e:     # reported by the consumer
            q.put(e)
        q.put(None)

    t = threading.Thread(target=producer, daemon=True)
    t.start()
    recs, k = [], 0
    try:
        while True:
            item = q.get()
            if item is None:
                break
            if isinstance(item, Exception):
                raise item
            info, dg, st, extra = item
            assert orc.step() == 0, "%s: oracle status %d at step %d" % (where, orc.s.status, k)
            w = "%s step %d" % (where, info.n)
            step_summary_equal(info, orc.s, w)
            if st is not None:
                compare(st, orc, True, w, complete=bool(info.outputs_complete))
            od = orc.state_digest()
            if od != dg:
                bad = [f for f, a, b in zip(digest.FIELDS, dg, od) if a != b]
                compare(eng.get_state(), orc, True, w, complete=bool(info.outputs_complete))
                raise AssertionError("%s: state digests differ %s" % (w, bad))
            keep = orc.finish_step()
            assert bool(info.keep_going) == keep, w
            recs.append((info.as_dict(), extra))
            k += 1
    finally:
        stop.set()
        while t.is_alive():
            try:
                q.get(timeout=0.1)
            except queue.Empty:
                pass
        t.join()
    return recs


def make_pair(gpu, O, name, tmp, draws=0):
    _, _, keys, _, mg = configs.ALL_CONFIGS[name]
    ini = configs.write_ini(os.path.join(tmp, name + ".ini"), name, os.path.join(tmp, "out"))
    opt = gpu.load_ini(ini)
    opt.min_grains = mg
    oopt = O.parse_ini(ini)
    oopt.min_grains = mg
    eng = gpu.Engine.from_files(opt)
    orc = O.Oracle.from_files(oopt)
    orc.set_threads(os.cpu_count() or 1)
    if draws:
        orc.rng_table(gpu.rng_record(8192, draws))
    return eng, orc


@pytest.mark.parametrize("name", ["example_ref2k", "c1_ref2k", "c1_m2000", "events_m1000"])
def test_configuration_against_oracle_and_reference(gpu, oracle_mod, name, tmp_path):
    tmp = str(tmp_path)
    eng, orc = make_pair(gpu, oracle_mod, name, tmp)
    g = GOLDEN[name]

    def on_step(e, info):
        if info.export_due:
            path = os.path.join(tmp, "snap.txt")
            e.export(path, info.t)
            return snapshot.digests(path)[1]
        return None

    recs = lockstep(eng, orc, name, on_step=on_step)
    eng.close()
    infos = [r for r, _ in recs]
    exports = [x for _, x in recs if x is not None]
    # against the reference's own run (its first steps)
    ref = g["steps"]
    assert len(infos) >= len(ref)
    for mine, r in zip(infos, ref):
        assert mine["n"] == r["n"] and mine["curr_n_grains"] == r["n_grains"], (name, r["n"])
        assert mine["two_three_counts"] == r["two_three"], (name, r["n"])
    assert len(exports) >= len(g["snapshots"])
    for k, (topo, (_, gtopo)) in enumerate(zip(exports, g["snapshots"])):
        assert topo == gtopo, "%s snapshot %d: integer state differs from the reference's" % (name, k)
    ev = {k: sum(i[k] for i in infos) for k in ("n_flips", "n_removals", "n_two_three", "n_conflicts")}
    assert ev["n_flips"] > 0 and ev["n_removals"] > 0
    if name in ("example_ref2k", "events_m1000"):
        assert ev["n_two_three"] > 0 and ev["n_conflicts"] > 0, ev
    if name.startswith("c1"):
        assert infos[-1]["curr_n_grains"] <= 1000


def test_nucleation_phase_window_100k(gpu, oracle_mod):
    """A 100,000-grain mesh with lognormal(-1, 0.5) stored energy, grains one
    unit across, dt = 1e-3 and one Metropolis attempt every 10 steps once
    1/6 of the grains are gone (src/main.cu:137-141): engine and oracle step
    together from t = 0 through the 5/6 gate and 80 steps past it, with the
    oracle replaying the engine's cuRAND draws."""
    import meshgen
    n = 100000
    m = meshgen.make_inputs(n, 77, se="lognormal", se_params=(-1.0, 0.5))
    kw = dict(n_grains=n, dt=1e-3, dtau=1e-2, nucleation_gap=10, domain_bound=float(np.sqrt(n)), GB_eps=0.0,
              GB_scaling=1.0, SE_eps=1.0, SE_min=999.0, SE_max=999.0, do_nucleation=1, MC_k=1.0, nmax=10 ** 8,
              tmax=-1, snap_gap=10 ** 8, n_blocks=32, n_threads=256)
    opt = gpu.default_options(**kw)
    opt.min_grains = -1
    eng = gpu.Engine.from_arrays(opt, m["xy"], m["ridges"], m["oris"], m["se"])
    oopt = oracle_mod.finish_options(oracle_mod.default_options(**kw))
    oopt.min_grains = -1
    orc = oracle_mod.Oracle.from_arrays(oopt, m["xy"], m["ridges"], m["oris"], m["se"])
    orc.set_threads(os.cpu_count() or 1)
    # draws per stream per attempt: two per enabled vertex of the stream's
    # stride set (at most 25 here) plus the picks
    orc.rng_table(gpu.rng_record(8192, 600))
    recs = []
    budget = 5000
    while True:
        chunk = lockstep(eng, orc, "nucl100k", max_steps=100, full_every=10 ** 9)
        recs += chunk
        gate = next((i for i, (r, _) in enumerate(recs) if r["curr_n_grains"] <= 5 * n // 6), None)
        if gate is not None and len(recs) >= gate + 81:
            break
        assert len(recs) < budget, "the 5/6 gate was not reached in %d steps" % budget
    eng.close()
    infos = [r for r, _ in recs]
    att = sum(i["nucleation_attempted"] for i in infos)
    assert att >= 7, att
    assert sum(i["n_removals"] for i in infos) > 1000


def test_state_digest_matches_its_definition(gpu, oracle_mod, tmp_path):
    """sevc_state_digest against the numpy restatement of its definition
    (tests/digest.py) applied to the downloaded state, before and after
    steps with events; and the oracle's C digest against the same
    restatement of the oracle's own arrays."""
    eng, orc = make_pair(gpu, oracle_mod, "events_m1000", str(tmp_path))
    for k in range(40):
        if k in (0, 1, 39):
            st = eng.get_state()
            assert eng.state_digest() == digest.digest(st.__getitem__), k
            assert orc.state_digest() == digest.digest(orc.field), k
        eng.step()
        orc.step()
        orc.finish_step()
    eng.close()


@pytest.mark.parametrize("grid", [(32, 256), (1, 1)])
def test_whole_step_graph_equals_host_loops(gpu, tmp_path, grid):
    """A step replayed as one CUDA graph, whose polling and 2x3 loops are
    conditional nodes the device drives, equals the step launched kernel by
    kernel with the loops on the host, and the step's fixed sequences as
    graphs with the loops on the host: every summary field and every state
    digest, through 2x3 pairs, conflicts and (on a 1 x 1 grid, where the
    convergence predicate covers every boundary) multi-iteration polling."""
    ini = configs.write_ini(os.path.join(str(tmp_path), "e.ini"), "events_m1000", os.path.join(str(tmp_path), "o"))
    engines = []
    for on in (1, 0, 2):
        o = gpu.load_ini(ini)
        o.min_grains = 10
        o.n_blocks, o.n_threads = grid
        e = gpu.Engine.from_files(o)
        e.set_graphs(on)
        engines.append(e)
    seen = {"tt": 0, "poll2": 0, "conf": 0}
    for k in range(300):
        a, b, c = (e.step() for e in engines)
        da, db, dc = a.as_dict(), b.as_dict(), c.as_dict()
        for key in ("gpu_ms", "kernel_launches"):
            for d in (da, db, dc):
                d.pop(key)
        assert da == db == dc, (k, da, db, dc)
        assert engines[0].state_digest() == engines[1].state_digest() == engines[2].state_digest(), k
        seen["tt"] += a.n_two_three
        seen["poll2"] += a.polling_iters >= 2
        seen["conf"] += a.n_conflicts
        if not a.keep_going:
            break
    assert seen["tt"] > 0 and seen["conf"] > 0, seen
    if grid == (1, 1):
        assert seen["poll2"] > 0, seen
    for e in engines:
        e.close()


def _nucleating_engines(gpu, count, batch):
    """`count` engines over the 300-grain fixture with its triangular
    stored energies (grains one unit across, one Metropolis attempt every 3
    steps past the 5/6 gate, no grain-count stop); batch: three copies of it
    as one batched handle"""
    import meshgen
    d = os.path.join(configs.MESH_DIR, "m300")
    mesh = meshgen.read_files(*[os.path.join(d, f) for f in ("vertices.txt", "ridges.txt", "oris.txt",
                                                              "se_triangular.txt")])
    dt = 4e-3
    o = gpu.default_options(n_grains=300, dt=dt, dtau=3 * dt, domain_bound=17.0, GB_eps=0.0, GB_scaling=1.0,
                            SE_eps=1.0, SE_min=999.0, SE_max=999.0, do_nucleation=1, MC_k=3.0, nmax=10 ** 8,
                            tmax=-1, snap_gap=10 ** 8, n_blocks=32, n_threads=256)
    o.min_grains = -1
    if batch:   # meshes of different sizes pass their gates at different steps
        meshes = [mesh] + [meshgen.make_inputs(n, 60 + n, se="triangular", generator="c") for n in (260, 330)]
        return [gpu.Engine.from_batch(o, meshes) for _ in range(count)]
    return [gpu.Engine.from_arrays(o, mesh["xy"], mesh["ridges"], mesh["oris"], mesh["se"]) for _ in range(count)]


@pytest.mark.parametrize("batch", [False, True])
def test_pipelined_run_equals_single_steps(gpu, batch):
    """sevc_run launches each step while the one before it runs and reads
    the summaries back afterwards; through the 5/6 gate (where an attempt
    step must wait for the count of the step before it) and the attempts
    after it, every step's summary equals the one sevc_step gives (timing
    aside) and so does the state digest at the end."""
    a, b = _nucleating_engines(gpu, 2, batch)
    ref, gate = [], None
    while gate is None or len(ref) < gate + 60:
        ref.append(b.step().as_dict())
        if gate is None and ref[-1]["nucleation_attempted"]:
            gate = len(ref)
        assert len(ref) < 5000, "the gate was not reached"
    got = []
    while len(got) < len(ref):
        got += [i.as_dict() for i in a.run(min(37, len(ref) - len(got)))]
    for k, (x, y) in enumerate(zip(got, ref)):
        for key in ("gpu_ms", "kernel_launches"):
            x.pop(key)
            y.pop(key)
        assert x == y, (k, x, y)
    assert sum(r["nucleation_attempted"] for r in ref) >= 10
    assert a.state_digest() == b.state_digest()
    a.close()
    b.close()
