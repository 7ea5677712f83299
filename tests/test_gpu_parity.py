"""GPU engine (through the C ABI) against the oracle and the reference.

Parity bar:
  * integer state (enabled flags, connectivity, candidate flags, grain lists,
    types) and every event count: bit-exact after every step;
  * positions, velocities, energies, areas, dA/dt, arclengths: bit-exact
    whenever no transcendental function feeds them (isotropic boundaries,
    GB_eps = 0); with anisotropic boundaries the boundary energy carries
    libm's last-bit differences, so these fields must agree to
    REL_TOL = 1e-12 relative per step (both sides restart every step from
    the GPU's floating-point state);
  * extinction times come from atan2/cos/sin (CUDA vs glibc): REL_TOL.
Nucleation draws: the oracle replays the exact cuRAND XORWOW draws that
the GPU consumes, recorded through sevc_rng_record.
"""
import json
import os

import numpy as np
import pytest

import configs
import snapshot

pytestmark = pytest.mark.gpu

REL_TOL = 1e-12
GOLDEN = json.load(open(os.path.join(configs.HERE, "golden.json")))

INT_FIELDS = ["ven", "vb", "vg", "bini", "bend", "ben", "bcand", "glist", "gvlen", "gen", "gtype"]
FLOAT_FIELDS = ["px", "py", "vx", "vy", "venergy", "vel_bnd_x", "vel_grn_x", "vel_bnd_y", "vel_grn_y", "blen",
                "benergy", "garea", "gori", "gse"]
RESYNC = ["px", "py", "vx", "vy", "venergy", "vel_bnd_x", "vel_grn_x", "vel_bnd_y", "vel_grn_y", "blen", "benergy",
          "btext", "garea", "gdadt", "gori"]


def close(a, b, rel):
    d = np.abs(a - b)
    scale = np.maximum(np.abs(a), np.abs(b))
    return np.all((d <= rel * scale) | (a == b))


def compare(st, orc, exact_float, where, complete=True):
    """complete: the step computed every output-only value (t_ext of every
    enabled boundary, dA/dt of every enabled grain); otherwise those are
    compared where the engine must have them: t_ext of candidates and of
    disabled boundaries, dA/dt of disabled grains."""
    for f in INT_FIELDS:
        a, b = st[f], orc.field(f)
        if not np.array_equal(a, b):
            i = int(np.nonzero(a != b)[0][0])
            raise AssertionError("%s: %s differs at %d: gpu %s oracle %s" % (where, f, i, a[i], b[i]))
    for f in FLOAT_FIELDS:
        a, b = st[f], orc.field(f)
        ok = np.array_equal(a, b) if exact_float else close(a, b, REL_TOL)
        if not ok:
            i = int(np.argmax(np.abs(a - b)))
            raise AssertionError("%s: %s differs at %d: gpu %r oracle %r" % (where, f, i, a[i], b[i]))
    a, b = st["gdadt"], orc.field("gdadt")
    sel = np.ones(len(a), bool) if complete else st["gen"] == 0
    ok = np.array_equal(a[sel], b[sel]) if exact_float else close(a[sel], b[sel], REL_TOL)
    assert ok, "%s: dA/dt differs" % where
    sel = np.ones(len(st["btext"]), bool) if complete else (st["bcand"] > 0) | (st["ben"] == 0)
    check_text(st["btext"], orc.field("btext"), st["ben"], where, sel)


def check_text(a, b, en, where, sel=None):
    """t_ext = -|d| / (T.P): libm's error in the unit tangent T enters the
    denominator linearly, so 1/t_ext is compared, against REL_TOL times the
    99th percentile of |1/t_ext| over enabled boundaries (a denominator that
    cancels makes the relative error of t_ext itself unbounded)."""
    ra, rb = 1.0 / a, 1.0 / b
    q = np.quantile(np.abs(ra[en > 0]), 0.99)
    bad = ~((a == b) | (np.abs(ra - rb) <= REL_TOL * (q + np.maximum(np.abs(ra), np.abs(rb)))))
    if sel is not None:
        bad &= sel
    if bad.any():
        i = int(np.nonzero(bad)[0][0])
        raise AssertionError("%s: t_ext differs at %d: gpu %r oracle %r (1/t scale %g)" % (where, i, a[i], b[i], q))


def make_pair(gpu, O, name, tmp, nucleation_draws=0):
    _, _, keys, seed, mg = configs.CONFIGS[name]
    ini = configs.write_ini(os.path.join(tmp, "run.ini"), name, os.path.join(tmp, "out"))
    opt = gpu.load_ini(ini)
    opt.min_grains = mg
    oopt = O.parse_ini(ini)
    oopt.min_grains = mg
    eng = gpu.Engine.from_files(opt)
    orc = O.Oracle.from_files(oopt)
    if nucleation_draws:
        orc.rng_table(gpu.rng_record(8192, nucleation_draws))
    return eng, orc, keys


def run_pair(gpu, O, name, tmp, steps=None, draws=0):
    eng, orc, keys = make_pair(gpu, O, name, tmp, draws)
    exact = float(keys["GB_eps"]) == 0.0
    k, events = 0, {"flips": 0, "removals": 0, "two_three": 0, "nucleations": 0}
    while orc.should_continue() and (steps is None or k < steps):
        info = eng.step()
        assert orc.step() == 0, "oracle status %d" % orc.s.status
        where = "%s step %d" % (name, info.n)
        compare(eng.get_state(), orc, exact, where, complete=bool(info.outputs_complete))
        s = orc.s
        assert info.curr_n_grains == s.curr_n_grains, where
        assert info.nucleated_area == s.nucleated_area or not exact, where
        assert info.polling_iters == s.polling_iters, where
        assert list(info.two_three_counts)[:info.n_two_three_iters] == \
            [s.last_two_three[i] for i in range(s.n_two_three_iters)], where
        assert (info.n_flips, info.n_removals, info.n_two_three, info.n_nucleations) == \
            (s.ev_flips, s.ev_removals, s.ev_two_three, s.ev_nucleations), where
        if info.nucleation_attempted:
            assert info.nucleation_candidate == s.vrt_id_candidate, where
        events["flips"] += info.n_flips
        events["removals"] += info.n_removals
        events["two_three"] += info.n_two_three
        events["nucleations"] += info.n_nucleations
        if not exact:
            st = eng.get_state()
            for f in RESYNC:
                orc.field(f)[:] = st[f]
        keep = orc.finish_step()
        assert bool(info.keep_going) == keep, where
        k += 1
        if not keep:
            break
    return events, k


def test_plain_unit_bit_exact_every_step(gpu, oracle_mod, tmp_path):
    ev, k = run_pair(gpu, oracle_mod, "plain_unit", str(tmp_path))
    assert k == 301 and ev["removals"] > 0 and ev["flips"] > 0


def test_nucleation_bit_exact_every_step(gpu, oracle_mod, tmp_path):
    ev, k = run_pair(gpu, oracle_mod, "perstep_nucl", str(tmp_path), draws=6 * 302 + 16)
    assert k == 301 and ev["nucleations"] > 0 and ev["removals"] > 0


def test_anisotropic_per_step_tolerance(gpu, oracle_mod, tmp_path):
    ev, k = run_pair(gpu, oracle_mod, "nucl_aniso", str(tmp_path), draws=6 * 82 + 16)
    assert k == 401 and ev["removals"] > 0


def test_gpu_matches_reference_snapshots(gpu, tmp_path):
    """GPU exports against the digests of the reference's own snapshots, for
    every snapshot before the first nucleation attempt (after it the random
    streams differ: the fixtures used the synthetic stream)."""
    for name in ("plain_unit", "nucl_aniso"):
        _, _, keys, _, mg = configs.CONFIGS[name]
        ini = configs.write_ini(os.path.join(str(tmp_path), name + ".ini"), name, "/tmp/unused")
        opt = gpu.load_ini(ini)
        opt.min_grains = mg
        eng = gpu.Engine.from_files(opt)
        g = GOLDEN[name]
        prog, checked = 0, 0
        for ref in g["steps"]:
            info = eng.step()
            if info.nucleation_attempted:
                break
            assert info.curr_n_grains == ref["n_grains"], (name, ref["n"])
            assert list(info.two_three_counts)[:info.n_two_three_iters] == ref["two_three"], (name, ref["n"])
            if float(keys["GB_eps"]) == 0.0:
                assert "%.16f" % info.nucleated_area == ref["nucl_area"]
            if info.export_due:
                path = os.path.join(str(tmp_path), "%s_%06d.txt" % (name, prog))
                eng.export(path, info.t)
                full, topo = snapshot.digests(path)
                assert topo == g["snapshots"][prog][1], (name, prog)
                prog += 1
                checked += 1
            if not info.keep_going:
                break
        assert checked >= 5, name
        eng.close()


@pytest.mark.parametrize("name,dt", [("plain_unit", None), ("nucl_aniso", None), ("plain_unit", 1e-3),
                                     ("nucl_aniso", 2e-2)])
def test_skipped_outputs_change_nothing_else(gpu, name, dt, tmp_path):
    """Steps that skip t_ext of provable non-candidates and dA/dt of grains
    that cannot vanish must leave every other value bit-identical to steps
    that compute everything, and must be complete whenever they can export.
    The runs at ten times the usual dt put many boundaries near the
    candidate threshold t_ext = dt, where the binary32 certificate has to
    hand over to the exact computation."""
    _, _, _, _, mg = configs.CONFIGS[name]
    ini = configs.write_ini(os.path.join(str(tmp_path), "r.ini"), name, "/tmp/unused")
    opt = gpu.load_ini(ini)
    opt.min_grains = mg
    if dt is not None:
        opt.dt = dt
    a, b = gpu.Engine.from_files(opt), gpu.Engine.from_files(opt)
    b.set_exact_all(True)
    skipped = 0
    while True:
        ia, ib = a.step(), b.step()
        assert ib.outputs_complete
        if ia.export_due:
            assert ia.outputs_complete
        sa, sb = a.get_state(), b.get_state()
        for f in INT_FIELDS + FLOAT_FIELDS:
            assert np.array_equal(sa[f], sb[f]), (name, ia.n, f)
        if ia.outputs_complete:
            assert np.array_equal(sa["btext"], sb["btext"]) and np.array_equal(sa["gdadt"], sb["gdadt"])
        else:
            skipped += 1
            c = (sa["bcand"] > 0) | (sa["ben"] == 0)
            assert np.array_equal(sa["btext"][c], sb["btext"][c])
            g = sa["gen"] == 0                       # dA/dt of every grain ever disabled
            assert np.array_equal(sa["gdadt"][g], sb["gdadt"][g]), (name, ia.n)
        if not ia.keep_going:
            break
    assert skipped > 0


def test_rng_record_is_curand_stream(gpu):
    a = gpu.rng_record(8192, 8)
    b = gpu.rng_record(16, 4)
    assert np.array_equal(a[:16, :4], b)
    assert a.min() > 0 and a.max() <= 1
    assert len(np.unique(a[:, 0])) == 8192


@pytest.mark.parametrize("n,steps", [(20000, 30)])
def test_meshgen_mesh_bit_exact(gpu, oracle_mod, n, steps):
    import meshgen
    inp = meshgen.make_inputs(n, 21)
    kw = dict(n_grains=n, dt=2e-5, dtau=2e-5, domain_bound=1.0, GB_eps=0.0, SE_min=0.0, SE_max=0.5, do_nucleation=0,
              nmax=steps, min_grains=10, snap_gap=1000)
    eng = gpu.Engine.from_arrays(gpu.default_options(**kw), inp["xy"], inp["ridges"], inp["oris"], inp["se"])
    oopt = oracle_mod.finish_options(oracle_mod.default_options(**kw))
    orc = oracle_mod.Oracle.from_arrays(oopt, inp["xy"], inp["ridges"], inp["oris"], inp["se"])
    orc.set_threads(os.cpu_count() or 1)
    for k in range(steps):
        info = eng.step()
        assert orc.step() == 0
        compare(eng.get_state(), orc, True, "meshgen step %d" % k, complete=bool(info.outputs_complete))
        assert info.n_removals == orc.s.ev_removals and info.n_flips == orc.s.ev_flips
        orc.finish_step()


def test_anisotropic_free_run_agrees_statistically(gpu, oracle_mod, tmp_path):
    """Third tier: with GB_eps != 0 the GPU's and the oracle's libm differ in
    the last bits, so free-running trajectories eventually take different
    events.  Without resynchronising, the grain-count curve and the final
    grain-area distribution must still agree statistically."""
    from scipy import stats
    eng, orc, keys = make_pair(gpu, oracle_mod, "nucl_aniso", str(tmp_path), nucleation_draws=6 * 402 + 16)
    counts_g, counts_o, first_diff = [], [], None
    for k in range(400):
        info = eng.step()
        assert orc.step() == 0
        orc.finish_step()
        counts_g.append(info.curr_n_grains)
        counts_o.append(orc.s.curr_n_grains)
        if first_diff is None and counts_g[-1] != counts_o[-1]:
            first_diff = k
    cg, co = np.array(counts_g), np.array(counts_o)
    assert np.all(np.abs(cg - co) <= np.maximum(5, 0.03 * co)), (first_diff, cg[-1], co[-1])
    st = eng.get_state()
    ag = np.abs(st["garea"][st["gen"] > 0])
    ao = np.abs(orc.field("garea")[orc.field("gen") > 0])
    ks = stats.ks_2samp(ag / ag.mean(), ao / ao.mean())
    assert ks.statistic < 0.1, ks
    assert abs(ag.std() / ag.mean() - ao.std() / ao.mean()) < 0.05 * (ao.std() / ao.mean())


def test_program_loop_snapshots_match_reference(gpu, tmp_path):
    """The drop-in program loop (sevc_run_program: snapshots written by a
    host thread while the next steps run) writes the files the reference
    writes: every snapshot before the first nucleation attempt has the
    digest of the reference's own, and the files are the ones the step-by-
    step API exports."""
    name = "plain_unit"
    _, _, keys, _, mg = configs.CONFIGS[name]
    out = os.path.join(str(tmp_path), "prog")
    ini = configs.write_ini(os.path.join(str(tmp_path), name + ".ini"), name, out)
    opt = gpu.load_ini(ini)
    opt.min_grains = mg
    rc = gpu.lib().sevc_run_program(gpu.C.byref(opt), 0)
    assert rc == 0, gpu.lib().sevc_last_error()
    files = sorted(f for f in os.listdir(os.path.join(out, "DATA")) if f.endswith(".txt"))
    g = GOLDEN[name]
    assert len(files) >= 5
    for prog, f in enumerate(files[:len(g["snapshots"])]):
        full, topo = snapshot.digests(os.path.join(out, "DATA", f))
        assert topo == g["snapshots"][prog][1], (f, prog)
    eng = gpu.Engine.from_files(opt)
    prog = 0
    while prog < 3:
        info = eng.step()
        if info.export_due:
            path = os.path.join(str(tmp_path), "api_%06d.txt" % prog)
            eng.export(path, info.t)
            assert open(path, "rb").read() == open(os.path.join(out, "DATA", files[prog]), "rb").read()
            prog += 1
    eng.close()


@pytest.mark.parametrize("name", ["plain_unit", "example_ref2k"])
def test_cli_log_lines_match_reference(gpu, name, tmp_path):
    """The drop-in executable prints the reference's per-step log lines
    (src/main.cu:122, 231, 324-325): `sevc -c run.ini` parsed as the
    reference's own log is parsed for the golden record (make_golden.
    parse_log) gives the same numbers at every step; its snapshots have the
    reference's integer digests."""
    import subprocess
    import make_golden
    _, _, keys, _, mg = configs.ALL_CONFIGS[name]
    out = os.path.join(str(tmp_path), "out")
    ini = configs.write_ini(os.path.join(str(tmp_path), "run.ini"), name, out, nmax=configs.golden_nmax(name))
    if "leave_percent" not in keys:
        with open(ini, "a") as f:
            f.write("[Temporal]\nleave_percent=%r\n" % (mg / int(keys["n_grains"])))
    exe = os.path.join(os.path.dirname(gpu.LIB_PATH), "sevc")
    r = subprocess.run([exe, "-c", ini, "--honor-leave-percent"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    mine, ref = make_golden.parse_log(r.stdout), GOLDEN[name]["steps"]
    assert len(mine) == len(ref)
    for a, b in zip(mine, ref):
        assert a == b, (a, b)
    files = sorted(os.listdir(os.path.join(out, "DATA")))
    assert len(files) == len(GOLDEN[name]["snapshots"])
    for f, (_, topo) in zip(files, GOLDEN[name]["snapshots"]):
        assert snapshot.digests(os.path.join(out, "DATA", f))[1] == topo, f
