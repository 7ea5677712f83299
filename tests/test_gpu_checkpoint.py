"""Checkpoint files resume a run bit for bit (random streams, polling
buffers and run counters included); grain statistics agree with the mesh
invariants."""
import numpy as np
import pytest

from test_gpu_parity import FLOAT_FIELDS, INT_FIELDS

pytestmark = pytest.mark.gpu


def nucl_options(sevc, n):
    o = sevc.default_options(n_grains=n, dt=4e-3, dtau=4e-3, nucleation_gap=1, domain_bound=22.0, GB_eps=0.0,
                             GB_scaling=1.0, SE_eps=1.0, SE_min=999.0, SE_max=999.0, do_nucleation=1, MC_k=3.0,
                             nmax=10 ** 8, tmax=-1, snap_gap=10 ** 8, n_blocks=32, n_threads=256)
    o.min_grains = -1
    return o


def same_state(a, b):
    for f in INT_FIELDS + FLOAT_FIELDS:
        x, y = a[f], b[f]
        if x.dtype.kind == "f":
            if not np.array_equal(x.view(np.int64), y.view(np.int64)):
                return f
        elif not np.array_equal(x, y):
            return f
    return None


def test_checkpoint_resumes_bit_exact(gpu, tmp_path):
    """The 300-grain fixture with nucleation at every step once a sixth of
    the grains are gone (from about step 200): save at step 190, resume in
    a second handle, compare the next 90 steps."""
    import configs
    ini = configs.write_ini(str(tmp_path / "run.ini"), "perstep_nucl", str(tmp_path / "out"))
    def mk():
        o = gpu.load_ini(ini)
        o.min_grains = -1
        return gpu.Engine.from_files(o)
    a = mk()
    for _ in range(190):
        a.step()
    path = str(tmp_path / "run.ckpt")
    a.checkpoint_save(path)
    ia = [a.step() for _ in range(90)]
    b = mk()
    b.step()
    b.checkpoint_load(path)
    ib = [b.step() for _ in range(90)]
    assert [(i.n, i.curr_n_grains, i.n_flips, i.n_removals, i.n_nucleations, i.nucleation_candidate) for i in ia] == \
           [(i.n, i.curr_n_grains, i.n_flips, i.n_removals, i.n_nucleations, i.nucleation_candidate) for i in ib]
    assert sum(i.n_nucleations for i in ia) > 0
    assert same_state(a.get_state(), b.get_state()) is None
    import meshgen
    other = gpu.Engine.from_arrays(nucl_options(gpu, 250), *[meshgen.make_inputs(250, 1)[k]
                                                            for k in ("xy", "ridges", "oris", "se")])
    with pytest.raises(gpu.SevcError):
        other.checkpoint_load(path)
    for e in (a, b, other):
        e.close()


def test_grain_stats_invariants(gpu):
    import meshgen
    meshes = [meshgen.make_inputs(n, s) for n, s in [(400, 1), (700, 2)]]
    o = nucl_options(gpu, 400)
    o.do_nucleation = 0
    e = gpu.Engine.from_batch(o, meshes)
    for _ in range(30):
        e.step()
    st = e.get_state()
    D = 22.0
    tot = 0
    for i in range(2):
        s = e.grain_stats(i)
        part = e.instance_state(st, i)
        n = int(part["gen"].sum())
        assert s["n_grains"] == n and s["n_grains"] == e.instance_info(i).curr_n_grains
        assert abs(s["mean_area"] * n - D * D) <= 1e-9 * D * D      # grains tile the domain
        assert s["mean_sides"] == 6.0                                # degree-3 periodic mesh
        assert s["n_three_sided"] == int(((part["gvlen"] == 3) & (part["gen"] == 1)).sum())
        assert 0 < s["min_area"] <= s["mean_area"] <= s["max_area"]
        tot += n
    assert e.grain_stats(-1)["n_grains"] == tot
    e.close()


def test_graph_replay_matches_direct_launches(gpu, tmp_path):
    """Steps replayed from CUDA graphs equal steps launched kernel by kernel,
    bit for bit, through removals, flips and nucleations."""
    import configs
    ini = configs.write_ini(str(tmp_path / "run.ini"), "perstep_nucl", str(tmp_path / "out"))
    engines = []
    for on in (True, False):
        o = gpu.load_ini(ini)
        o.min_grains = -1
        e = gpu.Engine.from_files(o)
        e.set_graphs(on)
        engines.append(e)
    nucl = 0
    for k in range(300):
        a, b = engines[0].step(), engines[1].step()
        assert (a.curr_n_grains, a.n_flips, a.n_removals, a.n_nucleations, a.polling_iters, a.outputs_complete) == \
               (b.curr_n_grains, b.n_flips, b.n_removals, b.n_nucleations, b.polling_iters, b.outputs_complete), k
        nucl += a.n_nucleations
        if k % 50 == 49:
            assert same_state(engines[0].get_state(), engines[1].get_state()) is None, k
    assert nucl > 0
    for e in engines:
        e.close()


def test_autotune_keeps_state_and_results(gpu):
    """The autotuner leaves the run where it was, and steps with the shapes
    it picks equal steps with the default shapes, bit for bit."""
    import meshgen
    mesh = meshgen.make_inputs(3000, 77, se="triangular")
    o = nucl_options(gpu, 3000)
    o.do_nucleation = 0
    o.domain_bound = 55.0
    a = gpu.Engine.from_arrays(o, mesh["xy"], mesh["ridges"], mesh["oris"], mesh["se"])
    b = gpu.Engine.from_arrays(o, mesh["xy"], mesh["ridges"], mesh["oris"], mesh["se"])
    for _ in range(20):
        a.step()
        b.step()
    chosen = a.autotune(steps=3)
    assert chosen[0] in (128, 256, 512) and chosen[1] in (128, 256, 512) and 9 <= chosen[2] <= 12
    assert chosen[3] in (4, 5, 6, 8)
    assert same_state(a.get_state(), b.get_state()) is None
    events = 0
    for k in range(60):
        ia, ib = a.step(), b.step()
        assert (ia.n, ia.curr_n_grains, ia.n_flips, ia.n_removals) == (ib.n, ib.curr_n_grains, ib.n_flips, ib.n_removals)
        events += ia.n_flips + ia.n_removals
    assert same_state(a.get_state(), b.get_state()) is None
    assert events > 0
    a.close()
    b.close()
