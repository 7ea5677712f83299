"""Batched ensembles: every instance of a batched handle must follow, bit
for bit, the plain handle built from the same arrays (both computing every
output on every step), including the per-instance polling, 2x3 loop, event
order, nucleation draws and the per-instance step summaries."""
import numpy as np
import pytest

from test_gpu_parity import FLOAT_FIELDS, INT_FIELDS

pytestmark = pytest.mark.gpu


def options(sevc, **kw):
    base = dict(dt=4e-3, dtau=4e-3, nucleation_gap=1, domain_bound=17.0, GB_eps=0.0, GB_scaling=1.0, SE_eps=1.0,
                SE_min=999.0, SE_max=999.0, do_nucleation=1, MC_k=3.0, nmax=10 ** 8, tmax=-1, snap_gap=10 ** 8,
                min_grains=-1, n_blocks=32, n_threads=256)
    base.update(kw)
    return base


def make(sevc, kw, mesh):
    o = sevc.default_options(**dict(kw, n_grains=len(mesh["oris"])))
    o.min_grains = -1
    return o


def run_batch_vs_plain(sevc, meshgen, sizes, seeds, steps, kw, se="triangular", full_every=10):
    meshes = [meshgen.make_inputs(n, s, se=se) for n, s in zip(sizes, seeds)]
    o = make(sevc, kw, meshes[0])
    batch = sevc.Engine.from_batch(o, meshes)
    plains = []
    for m in meshes:
        e = sevc.Engine.from_arrays(make(sevc, kw, m), m["xy"], m["ridges"], m["oris"], m["se"])
        plains.append(e)
    assert batch.instance_count() == len(meshes)
    vo, bo, go = batch.instance_ranges()
    assert list(np.diff(go)) == sizes
    totals = {"flips": 0, "removals": 0, "two_three": 0, "nucleations": 0}
    for k in range(steps):
        binfo = batch.step()
        n_ev = 0
        for i, e in enumerate(plains):
            pi = e.step()
            bi = batch.instance_info(i)
            where = "step %d instance %d" % (k, i)
            assert (bi.n, bi.curr_n_grains, bi.polling_iters, bi.n_two_three_iters) == \
                (pi.n, pi.curr_n_grains, pi.polling_iters, pi.n_two_three_iters), where
            assert list(bi.two_three_counts)[:bi.n_two_three_iters] == \
                list(pi.two_three_counts)[:pi.n_two_three_iters], where
            assert (bi.n_flips, bi.n_removals, bi.n_two_three, bi.n_nucleations) == \
                (pi.n_flips, pi.n_removals, pi.n_two_three, pi.n_nucleations), where
            assert bi.nucleation_attempted == pi.nucleation_attempted, where
            assert bi.nucleation_candidate == pi.nucleation_candidate, where
            assert bi.nucleated_area == pi.nucleated_area, where
            assert bi.outputs_complete == pi.outputs_complete == binfo.outputs_complete, where
            totals["flips"] += pi.n_flips
            totals["removals"] += pi.n_removals
            totals["two_three"] += pi.n_two_three
            totals["nucleations"] += pi.n_nucleations
            n_ev += pi.n_flips + pi.n_removals
        assert binfo.n_flips + binfo.n_removals == n_ev
        if k % full_every == full_every - 1 or k == steps - 1:
            st = batch.get_state()
            for i, e in enumerate(plains):
                part, ref = batch.instance_state(st, i), e.get_state()
                for f in INT_FIELDS + FLOAT_FIELDS:
                    a, b = part[f], ref[f]
                    if a.dtype.kind == "f":
                        same = np.array_equal(a.view(np.int64), b.view(np.int64))
                    else:
                        same = np.array_equal(a, b)
                    assert same, "step %d instance %d field %s differs" % (k, i, f)
    for e in plains:
        e.close()
    batch.close()
    return totals


def test_batch_matches_plain_runs_with_nucleation(gpu):
    import meshgen
    # nucleation opens once a sixth of an instance's grains are gone
    ev = run_batch_vs_plain(gpu, meshgen, [300, 260, 340, 220, 310], [11, 12, 13, 14, 15], 340, options(gpu),
                            full_every=20)
    assert ev["nucleations"] > 0 and ev["removals"] > 0 and ev["flips"] > 0, ev


def test_batch_matches_plain_runs_anisotropic(gpu):
    import meshgen
    kw = options(gpu, dt=2e-3, dtau=1e-2, nucleation_gap=5, domain_bound=30.0, GB_eps=0.02, MC_k=1.0)
    ev = run_batch_vs_plain(gpu, meshgen, [700, 450, 900], [21, 22, 23], 120, kw)
    assert ev["removals"] > 0 and ev["flips"] > 0, ev


def test_batch_instance_export_matches_plain(gpu, tmp_path):
    import meshgen
    kw = options(gpu, do_nucleation=0)
    meshes = [meshgen.make_inputs(n, s, se="triangular") for n, s in [(200, 5), (350, 6)]]
    batch = gpu.Engine.from_batch(make(gpu, kw, meshes[0]), meshes)
    plain = gpu.Engine.from_arrays(make(gpu, kw, meshes[1]), meshes[1]["xy"], meshes[1]["ridges"],
                                   meshes[1]["oris"], meshes[1]["se"])
    for _ in range(19):
        batch.step()
        plain.step()
    a, b = str(tmp_path / "batch.txt"), str(tmp_path / "plain.txt")
    if not batch.step().outputs_complete:           # a step that skipped output-only values
        with pytest.raises(gpu.SevcError):
            batch.export_instance(1, a, 0.08)
    plain.step()
    for e in (batch, plain):
        e.set_exact_all(True)
        e.step()
    batch.export_instance(1, a, 0.084)
    plain.export(b, 0.084)
    assert open(a).read() == open(b).read()
    with pytest.raises(gpu.SevcError):
        batch.export_instance(2, a, 0.0)
