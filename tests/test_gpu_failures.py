"""Bounded failure paths of the step, produced from the host on small
meshes (nothing faults the GPU: every device loop and list is bounded and
reports through a status word that sevc_step turns into a status code).

  NONCONVERGED  the polling loop (src/topological.h:549-578, unbounded in
                the reference) hits its cap: a 1 x 1 launch grid makes the
                convergence predicate cover every boundary, so a step with
                candidates needs two iterations; with the cap at 1 it fails
                at the step where the oracle counts two;
  CAPACITY      a grain list would exceed 100 vertices (src/geometry.h:
                615-619 writes past the array): a Voronoi mesh with a
                100-sided grain, whose neighbours flip onto it; the engine
                reports it at the step where the oracle does;
  worklist      the grain-list fix-up work lists, capped at one entry.
After each, a new handle on the same device steps normally.
"""
import os

import numpy as np
import pytest

import configs
from test_gpu_configs import make_pair, step_summary_equal

pytestmark = pytest.mark.gpu

ST_CAPACITY, ST_NONCONVERGED = 3, 4


def still_usable(gpu, tmp):
    ini = configs.write_ini(os.path.join(tmp, "u.ini"), "plain_unit", os.path.join(tmp, "u"))
    opt = gpu.load_ini(ini)
    opt.min_grains = 10
    eng = gpu.Engine.from_files(opt)
    for _ in range(3):
        eng.step()
    eng.close()


def test_polling_cap_reports_nonconverged(gpu, oracle_mod, tmp_path):
    tmp = str(tmp_path)
    ini = configs.write_ini(os.path.join(tmp, "g1.ini"), "events_m1000", os.path.join(tmp, "o"))
    opt, oopt = gpu.load_ini(ini), oracle_mod.parse_ini(ini)
    for o in (opt, oopt):
        o.min_grains, o.n_blocks, o.n_threads = 10, 1, 1
    eng, orc = gpu.Engine.from_files(opt), oracle_mod.Oracle.from_files(oopt)
    eng.set_limits(polling_cap=1)
    for k in range(50):
        assert orc.step() == 0
        if orc.s.polling_iters >= 2:
            with pytest.raises(gpu.SevcError) as e:
                eng.step()
            assert e.value.code == ST_NONCONVERGED, e.value
            break
        info = eng.step()
        step_summary_equal(info, orc.s, "grid 1x1 step %d" % k)
        orc.finish_step()
    else:
        pytest.fail("no step needed two polling iterations")
    eng.close()
    # the same run with the default cap converges and matches the oracle
    eng, orc = gpu.Engine.from_files(opt), oracle_mod.Oracle.from_files(oopt)
    iters = []
    for k in range(20):
        info = eng.step()
        assert orc.step() == 0
        step_summary_equal(info, orc.s, "grid 1x1 step %d" % k)
        iters.append(info.polling_iters)
        orc.finish_step()
    assert max(iters) >= 2
    eng.close()
    still_usable(gpu, tmp)


def hundred_sided_mesh(seed=3):
    """Seeds: a centre, a ring of 100 around it (radius 0.08) and a second
    ring of 100 offset by half a step (radius 0.084), then uniform seeds
    outside radius 0.16.  The centre's Voronoi cell has 100 sides; the
    short edges between the rings flip onto it."""
    import meshgen
    rng = np.random.default_rng(seed)
    k = 100
    th = 2 * np.pi * np.arange(k) / k
    ring1 = 0.5 + 0.08 * np.stack([np.cos(th), np.sin(th)], 1)
    ring2 = 0.5 + 0.084 * np.stack([np.cos(th + np.pi / k), np.sin(th + np.pi / k)], 1)
    outer = rng.random((4000, 2))
    outer = outer[np.hypot(outer[:, 0] - 0.5, outer[:, 1] - 0.5) > 0.16][:300]
    pts = np.concatenate([[[0.5, 0.5]], ring1, ring2, outer])
    xy, ridges = meshgen.periodic_voronoi(len(pts), rng, points=pts)
    return xy, ridges, rng.random(len(pts)), rng.random(len(pts))


def test_capacity_error_when_a_list_exceeds_100(gpu, oracle_mod, tmp_path):
    xy, ridges, oris, se = hundred_sided_mesh()
    n = len(oris)
    kw = dict(n_grains=n, dt=1e-4, dtau=1.0, domain_bound=1.0, GB_eps=0.0, GB_scaling=1.0, SE_eps=1.0, SE_min=0.0,
              SE_max=0.5, do_nucleation=0, nmax=5000, tmax=-1, snap_gap=10 ** 8, n_blocks=32, n_threads=256)
    opt = gpu.default_options(**kw)
    opt.min_grains = 10
    oopt = oracle_mod.finish_options(oracle_mod.default_options(**kw))
    oopt.min_grains = 10
    eng = gpu.Engine.from_arrays(opt, xy, ridges, oris, se)
    orc = oracle_mod.Oracle.from_arrays(oopt, xy, ridges, oris, se)
    assert eng.get_state()["gvlen"].max() == 100
    for k in range(3000):
        rc = orc.step()
        if rc:
            assert rc == ST_CAPACITY, rc
            with pytest.raises(gpu.SevcError) as e:
                eng.step()
            assert e.value.code == ST_CAPACITY and "100" in str(e.value), e.value
            break
        info = eng.step()
        step_summary_equal(info, orc.s, "100-gon step %d" % k)
        orc.finish_step()
    else:
        pytest.fail("no list reached 101 vertices")
    eng.close()
    still_usable(gpu, str(tmp_path))


def test_worklist_cap_reports_capacity(gpu, oracle_mod, tmp_path):
    eng, orc = make_pair(gpu, oracle_mod, "events_m1000", str(tmp_path))
    eng.set_limits(worklist_cap=1)
    with pytest.raises(gpu.SevcError) as e:
        for _ in range(100):
            eng.step()
    assert e.value.code == ST_CAPACITY and "worklist" in str(e.value), e.value
    eng.close()
    with pytest.raises(gpu.SevcError):
        gpu.Engine.from_arrays(gpu.default_options(n_grains=3, dt=1e-4), np.zeros((4, 2)),
                               np.array([[0, 1], [1, 2], [2, 3], [3, 0]], np.int32), np.zeros(3), np.zeros(3))
    still_usable(gpu, str(tmp_path))
