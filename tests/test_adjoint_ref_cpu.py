"""The FP64 torch restatement used to check the adjoint (oracle/adjoint_ref.py)
agrees with central differences of itself, on the host."""
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")


def state_of(sevc, meshgen, n, seed, tmp):
    mesh = meshgen.make_inputs(n, seed)
    p = meshgen.write_files(str(tmp), mesh)
    o = sevc.default_options(n_grains=n, dt=1e-5, domain_bound=1.0, GB_eps=0.0, GB_scaling=1.0, SE_eps=1.0,
                             SE_min=999.0, SE_max=999.0, do_nucleation=0,
                             vertex_fname=p["vertices"], boundary_fname=p["ridges"], orientation_fname=p["oris"],
                             SE_fname=p["se"])
    return sevc.load_mesh_host(o)


def test_reference_gradient_matches_its_central_differences(engine_mod, tmp_path):
    import meshgen
    from oracle import adjoint_ref
    st = state_of(engine_mod, meshgen, 60, 5, tmp_path)
    se = np.random.default_rng(0).uniform(0, 0.5, 60)
    dt, steps, D, nb, amax = 2e-5, 6, 1.0, 20, 3.0
    target = np.full(nb, 1.0 / nb)
    loss, gse, ggam, gmu, h = adjoint_ref.loss_and_grads(st, se, 1.0, 1.0, dt, steps, D, nb, amax, target)
    assert abs(h.sum() - 1.0) < 0.1

    def L(se_, g_, m_):
        return adjoint_ref.loss_and_grads(st, se_, g_, m_, dt, steps, D, nb, amax, target)[0]

    hs = 1e-4
    fd_mu = (L(se, 1.0, 1.0 + hs) - L(se, 1.0, 1.0 - hs)) / (2 * hs)
    fd_g = (L(se, 1.0 + hs, 1.0) - L(se, 1.0 - hs, 1.0)) / (2 * hs)
    d = np.random.default_rng(1).standard_normal(60)
    fd_se = (L(se + hs * d, 1.0, 1.0) - L(se - hs * d, 1.0, 1.0)) / (2 * hs)
    assert abs(gmu - fd_mu) <= 1e-4 * abs(fd_mu)
    assert abs(ggam - fd_g) <= 1e-4 * abs(fd_g)
    assert abs(gse @ d - fd_se) <= 1e-4 * abs(fd_se)
