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


def test_nucleation_map_restates_the_triangle_construction():
    """adjoint_ref.nucleation_map places the new corners where
    generate_grain_for_nucleation (src/nucleation2.cu:116-212, the
    do_scale branch nucleate uses) puts them: for each far end X of A,
    w = 0.99 r / |X - A| and the corner is dom_mod(A + w (X - A)), with
    r = 0.8 U min|X - A| + 0.1 over A's three boundaries; and its torch
    gradient agrees with central differences of itself."""
    from oracle import adjoint_ref
    rng = np.random.default_rng(7)
    D = 3.0
    for trial in range(20):
        x = rng.uniform(0, D, (8, 2))
        A, far = 0, [1, 2, 3]
        x[far] = (x[A] + rng.normal(0, 0.3, (3, 2))) % D        # near A, possibly across the wrap
        wrap = lambda d: d - D * np.round(d / D)
        L = [np.hypot(*wrap(x[X] - x[A])) for X in far]
        imin = int(np.argmin(L))
        U = rng.uniform()
        r = 0.8 * L[imin] * U + 0.1
        rec = {"A": A, "B": 4, "C": 5, "far": far, "xstar": far[imin], "k": 0.8 * U}
        y = adjoint_ref.nucleation_map(torch.tensor(x), rec, D).numpy()
        for X, Y in zip(far, (A, 4, 5)):
            t = wrap(x[X] - x[A])
            w = r / np.hypot(*t) * 0.99
            want = (w * t + x[A]) % D
            assert np.allclose(y[Y], want, rtol=1e-13, atol=1e-13), (trial, X, y[Y], want)
        assert np.array_equal(y[[1, 2, 3, 6, 7]], x[[1, 2, 3, 6, 7]])
    xt = torch.tensor(x, requires_grad=True)
    wts = torch.tensor(rng.standard_normal((8, 2)))
    f = lambda z: (adjoint_ref.nucleation_map(z, rec, D) * wts).sum()
    f(xt).backward()
    g = xt.grad.numpy()
    h = 1e-6
    for i in (0, 1, 2, 3):
        for c in (0, 1):
            e = np.zeros((8, 2))
            e[i, c] = h
            fd = (f(torch.tensor(x + e)) - f(torch.tensor(x - e))).item() / (2 * h)
            assert abs(fd - g[i, c]) <= 1e-6 * max(1.0, abs(fd)), (i, c, fd, g[i, c])
