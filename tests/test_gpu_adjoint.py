"""Adjoint of the time step: gradients of the smoothed grain-area histogram
loss with respect to per-grain stored energies, GB_scaling and mobility.

Checked (1) against the FP64 torch restatement in oracle/adjoint_ref.py on
a window without topological events, where both differentiate the same
map (tolerance 1e-6 relative: both evaluate the finite-difference velocity,
whose derivative has cancellation of order 1e-8), and (2) against central
finite differences of the GPU forward itself through windows with flips
and removals, with the event sequence checked identical in the perturbed
runs."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NB, AMAX = 20, 3.0


def options(sevc, n, dt):
    o = sevc.default_options(n_grains=n, dt=dt, dtau=1.0, domain_bound=1.0, GB_eps=0.0, GB_scaling=1.0, SE_eps=1.0,
                             SE_min=999.0, SE_max=999.0, do_nucleation=0, nmax=10 ** 8, tmax=-1, snap_gap=10 ** 8,
                             n_blocks=32, n_threads=256)
    o.min_grains = -1
    return o


def make(sevc, mesh, dt):
    return sevc.Engine.from_arrays(options(sevc, len(mesh["oris"]), dt), mesh["xy"], mesh["ridges"], mesh["oris"],
                                   mesh["se"])


def forward(sevc, mesh, dt, steps, se, gam, mu, every=None):
    e = make(sevc, mesh, dt)
    e.set_stored_energy(se)
    e.set_gb_scaling(gam)
    e.set_mobility(mu)
    if every:
        e.tape_start(every)
    events = []
    for _ in range(steps):
        i = e.step()
        events.append((i.n_flips, i.n_removals, i.n_two_three))
    return e, e.area_histogram(NB, AMAX), events


def loss_of(h, target):
    return float(((h - target) ** 2).mean())


def dloss(h, target):
    return 2.0 * (h - target) / len(h)


def test_histogram_matches_reference(gpu):
    import meshgen
    from oracle import adjoint_ref
    import torch
    mesh = meshgen.make_inputs(300, 3)
    e = make(gpu, mesh, 1e-6)
    st = e.get_state()
    h = e.area_histogram(NB, AMAX)
    topo = adjoint_ref.Topology(st)
    x = torch.tensor(np.stack([st["px"], st["py"]], 1))
    ref = adjoint_ref.histogram(x, topo, 1.0, NB, AMAX).numpy()
    assert np.allclose(h, ref, rtol=1e-12, atol=1e-15)
    assert abs(h.sum() - 1.0) < 0.05


def test_adjoint_matches_fp64_reference_without_events(gpu):
    import meshgen
    from oracle import adjoint_ref
    mesh = meshgen.make_inputs(80, 5)
    se = np.random.default_rng(1).uniform(0.0, 0.5, 80)
    dt, steps = 2e-6, 40
    e, h, events = forward(gpu, mesh, dt, steps, se, 1.0, 1.0)
    assert all(ev == (0, 0, 0) for ev in events), "window must have no topological event"
    target = h * 0.9 + 0.1 / NB
    e.close()
    e0 = make(gpu, mesh, dt)
    e0.set_stored_energy(se)
    st0 = e0.get_state()
    e0.close()
    e, h, _ = forward(gpu, mesh, dt, steps, se, 1.0, 1.0, every=15)
    gse, ggam, gmu = e.adjoint_histogram(NB, AMAX, dloss(h, target))
    loss_r, gse_r, ggam_r, gmu_r, h_r = adjoint_ref.loss_and_grads(st0, se, 1.0, 1.0, dt, steps, 1.0, NB, AMAX,
                                                                    target)
    assert np.allclose(h, h_r, rtol=1e-9, atol=1e-14)
    assert abs(loss_of(h, target) - loss_r) <= 1e-9 * abs(loss_r)
    scale = np.abs(gse_r).max()
    assert np.abs(gse - gse_r).max() <= 1e-6 * scale, (np.abs(gse - gse_r).max(), scale)
    assert abs(ggam - ggam_r) <= 1e-6 * abs(ggam_r), (ggam, ggam_r)
    assert abs(gmu - gmu_r) <= 1e-6 * abs(gmu_r), (gmu, gmu_r)
    e.close()


def central_fd(gpu, mesh, dt, steps, se, gam, mu, target, which, h, direction=None):
    """(loss(+h) - loss(-h)) / 2h of one parameter, with the event
    sequences of both runs returned for comparison."""
    out = []
    for sgn in (1.0, -1.0):
        s, g, m = se.copy(), gam, mu
        if which == "se":
            s = se + sgn * h * direction
        elif which == "gamma":
            g = gam + sgn * h
        else:
            m = mu + sgn * h
        e, hh, ev = forward(gpu, mesh, dt, steps, s, g, m)
        e.close()
        out.append((loss_of(hh, target), ev))
    return (out[0][0] - out[1][0]) / (2 * h), out[0][1], out[1][1]


def test_adjoint_matches_central_differences_through_events(gpu):
    """h = 1e-4: the forward's finite-difference velocity carries rounding
    noise of ~1e-8 relative, which a step of 1e-6 turns into differences of
    1e-6..1e-4 relative; at 1e-4 the central difference's own error
    (O(h^2)) stays below 1e-7."""
    import meshgen
    mesh = meshgen.make_inputs(400, 9)
    rng = np.random.default_rng(2)
    se = rng.uniform(0.0, 0.5, 400)
    dt, steps = 1e-4, 300
    e, h, events = forward(gpu, mesh, dt, steps, se, 1.0, 1.0, every=100)
    n_ev = np.array(events).sum(0)
    assert n_ev[0] > 0 and n_ev[1] > 0, "window should contain flips and removals: %s" % n_ev
    e2, h2, _ = forward(gpu, mesh, dt, steps, se * 1.3, 1.1, 0.9)
    e2.close()
    target = h2
    gse, ggam, gmu = e.adjoint_histogram(NB, AMAX, dloss(h, target))
    e.close()
    d = rng.standard_normal(400)
    checks = [("mu", gmu, None), ("gamma", ggam, None), ("se", float(gse @ d), d)]
    for which, adj, direction in checks:
        fd, ev_p, ev_m = central_fd(gpu, mesh, dt, steps, se, 1.0, 1.0, target, which, 1e-4, direction)
        assert ev_p == events and ev_m == events, "%s: perturbed runs changed the event sequence" % which
        assert abs(adj - fd) <= 2e-5 * abs(fd), (which, adj, fd)


def test_torch_function_gradients(gpu):
    torch = pytest.importorskip("torch")
    import meshgen
    import sevc_torch
    mesh = meshgen.make_inputs(200, 4)
    se0 = np.random.default_rng(3).uniform(0.0, 0.5, 200)
    dt, steps = 2e-5, 60
    target = torch.full((NB,), 1.0 / NB, dtype=torch.float64)
    se = torch.tensor(se0, requires_grad=True)
    gam = torch.tensor(1.0, dtype=torch.float64, requires_grad=True)
    mu = torch.tensor(1.0, dtype=torch.float64, requires_grad=True)
    h = sevc_torch.GrainAreaHistogram.apply(se, gam, mu, lambda: make(gpu, mesh, dt), steps, NB, AMAX, 25)
    loss = sevc_torch.histogram_loss(h, target)
    loss.backward()
    e, hh, _ = forward(gpu, mesh, dt, steps, se0, 1.0, 1.0, every=25)
    assert np.array_equal(h.detach().numpy(), hh)
    gse, ggam, gmu = e.adjoint_histogram(NB, AMAX, dloss(hh, target.numpy()))
    e.close()
    assert np.allclose(se.grad.numpy(), gse, rtol=1e-12, atol=0)
    assert np.isclose(float(gam.grad), ggam, rtol=1e-12) and np.isclose(float(mu.grad), gmu, rtol=1e-12)


def nucleation_window(gpu, tmp_path, dt_window=1e-3, before=1, after=2, quiet=False):
    """The 300-grain fixture with its triangular stored energies (3..6;
    grains about one unit across, where the Metropolis test accepts
    nucleations), run at dt 4e-3 until 1/6 of the grains are gone (the gate
    for nucleation attempts), then at dt_window with one attempt per step
    until an attempt is accepted with `before` steps ahead of it and
    `after` steps behind it (quiet: none of them with a flip or a removal).
    Returns the options, the mesh, a checkpoint at the window's start and
    the window's length: it moves the vertices, nucleates, and moves them
    again."""
    import os
    import configs
    import meshgen
    d = os.path.join(configs.MESH_DIR, "m300")
    mesh = meshgen.read_files(*[os.path.join(d, f) for f in ("vertices.txt", "ridges.txt", "oris.txt",
                                                              "se_triangular.txt")])
    n = 300

    def opts(dt):
        o = gpu.default_options(n_grains=n, dt=dt, dtau=dt, domain_bound=17.0, GB_eps=0.0, GB_scaling=1.0,
                                SE_eps=1.0, SE_min=999.0, SE_max=999.0, do_nucleation=1, MC_k=3.0,
                                nmax=10 ** 8, tmax=-1, snap_gap=10 ** 8, n_blocks=32, n_threads=256)
        o.min_grains = -1
        return o
    e = gpu.Engine.from_arrays(opts(4e-3), mesh["xy"], mesh["ridges"], mesh["oris"], mesh["se"])
    for _ in range(2000):
        if e.step().curr_n_grains <= 5 * n // 6:
            break
    gate = str(tmp_path / "gate.ckpt")
    e.checkpoint_save(gate)
    e.close()
    o = opts(dt_window)
    e = gpu.Engine.from_arrays(o, mesh["xy"], mesh["ridges"], mesh["oris"], mesh["se"])
    e.checkpoint_load(gate)
    R = before + after + 2
    ring = [str(tmp_path / ("w%d.ckpt" % i)) for i in range(R)]
    moves, nucl = [], []
    for k in range(6000):
        e.checkpoint_save(ring[k % R])
        i = e.step()
        moves.append(i.n_flips + i.n_removals + i.n_two_three)
        nucl.append(i.n_nucleations)
        c = k - after
        if c - before >= 0 and nucl[c] > 0 and not (quiet and any(moves[c - before:k + 1])):
            e.close()
            return o, mesh, ring[(c - before) % R], before + 1 + after
    pytest.fail("no suitable nucleation within 6000 steps past the gate")


def window_run(gpu, o, mesh, ckpt, window, se, gam, mu, every=None):
    ee = gpu.Engine.from_arrays(o, mesh["xy"], mesh["ridges"], mesh["oris"], mesh["se"])
    ee.checkpoint_load(ckpt)
    ee.set_stored_energy(se)
    ee.set_gb_scaling(gam)
    ee.set_mobility(mu)
    if every:
        ee.tape_start(every)
    ev = []
    for _ in range(window):
        i = ee.step()
        ev.append((i.n_flips, i.n_removals, i.n_two_three, i.n_nucleations,
                   i.nucleation_candidate if i.nucleation_attempted else -2))
    return ee, ee.area_histogram(NB, AMAX), ev


def window_state(gpu, o, mesh, ckpt):
    p = gpu.Engine.from_arrays(o, mesh["xy"], mesh["ridges"], mesh["oris"], mesh["se"])
    p.checkpoint_load(ckpt)
    st = p.get_state()
    p.close()
    return st


def test_adjoint_matches_central_differences_through_nucleation(gpu, tmp_path):
    """A window around an accepted nucleation (nucleation_window): the
    adjoint follows the inserted triangle's position map back to the
    positions the step before moved.  Five-point differences of the GPU
    forward over the same window (every run starts from the checkpoint; the
    perturbed runs are checked to take the same events, the nucleation site
    included) agree within 2e-5 relative for the mobility, the boundary
    energy scale and the stored energies of the original grains along the
    gradient (a nucleated grain's stored energy is 0, not a parameter).
    The loss compares the histogram with itself shifted by one bin, so its
    gradient is no near-cancellation of bins.  The forward's
    finite-difference velocity carries rounding noise of ~1e-8 relative, so
    a difference quotient over a few steps is good to ~1e-8/h only: h is
    3e-3..3e-2 (the exact check is the FP64 reference below)."""
    o, mesh, ckpt, window = nucleation_window(gpu, tmp_path)
    st = window_state(gpu, o, mesh, ckpt)
    se0 = st["gse"].copy()
    free = (st["gen"] > 0) & (st["gtype"] == 0)          # grains whose stored energy is a parameter
    run = lambda se, g, m, every=None: window_run(gpu, o, mesh, ckpt, window, se, g, m, every)
    e0, h0, events = run(se0, 1.0, 1.0)
    e0.close()
    assert events[1][3] == 1, events
    target = np.roll(h0, 1)
    e, h, _ = run(se0, 1.0, 1.0, every=2)
    gse, ggam, gmu = e.adjoint_histogram(NB, AMAX, dloss(h, target))
    e.close()
    assert np.all(gse[~free] == 0.0)
    dirn = np.where(free, gse, 0.0)
    dirn /= np.linalg.norm(dirn)
    for which, adj in (("mu", gmu), ("gamma", ggam), ("se", float(gse @ dirn))):
        errs = []
        for hstep in (3e-2, 1e-2, 3e-3):
            f = {}
            for k in (2, 1, -1, -2):
                s_, g, m = se0.copy(), 1.0, 1.0
                if which == "se":
                    s_ = se0 + k * hstep * dirn
                elif which == "gamma":
                    g += k * hstep
                else:
                    m += k * hstep
                ee, hh, ev = run(s_, g, m)
                ee.close()
                if ev != events:
                    break
                f[k] = loss_of(hh, target)
            if len(f) == 4:
                fd = (-f[2] + 8 * f[1] - 8 * f[-1] + f[-2]) / (12 * hstep)
                errs.append((abs(adj - fd) / abs(fd), hstep, fd))
        assert errs, "%s: every perturbed run changed the event sequence" % which
        assert min(errs)[0] <= 2e-5, (which, adj, errs)


def nucleation_record(gpu, o, mesh, ckpt, k):
    """What the FP64 reference needs of the nucleation at window step k:
    the vertices of the map and its factor k = 0.8 U, read from a copy of
    the run whose mobility is 1e-300 for that step only (the step then
    moves no vertex by a representable amount, so the new corners are where
    the nucleation put them; the attempt itself does not depend on the
    mobility), and the mesh right after it."""
    e = gpu.Engine.from_arrays(o, mesh["xy"], mesh["ridges"], mesh["oris"], mesh["se"])
    e.checkpoint_load(ckpt)
    for _ in range(k):
        e.step()
    pre = e.get_state()
    e.set_mobility(1e-300)
    info = e.step()
    post = e.get_state()
    e.close()
    assert info.n_nucleations == 1
    D = o.domain_bound
    wrap = lambda d: d - D * np.round(d / D)
    g = int(np.nonzero((post["gen"] > 0) & (pre["gen"] == 0))[0][0])
    A, B, C = (int(v) for v in post["glist"].reshape(-1, 100)[g, :3])
    far = []
    for j in range(3):
        b = pre["vb"].reshape(-1, 3)[A, j]
        far.append(int(pre["bend"][b] if pre["bini"][b] == A else pre["bini"][b]))
    pa = np.array([pre["px"][A], pre["py"][A]])
    AL = [np.hypot(*wrap(np.array([pre["px"][X], pre["py"][X]]) - pa)) for X in far]
    imin = int(np.argmin(AL))
    r = np.hypot(*wrap(np.array([post["px"][A], post["py"][A]]) - pa)) / 0.99
    return {"A": A, "B": B, "C": C, "far": far, "xstar": far[imin], "k": (r - 0.1) / AL[imin], "state": post}


def test_adjoint_matches_fp64_reference_through_nucleation(gpu, tmp_path):
    """A window whose only topology changes are nucleations (no flip, no
    removal; nucleation_window with quiet=True), against the FP64 torch
    restatement of the same map (oracle/adjoint_ref.py: the velocity and
    translation steps and the inserted triangle's position map with the
    recorded draw), differentiated by torch.autograd: every gradient within
    1e-6 relative, the same bound as the event-free window."""
    pytest.importorskip("torch")
    from oracle import adjoint_ref
    o, mesh, ckpt, window = nucleation_window(gpu, tmp_path, dt_window=2.5e-4, before=1, after=2, quiet=True)
    st = window_state(gpu, o, mesh, ckpt)
    se0 = st["gse"].copy()
    e, h, events = window_run(gpu, o, mesh, ckpt, window, se0, 1.0, 1.0, every=2)
    assert all(ev[:3] == (0, 0, 0) for ev in events), events
    nsteps = [k for k, ev in enumerate(events) if ev[3]]
    assert 1 in nsteps, events
    target = np.roll(h, 1)
    gse, ggam, gmu = e.adjoint_histogram(NB, AMAX, dloss(h, target))
    e.close()
    recs = {k: nucleation_record(gpu, o, mesh, ckpt, k) for k in nsteps}
    loss_r, gse_r, ggam_r, gmu_r, h_r = adjoint_ref.loss_and_grads_nucleation(
        st, recs, se0, 1.0, 1.0, o.dt, window, o.domain_bound, NB, AMAX, target)
    # the restated map rounds differently from the engine's (and k comes
    # back from the corners' positions): last-bit differences that the
    # finite-difference velocity (a quotient by 1e-8) turns into ~1e-10
    # relative in the new grain's area
    err = {"hist": float(np.max(np.abs(h - h_r) / np.maximum(np.abs(h_r), 1e-3))),
           "se": float(np.abs(gse - gse_r).max() / np.abs(gse_r).max()),
           "gamma": abs(ggam - ggam_r) / abs(ggam_r), "mu": abs(gmu - gmu_r) / abs(gmu_r)}
    assert err["hist"] <= 1e-7 and max(err["se"], err["gamma"], err["mu"]) <= 1e-6, err
