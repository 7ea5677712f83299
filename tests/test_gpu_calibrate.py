"""Batched calibration through the adjoint: gradient steps on (gamma, mu,
stored-energy scale) must drive the histogram loss down and move the
identifiable products mu*gamma and mu*scale toward the generating values."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_calibration_reduces_loss_and_error(gpu):
    import meshgen
    import calibrate
    meshes = [meshgen.make_inputs(n, s) for n, s in [(700, 41), (900, 42), (800, 43), (600, 44)]]
    r = calibrate.run(meshes, dt=1e-4, steps=120, iters=15, start=(1.25, 0.85, 0.7), lr=0.06,
                      checkpoint_every=40)
    assert r["loss_final"] < 0.5 * r["loss_first"], r
    assert max(r["rel_err_identifiable_final"]) < max(r["rel_err_identifiable_start"]), r
    assert r["backward_forward_ratio"] < 3.0, r


def test_calibration_with_nucleation(gpu):
    """The same through a window past the 5/6 gate with one Metropolis
    attempt every 5 steps (triangular 3..6 stored energies, where attempts
    are accepted): nucleations happen in the window, the forward replays
    the same draws every iteration and the adjoint follows them; the loss
    falls and the backward pass costs under 3 forwards."""
    import meshgen
    import calibrate
    meshes = [meshgen.make_inputs(n, s, se="triangular", generator="c") for n, s in [(1500, 51), (1200, 52), (1800, 53)]]
    r = calibrate.run(meshes, dt=1e-4, steps=40, iters=20, start=(1.25, 0.85, 0.7), lr=0.06, checkpoint_every=20,
                      domain=float(np.sqrt(1500)), nucleation=(5, 3.0))
    assert r["window_events_at_truth"]["nucleations"] > 0, r
    assert r["loss_final"] < 0.7 * r["loss_first"], r
    assert r["backward_forward_ratio"] < 3.0, r
