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
