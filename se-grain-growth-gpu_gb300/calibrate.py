"""Batched stored-energy calibration through the adjoint.

A batch of microstructures is advanced `steps` steps with shared boundary
energy scale gamma, mobility mu and a stored-energy scale c (every grain's
stored energy is c times its base value); the loss is the mean squared
error between the batch's smoothed grain-area histogram and a target
histogram.  Each iteration restores the initial state from a checkpoint
file, runs the forward pass with a tape, and takes one Adam step on
(log gamma, log mu, log c) with the gradients of sevc_adjoint_histogram.

The histogram depends on the parameters through the velocity
mu * (gamma * line-tension term + c * stored-energy term) only, so the
identifiable combinations are mu*gamma and mu*c; `run` reports the errors
of both the individual parameters and of those products.

With nucleation on, the batch is first run until every instance has lost
1/6 of its grains (the reference's gate for nucleation attempts,
src/main.cu:137) and the calibration window starts there; every forward
pass restores the random streams with the checkpoint, so the attempts
replay the same draws, and the adjoint follows the inserted triangles.
"""
import os
import tempfile
import time

import numpy as np

import sevc

NB, AMAX = 20, 3.0


def batch_options(n_grains, dt, domain=1.0, nucleation=None):
    """nucleation: None, or (gap, MC_k): one Metropolis attempt every gap
    steps once an instance's gate is open"""
    gap, mck = nucleation if nucleation else (0, 1.0)
    o = sevc.default_options(n_grains=n_grains, dt=dt, dtau=gap * dt if nucleation else 1.0, nucleation_gap=gap,
                             domain_bound=domain, GB_eps=0.0, GB_scaling=1.0, SE_eps=1.0, SE_min=999.0,
                             SE_max=999.0, do_nucleation=1 if nucleation else 0, MC_k=mck, nmax=10 ** 8, tmax=-1,
                             snap_gap=10 ** 8, n_blocks=32, n_threads=256)
    o.min_grains = -1
    return o


def run_to_gate(eng, meshes, max_steps=100000):
    """step until every instance holds at most 5/6 of its initial grains"""
    n0 = [len(m["oris"]) for m in meshes]
    for k in range(max_steps):
        eng.step()
        if all(eng.instance_info(i).curr_n_grains <= 5 * n0[i] // 6 for i in range(len(meshes))):
            return k + 1
    raise RuntimeError("the nucleation gate was not reached in %d steps" % max_steps)


class Calibration:
    def __init__(self, meshes, dt, steps, checkpoint_every=50, domain=1.0, nucleation=None):
        self.meshes, self.dt, self.steps, self.every = meshes, dt, steps, checkpoint_every
        self.eng = sevc.Engine.from_batch(batch_options(len(meshes[0]["oris"]), dt, domain, nucleation), meshes)
        self.gate_steps = run_to_gate(self.eng, meshes) if nucleation else 0
        self.se0 = self.eng.get_state()["gse"].copy()
        self.dir = tempfile.mkdtemp(prefix="sevc_cal_")
        self.ckpt = os.path.join(self.dir, "initial.ckpt")
        self.eng.checkpoint_save(self.ckpt)
        self.t_fwd = self.t_bwd = 0.0

    def _forward(self, gamma, mu, c, tape):
        e = self.eng
        e.tape_stop()
        e.checkpoint_load(self.ckpt)
        e.set_gb_scaling(gamma)
        e.set_mobility(mu)
        e.set_stored_energy(self.se0 * c)
        if tape:
            e.tape_start(self.every)
        t0 = time.time()
        self.events = [0, 0, 0]
        for _ in range(self.steps):
            i = e.step()
            self.events = [self.events[0] + i.n_removals, self.events[1] + i.nucleation_attempted,
                           self.events[2] + i.n_nucleations]
        self.t_fwd += time.time() - t0
        return e.area_histogram(NB, AMAX)

    def histogram(self, gamma, mu, c):
        return self._forward(gamma, mu, c, tape=False)

    def loss_and_grad(self, gamma, mu, c, target):
        h = self._forward(gamma, mu, c, tape=True)
        loss = float(((h - target) ** 2).mean())
        t0 = time.time()
        gse, ggam, gmu = self.eng.adjoint_histogram(NB, AMAX, 2.0 * (h - target) / NB)
        self.t_bwd += time.time() - t0
        gc = float(gse @ self.se0)          # d loss / d c
        return loss, np.array([ggam, gmu, gc])

    def close(self):
        self.eng.tape_stop()
        self.eng.close()
        try:
            os.remove(self.ckpt)
            os.rmdir(self.dir)
        except OSError:
            pass


def run(meshes, dt, steps, iters, truth=(1.0, 1.0, 1.0), start=(1.3, 0.8, 0.6), lr=0.08, checkpoint_every=50,
        domain=1.0, nucleation=None):
    """Calibrate (gamma, mu, c) from `start` against the histogram the
    batch produces with `truth`.  Returns a summary dict.  The stored-energy
    term weighs against line tension in proportion to the grain size, so a
    domain of about sqrt(grains per instance) (grains one unit across, as
    in the reference's example) keeps c observable.  nucleation: None or
    (gap, MC_k), see batch_options."""
    cal = Calibration(meshes, dt, steps, checkpoint_every, domain, nucleation)
    target = cal.histogram(*truth)
    events_truth = list(cal.events)
    cal.t_fwd = 0.0
    theta = np.log(np.array(start, float))
    m = np.zeros(3)
    v = np.zeros(3)
    losses = []
    b1, b2 = 0.9, 0.999
    for k in range(1, iters + 1):
        p = np.exp(theta)
        loss, g = cal.loss_and_grad(p[0], p[1], p[2], target)
        losses.append(loss)
        g = g * p                              # chain rule to log-parameters
        m = b1 * m + (1 - b1) * g
        v = b2 * v + (1 - b2) * g * g
        theta -= lr * (m / (1 - b1 ** k)) / (np.sqrt(v / (1 - b2 ** k)) + 1e-30)
    p = np.exp(theta)
    final_loss = float(((cal.histogram(*p) - target) ** 2).mean())
    t_fwd, t_bwd = cal.t_fwd, cal.t_bwd
    cal_gate = cal.gate_steps
    cal.close()
    truth = np.array(truth, float)
    start = np.array(start, float)
    ident = lambda q: np.array([q[1] * q[0], q[1] * q[2]])
    return {"instances": len(meshes), "grains": int(sum(len(mm["oris"]) for mm in meshes)), "steps": steps,
            "iterations": iters, "dt": dt, "domain_bound": domain, "params": ["gamma", "mu", "se_scale"],
            "truth": truth.tolist(), "start": start.tolist(), "final": p.tolist(),
            "rel_err_start": (np.abs(start - truth) / truth).tolist(),
            "rel_err_final": (np.abs(p - truth) / truth).tolist(),
            "identifiable": ["mu*gamma", "mu*se_scale"],
            "rel_err_identifiable_start": (np.abs(ident(start) - ident(truth)) / ident(truth)).tolist(),
            "rel_err_identifiable_final": (np.abs(ident(p) - ident(truth)) / ident(truth)).tolist(),
            "loss_first": losses[0], "loss_last": losses[-1], "loss_final": final_loss,
            "forward_s": t_fwd, "backward_s": t_bwd,
            "backward_forward_ratio": t_bwd / t_fwd if t_fwd > 0 else None,
            "nucleation": None if not nucleation else {"gap": nucleation[0], "MC_k": nucleation[1],
                                                       "steps_to_gate": cal_gate},
            "window_events_at_truth": {"removals": events_truth[0], "nucleation_attempts": events_truth[1],
                                       "nucleations": events_truth[2]}}
