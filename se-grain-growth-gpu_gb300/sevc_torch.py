"""torch.autograd.Function over the engine's C ABI, for gradient use only.

GrainAreaHistogram.apply(se, gb_scaling, mu, make_engine, steps, nbins,
amax, checkpoint_every) runs `steps` time steps on the GPU from the state
`make_engine()` returns, with the given per-grain stored energies, boundary
energy scaling and mobility, and returns the smoothed histogram of
normalised grain areas (sevc_area_histogram).  Its backward pass calls the
hand-written adjoint (sevc_adjoint_histogram) and returns float64 gradients
for the three parameter tensors.  Nothing here runs the simulation in
torch: the tensors are host-side views of what the C ABI returns.
"""
import numpy as np
import torch


class GrainAreaHistogram(torch.autograd.Function):
    @staticmethod
    def forward(ctx, se, gb_scaling, mu, make_engine, steps, nbins, amax, checkpoint_every):
        eng = make_engine()
        eng.set_stored_energy(se.detach().to(torch.float64).cpu().numpy())
        eng.set_gb_scaling(float(gb_scaling))
        eng.set_mobility(float(mu))
        eng.tape_start(checkpoint_every)
        for _ in range(steps):
            eng.step()
        hist = eng.area_histogram(nbins, amax)
        ctx.eng, ctx.nbins, ctx.amax = eng, nbins, amax
        return torch.from_numpy(hist)

    @staticmethod
    def backward(ctx, grad_hist):
        eng = ctx.eng
        g = np.ascontiguousarray(grad_hist.detach().to(torch.float64).cpu().numpy())
        gse, ggb, gmu = eng.adjoint_histogram(ctx.nbins, ctx.amax, g)
        eng.close()
        ctx.eng = None
        return (torch.from_numpy(gse), torch.tensor(ggb, dtype=torch.float64), torch.tensor(gmu, dtype=torch.float64),
                None, None, None, None, None)


def histogram_loss(hist, target):
    """Mean squared error of two histograms."""
    return ((hist - target) ** 2).mean()
