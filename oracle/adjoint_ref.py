"""FP64 reference gradient of the time step (test infrastructure only).

A plain torch float64 restatement of the forward map that the engine's
adjoint differentiates, for a window of steps with a fixed topology:

  v_i^c = mu * ( -[ sum_j gamma (L_j(x + eps e_i^c) - L_j(x))
                    + sum_g SE_g (|A_g(x + eps e_i^c)| - |A_g(x)|) ] / eps )
  x <- (x + dt v) mod D

(the reference's compute_vertex_velocities, src/calculus.h:19-73, with
energy_diff's perturbed arclengths and perturbed polygon areas computed
explicitly here, and update_vertices_positions, src/calculus.h:391-404),
followed by the smoothed area histogram and a mean-squared-error loss.
torch.autograd then gives the gradient the adjoint must reproduce.  Only
isotropic boundaries (GB_eps = 0, gamma = GB_scaling) are restated.
Nothing in the engine imports this file.
"""
import numpy as np
import torch

GRAD_EPS = 1e-8


def _wrap(d, D):
    return d - D * torch.round(d / D)


class Topology:
    """Index arrays of one fixed mesh, from a get_state() dict."""

    def __init__(self, st):
        self.ven = st["ven"].astype(bool)
        vb = st["vb"].reshape(-1, 3)
        vg = st["vg"].reshape(-1, 3)
        bini, bend = st["bini"], st["bend"]
        gl = st["glist"].reshape(-1, 100)
        gvl = st["gvlen"]
        gen = st["gen"].astype(bool)
        self.grains = np.nonzero(gen)[0]
        maxn = int(gvl[self.grains].max())
        L = np.zeros((len(self.grains), maxn), np.int64)
        for r, g in enumerate(self.grains):
            n = gvl[g]
            L[r, :n] = gl[g, :n]
            L[r, n:] = gl[g, n - 1]          # padding repeats the last vertex: zero edges
        self.L, self.n = L, gvl[self.grains]
        row = {g: r for r, g in enumerate(self.grains)}
        vi, vq, vbnd, pi, pg, pp = [], [], [], [], [], []
        for i in np.nonzero(self.ven)[0]:
            for j in range(3):
                b = vb[i, j]
                vi.append(i)
                vq.append(bend[b] if bini[b] == i else bini[b])
                vbnd.append(b)
            for j in range(3):
                g = vg[i, j]
                if g < 0 or not gen[g]:
                    continue
                p = int(np.nonzero(gl[g, :gvl[g]] == i)[0][0])
                pi.append(i)
                pg.append(row[g])
                pp.append(p)
        self.vi, self.vq = torch.tensor(vi), torch.tensor(vq)
        self.pi, self.pg, self.pp = torch.tensor(pi), torch.tensor(pg), torch.tensor(pp)
        self.verts = torch.tensor(np.nonzero(self.ven)[0])
        self.bini, self.bend = torch.tensor(bini[st["ben"].astype(bool)]), torch.tensor(bend[st["ben"].astype(bool)])


def polygon_areas(pts, D):
    """Signed shoelace areas of polygons pts (K, n, 2), unwrapped from vertex 0."""
    d = _wrap(pts[:, 1:] - pts[:, :-1], D)
    r = torch.cat([torch.zeros_like(pts[:, :1]), torch.cumsum(d, 1)], 1)
    cr = r[:, :-1, 0] * r[:, 1:, 1] - r[:, :-1, 1] * r[:, 1:, 0]
    return 0.5 * cr.sum(1)


def velocities(x, topo, se, gamma, mu, D):
    L = torch.as_tensor(topo.L)
    A = polygon_areas(x[L], D)
    # boundary term: each vertex's three boundaries, moved copies of the vertex
    xi, xq = x[topo.vi], x[topo.vq]
    d0 = _wrap(xi - xq, D)
    L0 = torch.sqrt((d0 ** 2).sum(1))
    out = []
    for c in range(2):
        e = torch.zeros(2, dtype=x.dtype)
        e[c] = GRAD_EPS
        d1 = _wrap(xi + e - xq, D)
        L1 = torch.sqrt((d1 ** 2).sum(1))
        bt = torch.zeros(x.shape[0], dtype=x.dtype).index_add(0, topo.vi, gamma * (L1 - L0))
        # stored-energy term: the vertex's grains with the vertex moved
        pts = x[L[topo.pg]].clone()
        rows = torch.arange(len(topo.pg))
        pts[rows, topo.pp] = pts[rows, topo.pp] + e
        # padding copies of the moved vertex (when it is the list's last) move too
        last = torch.as_tensor(topo.n)[topo.pg] - 1
        pad = torch.arange(L.shape[1])[None, :] > last[:, None]
        moved_last = (topo.pp == last)[:, None] & pad
        pts = torch.where(moved_last[..., None], pts[rows, topo.pp][:, None, :].expand_as(pts), pts)
        A1 = polygon_areas(pts, D)
        gt = torch.zeros(x.shape[0], dtype=x.dtype).index_add(
            0, topo.pi, se[torch.as_tensor(topo.grains)][topo.pg] * (A1.abs() - A[topo.pg].abs()))
        out.append(mu * (-(bt + gt) / GRAD_EPS))
    return torch.stack(out, 1)


def bspline2(s):
    a = s.abs()
    return torch.where(a <= 0.5, 0.75 - s * s, torch.where(a <= 1.5, 0.5 * (1.5 - a) ** 2, torch.zeros_like(s)))


def histogram(x, topo, D, nbins, amax):
    A = polygon_areas(x[torch.as_tensor(topo.L)], D)
    N = len(topo.grains)
    a = A.abs() * N / (D * D)
    w = amax / nbins
    k = torch.arange(nbins, dtype=x.dtype)
    return bspline2(a[:, None] / w - k[None, :] - 0.5).sum(0) / N


def loss_and_grads(st, se0, gamma0, mu0, dt, steps, D, nbins, amax, target):
    """Loss after `steps` steps from state `st` and its gradients with
    respect to (se, gamma, mu), all float64."""
    topo = Topology(st)
    se = torch.tensor(se0, dtype=torch.float64, requires_grad=True)
    gamma = torch.tensor(float(gamma0), dtype=torch.float64, requires_grad=True)
    mu = torch.tensor(float(mu0), dtype=torch.float64, requires_grad=True)
    x = torch.tensor(np.stack([st["px"], st["py"]], 1), dtype=torch.float64)
    V = topo.verts
    for _ in range(steps):
        v = velocities(x, topo, se, gamma, mu, D)
        x = x.clone()
        x[V] = torch.remainder(x[V] + dt * v[V], D)
    h = histogram(x, topo, D, nbins, amax)
    loss = ((h - torch.as_tensor(target)) ** 2).mean()
    loss.backward()
    return float(loss.detach()), se.grad.numpy(), float(gamma.grad), float(mu.grad), h.detach().numpy()


def nucleation_map(x, rec, D):
    """Positions after a nucleation at vertex A (nucleation2.cu:116-212 with
    the move of nucleate, :474-676): the new corners A, B, C sit at
    A + 0.99 r (X - A)/|X - A| for A's far ends X = D, E, F, with
    r = k |X* - A| + 0.1 (X* the end of A's shortest boundary, k = 0.8 U
    for the recorded draw U).  rec: A, B, C, far (D, E, F), xstar, k."""
    pa = x[rec["A"]]
    ds = _wrap(x[rec["xstar"]] - pa, D)
    r = rec["k"] * torch.sqrt((ds ** 2).sum()) + 0.1
    out = []
    for X in rec["far"]:
        t = _wrap(x[X] - pa, D)
        out.append(torch.remainder(pa + 0.99 * r * t / torch.sqrt((t ** 2).sum()), D))
    x = x.clone()
    x[rec["A"]], x[rec["B"]], x[rec["C"]] = out[0], out[1], out[2]
    return x


def loss_and_grads_nucleation(st, nucl, se0, gamma0, mu0, dt, steps, D, nbins, amax, target):
    """loss_and_grads for a window whose only topology changes are
    nucleations: nucl maps a step index to a record (nucleation_map's
    fields plus "state", a get_state() dict holding the mesh right after
    that nucleation), applied before the step's velocities.  A grain of
    nonzero type (nucleated) has stored energy 0, not a parameter."""
    se = torch.tensor(se0, dtype=torch.float64, requires_grad=True)
    gamma = torch.tensor(float(gamma0), dtype=torch.float64, requires_grad=True)
    mu = torch.tensor(float(mu0), dtype=torch.float64, requires_grad=True)
    x = torch.tensor(np.stack([st["px"], st["py"]], 1), dtype=torch.float64)

    def setup(s):
        return Topology(s), torch.tensor((s["gtype"] == 0).astype(np.float64))
    topo, free = setup(st)
    for k in range(steps):
        if k in nucl:
            x = nucleation_map(x, nucl[k], D)
            topo, free = setup(nucl[k]["state"])
        v = velocities(x, topo, se * free, gamma, mu, D)
        V = topo.verts
        x = x.clone()
        x[V] = torch.remainder(x[V] + dt * v[V], D)
    h = histogram(x, topo, D, nbins, amax)
    loss = ((h - torch.as_tensor(target)) ** 2).mean()
    loss.backward()
    return float(loss.detach()), se.grad.numpy(), float(gamma.grad), float(mu.grad), h.detach().numpy()
