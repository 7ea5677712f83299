"""Periodic Voronoi initial microstructures in the reference's input format.

The reference ships voronoi/voronoi.py, a pure-Python generator (3x3 tiling,
Python loops; about 3-4 minutes at 1M grains).  Two generators produce the
same kind of input: the library's C generator (sevc_voronoi_generate,
OpenMP cell clipping; a few seconds at 1M grains), and this module's
numpy/scipy version:

* N seeds uniform in the unit square; only seeds within a margin of the
  border are replicated into the eight periodic images (the Voronoi cells
  of the original seeds are then exact);
* ridges with at least one vertex inside the unit square are kept, vertex
  positions are folded into [0, 1) and merged on a 2**-32 grid, the same
  rule voronoi.py uses (voronoi.py:47-48);
* every kept vertex must be a triple junction, otherwise a new sample is
  drawn (voronoi.py:75-84).

Outputs: vertices (V x 2, in [0, 1)), ridges (B x 2), orientations in
[0, 1) and stored energies, with V = 2N and B = 3N.
"""
import os

import numpy as np

RES = 2 ** 32


def periodic_voronoi(n, rng, max_attempts=20, points=None):
    """points: the n seeds (in [0, 1)^2) instead of uniform draws; a mesh
    that is not made of triple junctions then raises instead of redrawing."""
    from scipy.spatial import Voronoi

    for _ in range(1 if points is not None else max_attempts):
        pts = rng.random((n, 2)) if points is None else np.asarray(points, np.float64)
        margin = min(0.5, 8.0 / np.sqrt(n))
        imgs = [pts]
        for dx in (-1.0, 0.0, 1.0):
            for dy in (-1.0, 0.0, 1.0):
                if dx == 0.0 and dy == 0.0:
                    continue
                sh = pts + (dx, dy)
                keep = (sh[:, 0] > -margin) & (sh[:, 0] < 1 + margin) & (sh[:, 1] > -margin) & (sh[:, 1] < 1 + margin)
                imgs.append(sh[keep])
        vor = Voronoi(np.concatenate(imgs))
        V = vor.vertices
        inside = (V[:, 0] >= 0) & (V[:, 0] < 1) & (V[:, 1] >= 0) & (V[:, 1] < 1)
        kx = np.mod(np.round(V[:, 0] * RES), RES).astype(np.uint64)
        ky = np.mod(np.round(V[:, 1] * RES), RES).astype(np.uint64)
        key = (kx << np.uint64(32)) | ky
        ukey, inv = np.unique(key, return_inverse=True)
        rv = np.asarray(vor.ridge_vertices, dtype=np.int64)
        ok = (rv[:, 0] >= 0) & (rv[:, 1] >= 0)
        rv = rv[ok]
        ok = inside[rv[:, 0]] | inside[rv[:, 1]]
        rv = rv[ok]
        a, b = inv[rv[:, 0]], inv[rv[:, 1]]
        ok = a != b
        a, b = a[ok], b[ok]
        lo, hi = np.minimum(a, b), np.maximum(a, b)
        pair = np.unique(lo.astype(np.int64) * len(ukey) + hi)
        lo, hi = pair // len(ukey), pair % len(ukey)
        deg = np.bincount(np.concatenate([lo, hi]), minlength=len(ukey))
        if np.any((deg != 0) & (deg != 3)):
            continue
        used = np.nonzero(deg == 3)[0]
        newid = -np.ones(len(ukey), np.int64)
        newid[used] = np.arange(len(used))
        xy = np.stack([(ukey[used] >> np.uint64(32)).astype(np.float64) / RES,
                       (ukey[used] & np.uint64(0xFFFFFFFF)).astype(np.float64) / RES], axis=1)
        ridges = np.stack([newid[lo], newid[hi]], axis=1).astype(np.int32)
        if len(xy) != 2 * n or len(ridges) != 3 * n:
            continue
        return xy, ridges
    raise RuntimeError("could not build a periodic Voronoi mesh of %d grains" % n)


def make_inputs(n, seed, se="uniform", se_params=None, generator="scipy"):
    """Mesh, orientations and stored energies for `n` grains.

    se: "uniform" U[0,1) (rescaled by SE_min/SE_max in the options),
        "lognormal" with se_params=(mu, sigma), "triangular" (3, 6, 6) like
        voronoi.py --sedist triangular.
    generator: "scipy" (this module, numpy + scipy.spatial.Voronoi) or "c"
        (the library's OpenMP generator sevc_voronoi_generate, several
        times faster; same distribution, different sample for a seed).
    """
    rng = np.random.default_rng(seed)
    if generator == "c":
        import sevc
        m = sevc.voronoi(n, seed, "triangular" if se == "triangular" else "uniform")
        if se == "lognormal":
            mu, sigma = se_params or (-1.0, 0.5)
            m["se"] = rng.lognormal(mu, sigma, n)
        return m
    xy, ridges = periodic_voronoi(n, rng)
    oris = rng.random(n)
    if se == "lognormal":
        mu, sigma = se_params or (-1.0, 0.5)
        sev = rng.lognormal(mu, sigma, n)
    elif se == "triangular":
        sev = rng.triangular(3, 6, 6, n)
    else:
        sev = rng.random(n)
    return {"xy": xy, "ridges": ridges, "oris": oris, "se": sev, "n_grains": n}


def write_files(dirpath, inp):
    """Write vertices.txt, ridges.txt, oris.txt, se.txt (voronoi.py formats)."""
    os.makedirs(dirpath, exist_ok=True)
    paths = {k: os.path.join(dirpath, k + ".txt") for k in ("vertices", "ridges", "oris", "se")}
    np.savetxt(paths["vertices"], inp["xy"], fmt="%.16f %.16f")
    np.savetxt(paths["ridges"], inp["ridges"], fmt="%d %d")
    np.savetxt(paths["oris"], inp["oris"], fmt="%.16f")
    np.savetxt(paths["se"], inp["se"], fmt="%.16f")
    return paths


def read_files(vertices, ridges, oris, se):
    xy = np.loadtxt(vertices, dtype=np.float64, ndmin=2)
    rd = np.loadtxt(ridges, dtype=np.int32, ndmin=2)
    return {"xy": xy, "ridges": rd, "oris": np.loadtxt(oris, ndmin=1), "se": np.loadtxt(se, ndmin=1),
            "n_grains": len(xy) // 2}
