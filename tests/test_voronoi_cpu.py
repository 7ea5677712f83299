"""The C input generator (sevc_voronoi_generate, the job of the reference's
voronoi/voronoi.py) on the host: valid periodic triple-junction meshes that
the reference's loader accepts, the drop-in command line writes voronoi.py's
four files, and the meshes agree in distribution with the ones voronoi.py
itself made (the fixtures in tests/golden/meshes, regenerated by
make_golden.py): side counts and normalised grain areas."""
import os
import subprocess

import numpy as np
import pytest

import configs


def areas_and_sides(m):
    """|area| (unit square) and side count of every grain of a loaded mesh"""
    L, n = m["glist"].reshape(-1, 100), m["gvlen"]
    px, py = m["px"], m["py"]
    out = np.empty(len(n))
    for g in range(len(n)):
        v = L[g, :n[g]]
        x, y = px[v], py[v]
        dx, dy = np.diff(np.r_[x, x[0]]), np.diff(np.r_[y, y[0]])
        dx -= np.round(dx)
        dy -= np.round(dy)
        X, Y = np.r_[0.0, np.cumsum(dx)[:-1]], np.r_[0.0, np.cumsum(dy)[:-1]]
        out[g] = abs(0.5 * np.sum(X * np.roll(Y, -1) - Y * np.roll(X, -1)))
    return out, n.astype(int)


def load(engine_mod, inp, tmp, name):
    paths = [os.path.join(tmp, name + s) for s in (".v", ".r", ".o", ".s")]
    engine_mod.voronoi_write(inp, *paths)
    n = len(inp["oris"])
    opt = engine_mod.default_options(n_grains=n, dt=1e-4, dtau=1e-4, domain_bound=1.0, vertex_fname=paths[0],
                                     boundary_fname=paths[1], orientation_fname=paths[2], SE_fname=paths[3])
    return engine_mod.load_mesh_host(opt)


@pytest.mark.parametrize("n,seed", [(64, 1), (300, 2), (5000, 3)])
def test_generator_meshes_load_and_check(engine_mod, n, seed, tmp_path):
    inp = engine_mod.voronoi(n, seed)
    assert inp["xy"].shape == (2 * n, 2) and inp["ridges"].shape == (3 * n, 2)
    assert inp["xy"].min() >= 0 and inp["xy"].max() < 1
    assert np.all(np.bincount(inp["ridges"].ravel(), minlength=2 * n) == 3)
    assert np.all(inp["xy"] * 2.0 ** 32 == np.round(inp["xy"] * 2.0 ** 32))     # the 2^-32 grid
    m = load(engine_mod, inp, str(tmp_path), "g")
    assert engine_mod.check_mesh_host(m) == 0
    a, _ = areas_and_sides(m)
    assert abs(a.sum() - 1.0) < 1e-9
    again = engine_mod.voronoi(n, seed)
    assert all(np.array_equal(again[k], inp[k]) for k in ("xy", "ridges", "oris", "se"))


def test_generator_command_line(engine_mod, tmp_path):
    exe = os.path.join(os.path.dirname(engine_mod.LIB_PATH), "sevc-voronoi")
    f = [str(tmp_path / x) for x in ("v.txt", "r.txt", "o.txt", "se.txt")]
    r = subprocess.run([exe, "500", "9"] + f + ["--sedist", "triangular"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert "Vertices: 1000" in r.stdout and "Ridges: 1500" in r.stdout
    se = np.loadtxt(f[3])
    assert len(se) == 500 and se.min() >= 3 and se.max() <= 6
    opt = engine_mod.default_options(n_grains=500, dt=1e-4, dtau=1e-4, vertex_fname=f[0], boundary_fname=f[1],
                                     orientation_fname=f[2], SE_fname=f[3])
    m = engine_mod.load_mesh_host(opt)
    assert engine_mod.check_mesh_host(m) == 0


def test_generator_distribution_matches_voronoi_py(engine_mod, tmp_path):
    """Poisson-Voronoi statistics against the reference generator's own
    meshes (5,300 grains over four fixtures): side-count frequencies
    (chi-square) and normalised areas a = A N (two-sample KS)."""
    from scipy import stats
    ref_a, ref_s = [], []
    for mesh, n in (("m300", 300), ("m1000", 1000), ("m2000", 2000), ("ref2k", 2000)):
        d = os.path.join(configs.MESH_DIR, mesh)
        opt = engine_mod.default_options(n_grains=n, dt=1e-4, dtau=1e-4,
                                         vertex_fname=os.path.join(d, "vertices.txt"),
                                         boundary_fname=os.path.join(d, "ridges.txt"),
                                         orientation_fname=os.path.join(d, "oris.txt"),
                                         SE_fname=os.path.join(d, "se_uniform.txt"))
        a, s = areas_and_sides(engine_mod.load_mesh_host(opt))
        ref_a.append(a * n)
        ref_s.append(s)
    ref_a, ref_s = np.concatenate(ref_a), np.concatenate(ref_s)
    mine_a, mine_s = [], []
    for seed in (11, 12):
        n = 10000
        a, s = areas_and_sides(load(engine_mod, engine_mod.voronoi(n, seed), str(tmp_path), "s%d" % seed))
        mine_a.append(a * n)
        mine_s.append(s)
    mine_a, mine_s = np.concatenate(mine_a), np.concatenate(mine_s)
    assert stats.ks_2samp(mine_a, ref_a).pvalue > 0.01
    bins = np.arange(3, 12)
    ref_c = np.array([np.sum(np.clip(ref_s, 3, 11) == k) for k in bins], float)
    mine_c = np.array([np.sum(np.clip(mine_s, 3, 11) == k) for k in bins], float)
    keep = (ref_c >= 5) & (mine_c >= 5)
    chi = stats.chi2_contingency(np.vstack([ref_c[keep], mine_c[keep]]))
    assert chi.pvalue > 0.01, (ref_c, mine_c)
    assert abs(mine_s.mean() - 6.0) < 1e-12                         # Euler
    assert abs(mine_s.var() - 1.78) < 0.08                          # Poisson-Voronoi side variance
