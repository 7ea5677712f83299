"""Golden run configurations shared by make_golden.py and the tests.

Each configuration is an .ini (the reference's keys) over one of the
fixture meshes in tests/golden/meshes, which were produced by the
reference's own generator (voronoi/voronoi.py) by make_golden.py.
"""
import os

HERE = os.path.dirname(os.path.abspath(__file__))
MESH_DIR = os.path.join(HERE, "meshes")

# name -> (mesh, se file, ini keys, rng seed of the synthetic stream, min_grains)
CONFIGS = {
    # plain vertex model with stored energy on the unit square, isotropic
    # boundaries (GB_eps = 0), SE uniform in [0, 0.5], no nucleation
    "plain_unit": ("m1000", "se_uniform.txt", dict(
        dt="1e-4", dtau="1e-4", nmax="300", snap_gap="10", n_grains="1000", GB_eps="0.0", GB_scaling="1.0",
        SE_eps="1", SE_min="0", SE_max="0.5", domain_bound="1.0", do_nucleation="false"), 0, 10),
    # anisotropic boundaries, raw SE, nucleation every 5 steps once 1/6 of the
    # grains are gone (domain scaled so grains are ~1 unit across)
    "nucl_aniso": ("m1000", "se_uniform.txt", dict(
        dt="2e-3", dtau="1e-2", nmax="400", snap_gap="20", n_grains="1000", GB_eps="0.02", GB_scaling="1.0",
        SE_eps="1", SE_min="3", SE_max="6", domain_bound="30.0", do_nucleation="true", MC_k="1.0"), 7, 10),
    # small mesh, every step exported: per-step pin of the event sequence,
    # isotropic boundaries and nucleation at every step
    "perstep_nucl": ("m300", "se_triangular.txt", dict(
        dt="4e-3", dtau="4e-3", nmax="300", snap_gap="1", n_grains="300", GB_eps="0.0", GB_scaling="1.0",
        SE_eps="1.0", domain_bound="17.0", do_nucleation="true", MC_k="3.0"), 3, 10),
}


def write_ini(path, name, folder):
    mesh, se, keys, _, _ = CONFIGS[name]
    md = os.path.join(MESH_DIR, mesh)
    lines = ["[Temporal]"]
    lines += ["%s=%s" % (k, keys[k]) for k in ("dt", "dtau", "nmax", "snap_gap") if k in keys]
    lines += ["[Grains]", "n_grains=%s" % keys["n_grains"],
              "vertex_fname=%s" % os.path.join(md, "vertices.txt"),
              "boundary_fname=%s" % os.path.join(md, "ridges.txt"),
              "orientation_fname=%s" % os.path.join(md, "oris.txt"),
              "SE_fname=%s" % os.path.join(md, se)]
    for k in ("GB_eps", "GB_scaling", "SE_eps", "SE_min", "SE_max", "MC_k", "domain_bound", "do_nucleation"):
        if k in keys:
            lines.append("%s=%s" % (k, keys[k]))
    lines += ["[System]", "n_blocks=32", "n_threads=256", "debug_lvl=0", "[Output]", "folder=%s" % folder]
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")
    return path
