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


# Long runs on the configurations the benchmark specification names.  The
# reference's own sources built for the CPU take ~0.1 s per step, so their
# golden record covers the first FIRST_STEPS steps of each (the stop rule
# replaced by nmax; the trajectory up to there is the same): the oracle is
# pinned on that prefix in the CPU suite, the GPU engine against the
# oracle on the whole run and against the reference on the prefix.
LONG_CONFIGS = {
    # the reference's own fixture (voronoi/2K) with config/example.ini as
    # shipped; min_grains = leave_percent * n_grains = 100 (the reference
    # hard-codes 5000, src/main.cu:49, which stops a 2000-grain run at once).
    # Flips, removals, 2x3 pairs and conflicts all occur.
    "example_ref2k": ("ref2k", "se_uniform.txt", dict(
        dt="1e-4", dtau="1e-4", tmax="10", snap_gap="100", leave_percent="0.05", n_grains="2000", GB_eps="0.0",
        GB_scaling="1.0", SE_eps="1", SE_min="3", SE_max="6", domain_bound="40.0", do_nucleation="false"), 0, 100),
    # plain method, small: 2,000 grains, isotropic, SE uniform in [0, 0.5],
    # dt = 1e-6, unit square, nucleation off, run until 50% of the grains
    # are removed -- on the reference's fixture and on a voronoi.py mesh
    "c1_ref2k": ("ref2k", "se_uniform.txt", dict(
        dt="1e-6", dtau="1e-6", nmax="1000000", snap_gap="2500", n_grains="2000", GB_eps="0.0", GB_scaling="1.0",
        SE_eps="1", SE_min="0", SE_max="0.5", domain_bound="1.0", do_nucleation="false"), 0, 1000),
    "c1_m2000": ("m2000", "se_uniform.txt", dict(
        dt="1e-6", dtau="1e-6", nmax="1000000", snap_gap="2500", n_grains="2000", GB_eps="0.0", GB_scaling="1.0",
        SE_eps="1", SE_min="0", SE_max="0.5", domain_bound="1.0", do_nucleation="false"), 0, 1000),
    # dense events: grains ~1 unit across, raw SE U[0,1), dt = 0.01: tens of
    # removals and flips per step, conflicts and 2x3 pairs within 200 steps
    "events_m1000": ("m1000", "se_uniform.txt", dict(
        dt="1e-2", dtau="1e-2", nmax="300", snap_gap="10", n_grains="1000", GB_eps="0.0", GB_scaling="1.0",
        SE_eps="1", domain_bound="31.622776601683793", do_nucleation="false"), 0, 10),
}
FIRST_STEPS = 3000


def golden_nmax(name):
    """steps the golden record of a configuration covers (None: the whole run)"""
    if name not in LONG_CONFIGS:
        return None
    own = LONG_CONFIGS[name][2].get("nmax")
    return None if own is not None and "tmax" not in LONG_CONFIGS[name][2] and int(own) <= FIRST_STEPS \
        else FIRST_STEPS

ALL_CONFIGS = dict(CONFIGS, **LONG_CONFIGS)


def write_ini(path, name, folder, nmax=None):
    """nmax: run that many steps instead (the configuration's own stop
    rule is replaced; the trajectory up to then is the same)."""
    mesh, se, keys, _, _ = ALL_CONFIGS[name]
    if nmax is not None:
        keys = {k: v for k, v in keys.items() if k != "tmax"}
        keys["nmax"] = str(nmax)
    md = os.path.join(MESH_DIR, mesh)
    lines = ["[Temporal]"]
    lines += ["%s=%s" % (k, keys[k]) for k in ("dt", "dtau", "tmax", "nmax", "snap_gap", "leave_percent")
              if k in keys]
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
