"""Host-side logic on the CPU: the C ABI library, option parsing, mesh
loading, the mesh generator, and the oracle's own checks."""
import os
import re

import numpy as np
import pytest

import configs
from conftest import ROOT, gpu_available


def header_functions():
    text = open(os.path.join(ROOT, "include", "sevc.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(sevc_[a-z_0-9]+)\s*\(", text)))


def test_library_exports_every_declared_symbol(engine_mod):
    lib = engine_mod.lib()
    names = header_functions()
    assert len(names) >= 15
    for n in names:
        assert hasattr(lib, n), n
    assert sorted(engine_mod.EXPORTS) == names


@pytest.mark.skipif(gpu_available(), reason="checks the no-GPU error path")
def test_compute_calls_fail_without_gpu(engine_mod):
    opt = engine_mod.default_options(n_grains=2, dt=1e-3, dtau=1e-3, do_nucleation=0)
    xy = np.zeros((4, 2))
    with pytest.raises(engine_mod.SevcError) as e:
        engine_mod.Engine.from_arrays(opt, xy, np.zeros((6, 2), np.int32), np.zeros(2), np.zeros(2))
    assert e.value.code == 6
    with pytest.raises(engine_mod.SevcError):
        engine_mod.rng_record(4, 4)


def write(tmp, name, text):
    p = os.path.join(tmp, name)
    with open(p, "w") as f:
        f.write(text)
    return p


def options_dict(o):
    return {k: getattr(o, k) for k, _ in o._fields_}


@pytest.mark.parametrize("name", sorted(configs.CONFIGS))
def test_ini_parser_matches_oracle(engine_mod, oracle_mod, name, tmp_path):
    ini = configs.write_ini(str(tmp_path / "r.ini"), name, "/tmp/x")
    a, b = options_dict(engine_mod.load_ini(ini)), options_dict(oracle_mod.parse_ini(ini))
    assert a == b


def test_ini_parser_quirks(engine_mod, oracle_mod, tmp_path):
    # src/options.h:99-163: keys are not trimmed, '#'/'[' lines skipped,
    # strings lose their last character, do_nucleation only for "true\n"
    text = ("# comment\n[Temporal]\ndt=0.5\n dtau=9\ndtau =9\ndtau=1.5\nnmax=7\n"
            "vertex_fname=abc.txt\nfolder=/out/dir\ndo_nucleation=True\nGB_eps=0.25\nSE_fname=last")
    p = write(str(tmp_path), "q.ini", text)
    for o in (engine_mod.load_ini(p), oracle_mod.parse_ini(p)):
        assert o.dt == 0.5 and o.dtau == 1.5 and o.nmax == 7
        assert o.vertex_fname == b"abc.txt" and o.output_folder == b"/out/dir"
        assert o.SE_fname == b"las"          # no trailing newline: a real character is chopped
        assert o.do_nucleation == 0          # "True\n" is not "true\n"
        assert o.nucleation_gap == 3         # int(dtau / dt)
        assert o.tmax == -1 and o.GB_eps == 0.25
    p = write(str(tmp_path), "d.ini", "dt=1e-3\n")
    for o in (engine_mod.load_ini(p), oracle_mod.parse_ini(p)):
        assert o.tmax == 1.0 and o.nmax == -1 and o.do_nucleation == 1 and o.GB_eps == 0.02
        assert o.SE_min == 999 and o.min_grains == 5000


ORACLE_FIELDS = {"px": "px", "py": "py", "ven": "ven", "vb": "vb", "vg": "vg", "bini": "bini", "bend": "bend",
                 "ben": "ben", "btext": "btext", "glist": "glist", "gvlen": "gvlen", "gori": "gori", "gse": "gse",
                 "gen": "gen", "gtype": "gtype"}


@pytest.mark.parametrize("name", sorted(configs.CONFIGS))
def test_host_loader_matches_oracle(engine_mod, oracle_mod, name, tmp_path):
    ini = configs.write_ini(str(tmp_path / "r.ini"), name, "/tmp/x")
    mine = engine_mod.load_mesh_host(engine_mod.load_ini(ini))
    o = oracle_mod.Oracle.from_files(oracle_mod.parse_ini(ini))
    for k, ok in ORACLE_FIELDS.items():
        np.testing.assert_array_equal(mine[k], o.field(ok), err_msg=k)


def test_loader_rejects_bad_inputs(engine_mod, oracle_mod, tmp_path):
    ini = configs.write_ini(str(tmp_path / "r.ini"), "perstep_nucl", "/tmp/x")
    opt = engine_mod.load_ini(ini)
    opt.n_grains = 299                       # src/io.h:182-186 grain-count check
    with pytest.raises(engine_mod.SevcError) as e:
        engine_mod.load_mesh_host(opt)
    assert e.value.code == 2
    opt = engine_mod.load_ini(ini)
    opt.vertex_fname = str(tmp_path / "missing.txt").encode()
    with pytest.raises(engine_mod.SevcError) as e:
        engine_mod.load_mesh_host(opt)
    assert e.value.code == 1


@pytest.mark.parametrize("n,seed", [(50, 1), (777, 2), (5000, 3)])
def test_meshgen_builds_valid_periodic_meshes(oracle_mod, n, seed):
    import meshgen
    inp = meshgen.make_inputs(n, seed)
    assert inp["xy"].shape == (2 * n, 2) and inp["ridges"].shape == (3 * n, 2)
    assert inp["xy"].min() >= 0 and inp["xy"].max() < 1
    deg = np.bincount(inp["ridges"].ravel(), minlength=2 * n)
    assert np.all(deg == 3)
    opt = oracle_mod.finish_options(oracle_mod.default_options(n_grains=n, dt=1e-3, dtau=1e-3, domain_bound=1.0))
    o = oracle_mod.Oracle.from_arrays(opt, inp["xy"], inp["ridges"], inp["oris"], inp["se"])
    assert o.check_data() == 0
    oracle_mod.lib().orc_compute_grain_areas(o._p)
    assert abs(o.field("garea").sum() - 1.0) < 1e-9


def test_meshgen_file_roundtrip(engine_mod, tmp_path):
    import meshgen
    inp = meshgen.make_inputs(64, 5)
    paths = meshgen.write_files(str(tmp_path), inp)
    back = meshgen.read_files(paths["vertices"], paths["ridges"], paths["oris"], paths["se"])
    np.testing.assert_array_equal(back["ridges"], inp["ridges"])
    np.testing.assert_allclose(back["xy"], inp["xy"], rtol=0, atol=1e-16)  # %.16f keeps 16 decimals
    opt = engine_mod.default_options(n_grains=64, dt=1e-3, dtau=1e-3, vertex_fname=paths["vertices"],
                                     boundary_fname=paths["ridges"], orientation_fname=paths["oris"],
                                     SE_fname=paths["se"])
    m = engine_mod.load_mesh_host(opt)
    assert m["gvlen"].sum() == 3 * 128


def test_check_data_flags_planted_faults(oracle_mod, tmp_path):
    ini = configs.write_ini(str(tmp_path / "r.ini"), "perstep_nucl", "/tmp/x")
    o = oracle_mod.Oracle.from_files(oracle_mod.parse_ini(ini))
    assert o.check_data() == 0
    o.field("bend")[5] = o.field("bini")[5]          # a self-loop boundary
    assert o.check_data() > 0
    o2 = oracle_mod.Oracle.from_files(oracle_mod.parse_ini(ini))
    o2.field("gvlen")[3] -= 1                          # list length no longer matches
    assert o2.check_data() > 0


def test_synthetic_stream_range():
    import ctypes
    from oracle import oracle as O
    o = O.Oracle.from_files(O.parse_ini(configs.write_ini("/tmp/_s.ini", "perstep_nucl", "/tmp/x")))
    o.rng_synthetic(5)
    pos = o.field("rng_pos")
    assert pos.shape == (8192,) and pos.max() == 0


def test_fixed16_formatter_matches_printf(engine_mod):
    """The snapshot number writer equals printf("%.16f") (the C library's
    and Python's, both correctly rounded) on random doubles of every scale,
    exact decimal ties, signed zeros, subnormals and large values."""
    import ctypes
    import numpy as np
    libc = ctypes.CDLL(None)
    buf = ctypes.create_string_buffer(128)

    def c_printf(x):
        n = libc.snprintf(buf, 128, b"%.16f", ctypes.c_double(x))
        return buf.raw[:n].decode()

    rng = np.random.default_rng(0)
    vals = list(rng.uniform(-1, 1, 20000) * 10.0 ** rng.integers(-20, 22, 20000))
    vals += list(rng.uniform(0, 1000, 5000)) + list(rng.standard_normal(5000) * 1e-8)
    vals += [0.0, -0.0, 5e-324, -5e-324, 2.0 ** -17, 3 * 2.0 ** -17, 2.0 ** -18, 0.5e-16, 1.5e-16, 2.5e-16,
             100000.0, 99999.99999999999, 1e21, -1e21, 2.0 ** 72, 9.3e21, 1 / 3, 2 / 3, 0.1, 1e-17, 5e-17,
             float(np.nextafter(5e-17, 1)), float(np.nextafter(5e-17, 0))]
    vals += [k * 2.0 ** -20 for k in range(1, 4000, 7)]         # many exact decimal ties
    for x in vals:
        got = engine_mod.format_fixed16(x)
        assert got == c_printf(x) == "%.16f" % x, (x, got, c_printf(x))


def test_host_check_counts_planted_faults(engine_mod, tmp_path):
    """check_data's host restatement: a freshly loaded mesh has no violation,
    each planted fault is counted."""
    import numpy as np
    import meshgen
    from test_gpu_check import plant
    mesh = meshgen.make_inputs(200, 3)
    p = meshgen.write_files(str(tmp_path), mesh)
    o = engine_mod.default_options(n_grains=200, domain_bound=1.0, vertex_fname=p["vertices"],
                                   boundary_fname=p["ridges"], orientation_fname=p["oris"], SE_fname=p["se"])
    st = engine_mod.load_mesh_host(o)
    assert engine_mod.check_mesh_host(st) == 0
    rng = np.random.default_rng(0)
    for kind in ["boundary_off", "dup_boundary_slot", "dup_grain_slot", "self_loop", "short_list", "grain_off",
                 "vertex_off", "foreign_grain"]:
        assert engine_mod.check_mesh_host(plant(st, kind, rng)) > 0, kind


@pytest.mark.parametrize("name", ["plain_unit", "perstep_nucl"])
def test_snapshot_writer_matches_oracle_export(engine_mod, oracle_mod, name, tmp_path):
    """The library's snapshot writer (chunks formatted by all host threads,
    written in order) gives the oracle's printf export byte for byte, here
    for the freshly loaded mesh (no GPU needed)."""
    ini = configs.write_ini(str(tmp_path / "r.ini"), name, str(tmp_path / "out"))
    opt = engine_mod.load_ini(ini)
    mine = engine_mod.load_mesh_host(opt)
    a, b = str(tmp_path / "lib.txt"), str(tmp_path / "orc.txt")
    engine_mod.write_snapshot(mine, opt, a, 0.0)
    o = oracle_mod.Oracle.from_files(oracle_mod.parse_ini(ini))
    o.export(b, 0.0)
    assert open(a, "rb").read() == open(b, "rb").read()
