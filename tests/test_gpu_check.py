"""check_data on the device counts exactly what the host restatement counts:
on meshes in the middle of runs (no violation) and on meshes with planted
faults (indices kept inside their arrays)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def opts(sevc, n):
    o = sevc.default_options(n_grains=n, dt=4e-3, dtau=4e-3, nucleation_gap=1, domain_bound=17.0, GB_eps=0.0,
                             GB_scaling=1.0, SE_eps=1.0, SE_min=999.0, SE_max=999.0, do_nucleation=0,
                             nmax=10 ** 8, tmax=-1, snap_gap=10 ** 8, n_blocks=32, n_threads=256)
    o.min_grains = -1
    return o


def plant(st, kind, rng):
    s = {k: v.copy() for k, v in st.items()}
    ven = np.nonzero(s["ven"])[0]
    v = int(rng.choice(ven))
    gen = np.nonzero(s["gen"])[0]
    g = int(rng.choice(gen))
    b = int(s["vb"][3 * v])
    if kind == "boundary_off":
        s["ben"][b] = 0
    elif kind == "dup_boundary_slot":
        s["vb"][3 * v + 1] = s["vb"][3 * v]
    elif kind == "dup_grain_slot":
        s["vg"][3 * v + 2] = s["vg"][3 * v]
    elif kind == "self_loop":
        s["bend"][b] = s["bini"][b]
    elif kind == "short_list":
        n = s["gvlen"][g]
        s["glist"][100 * g + n - 1] = -1
    elif kind == "grain_off":
        s["gen"][g] = 0
    elif kind == "vertex_off":
        s["ven"][v] = 0
    elif kind == "foreign_grain":
        others = [x for x in gen if x not in s["vg"][3 * v:3 * v + 3]]
        s["vg"][3 * v] = int(others[0])
    return s


def test_device_check_matches_host(gpu):
    import meshgen
    mesh = meshgen.make_inputs(600, 8, se="triangular")
    e = gpu.Engine.from_arrays(opts(gpu, 600), mesh["xy"], mesh["ridges"], mesh["oris"], mesh["se"])
    events = 0
    for k in range(120):
        i = e.step()
        events += i.n_flips + i.n_removals
        if k % 30 == 29:
            assert e.check_data() == e.check_data_host() == 0
    assert events > 0
    st = e.get_state()
    assert gpu.check_mesh(st) == gpu.check_mesh_host(st) == 0
    rng = np.random.default_rng(4)
    kinds = ["boundary_off", "dup_boundary_slot", "dup_grain_slot", "self_loop", "short_list", "grain_off",
             "vertex_off", "foreign_grain"]
    for kind in kinds:
        for _ in range(3):
            bad = plant(st, kind, rng)
            d, h = gpu.check_mesh(bad), gpu.check_mesh_host(bad)
            assert d == h and d > 0, (kind, d, h)
    e.close()


def test_certified_division_and_sqrt_are_correctly_rounded(gpu):
    """Every arclength divides and takes a square root with the certified
    fast operations; on 2^26 random cases (general operands, quotients and
    roots next to rounding midpoints, special operands) each certified
    result, and each whole vector2_mag, equals the native operation bit for
    bit, and only a small share falls back to the native path."""
    for seed in (1, 2):
        c = gpu.selftest_arith(1 << 26, seed=seed)
        assert c["div"] == c["sqrt"] == c["vmag"] == 1 << 26
        assert c["div_mismatch"] == 0 and c["sqrt_mismatch"] == 0 and c["vmag_mismatch"] == 0, c
        assert c["div_uncertified"] < 0.1 * c["div"] and c["sqrt_uncertified"] < 0.1 * c["sqrt"], c
