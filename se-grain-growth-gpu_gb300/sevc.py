"""Python binding of the engine's C ABI (include/sevc.h), over ctypes.

This is a thin host-side mirror for tests, benchmarks and scripting: every
call goes through libsevc.so, built in-tree by build.py.  There is no CPU
fallback; importing works without a GPU, but every compute call raises
SevcError when no CUDA device is present.
"""
import ctypes as C
import os

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libsevc.so")
MAXV = 100

STATUS = {0: "OK", 1: "IO", 2: "PARSE", 3: "CAPACITY", 4: "NONCONVERGED", 5: "TOPOLOGY", 6: "CUDA", 7: "ARG"}

# every symbol include/sevc.h declares
EXPORTS = ["sevc_default_options", "sevc_load_ini", "sevc_create", "sevc_create_from_arrays", "sevc_destroy", "sevc_load_mesh_host",
           "sevc_step", "sevc_run_steps", "sevc_run", "sevc_should_continue", "sevc_export_text", "sevc_get_state",
           "sevc_mesh_sizes", "sevc_check_data", "sevc_run_program", "sevc_rng_record", "sevc_set_profiling",
           "sevc_get_profile", "sevc_last_error", "sevc_set_exact_all", "sevc_rng_record_noalloc",
           "sevc_create_batch", "sevc_instance_count", "sevc_instance_ranges", "sevc_instance_info",
           "sevc_export_instance_text", "sevc_set_mobility", "sevc_set_gb_scaling", "sevc_set_stored_energy",
           "sevc_tape_start", "sevc_tape_stop", "sevc_area_histogram", "sevc_adjoint_histogram",
           "sevc_checkpoint_save", "sevc_checkpoint_load", "sevc_grain_stats", "sevc_format_fixed16",
           "sevc_check_data_host", "sevc_check_mesh", "sevc_set_graphs", "sevc_measure_fp64_rate",
           "sevc_autotune", "sevc_selftest_arith", "sevc_write_snapshot", "sevc_state_digest", "sevc_set_limits",
           "sevc_voronoi_generate", "sevc_voronoi_write"]


class SevcError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("sevc error %d (%s): %s" % (code, STATUS.get(code, "?"), msg))
        self.code = code


class Options(C.Structure):
    """sevc_options (src/options.h:15-46 + min_grains)."""
    _fields_ = [
        ("dt", C.c_double), ("dtau", C.c_double), ("nucleation_gap", C.c_int), ("tmax", C.c_double),
        ("nmax", C.c_int), ("snap_gap", C.c_int), ("leave_percent", C.c_double), ("n_grains", C.c_int),
        ("vertex_fname", C.c_char * 256), ("boundary_fname", C.c_char * 256),
        ("orientation_fname", C.c_char * 256), ("SE_fname", C.c_char * 256),
        ("GB_eps", C.c_double), ("GB_scaling", C.c_double), ("SE_eps", C.c_double), ("SE_min", C.c_double),
        ("SE_max", C.c_double), ("nucleation_scaling", C.c_double), ("domain_bound", C.c_double),
        ("do_nucleation", C.c_int), ("MC_k", C.c_double), ("n_blocks", C.c_int), ("n_threads", C.c_int),
        ("debug_lvl", C.c_int), ("output_folder", C.c_char * 256), ("min_grains", C.c_int),
    ]


_MESH_FIELDS = [
    ("px", "v", np.float64), ("py", "v", np.float64), ("vx", "v", np.float64), ("vy", "v", np.float64),
    ("venergy", "v", np.float64), ("vel_bnd_x", "v", np.float64), ("vel_grn_x", "v", np.float64),
    ("vel_bnd_y", "v", np.float64), ("vel_grn_y", "v", np.float64), ("ven", "v", np.uint8),
    ("vb", "v3", np.int32), ("vg", "v3", np.int32), ("bini", "b", np.int32), ("bend", "b", np.int32),
    ("benergy", "b", np.float64), ("blen", "b", np.float64), ("btext", "b", np.float64), ("ben", "b", np.uint8),
    ("bcand", "b", np.uint8), ("glist", "g100", np.int32), ("gvlen", "g", np.int32), ("garea", "g", np.float64),
    ("gdadt", "g", np.float64), ("gori", "g", np.float64), ("gse", "g", np.float64), ("gen", "g", np.uint8),
    ("gtype", "g", np.uint8),
]


class MeshHost(C.Structure):
    _fields_ = [("nv", C.c_int), ("nb", C.c_int), ("ng", C.c_int)] + [(f, C.c_void_p) for f, _, _ in _MESH_FIELDS]


class GrainStats(C.Structure):
    _fields_ = [("n_grains", C.c_int), ("n_three_sided", C.c_int), ("mean_area", C.c_double),
                ("std_area", C.c_double), ("min_area", C.c_double), ("max_area", C.c_double),
                ("mean_sides", C.c_double)]


class StepInfo(C.Structure):
    _fields_ = [
        ("n", C.c_int), ("t", C.c_double), ("curr_n_grains", C.c_int), ("nucleated_area", C.c_double),
        ("export_due", C.c_int), ("keep_going", C.c_int), ("polling_iters", C.c_int),
        ("n_two_three_iters", C.c_int), ("two_three_counts", C.c_int * 20), ("n_flips", C.c_int),
        ("n_removals", C.c_int), ("n_two_three", C.c_int), ("n_nucleations", C.c_int),
        ("nucleation_attempted", C.c_int), ("nucleation_candidate", C.c_int), ("gpu_ms", C.c_double),
        ("outputs_complete", C.c_int), ("kernel_launches", C.c_int), ("n_conflicts", C.c_int),
    ]

    def as_dict(self):
        d = {k: getattr(self, k) for k, _ in self._fields_}
        d["two_three_counts"] = list(self.two_three_counts)[: self.n_two_three_iters]
        return d


_lib = None


def lib():
    """Load the in-tree libsevc.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise OSError("libsevc.so is not built: run __graft_entry__.build()")
        L = C.CDLL(LIB_PATH)
        H = C.c_void_p
        L.sevc_default_options.argtypes = [C.POINTER(Options)]
        L.sevc_load_ini.argtypes = [C.c_char_p, C.POINTER(Options)]
        L.sevc_create.argtypes = [C.POINTER(Options), C.POINTER(H)]
        L.sevc_create_from_arrays.argtypes = [C.POINTER(Options), C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_int,
                                              C.c_void_p, C.c_void_p, C.POINTER(H)]
        L.sevc_destroy.argtypes = [H]
        L.sevc_destroy.restype = None
        L.sevc_step.argtypes = [H, C.POINTER(StepInfo)]
        L.sevc_run_steps.argtypes = [H, C.c_int, C.POINTER(C.c_int), C.POINTER(StepInfo)]
        L.sevc_run.argtypes = [H, C.c_int, C.POINTER(StepInfo), C.POINTER(C.c_int)]
        L.sevc_should_continue.argtypes = [H]
        L.sevc_export_text.argtypes = [H, C.c_char_p, C.c_double]
        L.sevc_get_state.argtypes = [H, C.POINTER(MeshHost)]
        L.sevc_mesh_sizes.argtypes = [H, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int)]
        L.sevc_check_data.argtypes = [H, C.POINTER(C.c_int)]
        L.sevc_run_program.argtypes = [C.POINTER(Options), C.c_int]
        L.sevc_rng_record.argtypes = [C.c_int, C.c_int, C.c_void_p]
        L.sevc_set_profiling.argtypes = [H, C.c_int]
        L.sevc_get_profile.argtypes = [H, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(C.c_int)]
        L.sevc_last_error.restype = C.c_char_p
        _lib = L
    return _lib


def _check(rc):
    if rc:
        raise SevcError(rc, lib().sevc_last_error().decode(errors="replace"))


def default_options(**kw):
    o = Options()
    _check(lib().sevc_default_options(C.byref(o)))
    for k, v in kw.items():
        setattr(o, k, v.encode() if isinstance(v, str) else v)
    return o


def load_ini(path):
    o = Options()
    _check(lib().sevc_load_ini(path.encode(), C.byref(o)))
    return o


def load_mesh_host(opt):
    """Host-only loader (src/io.h:66-264): the mesh as numpy arrays."""
    L = lib()
    L.sevc_load_mesh_host.argtypes = [C.POINTER(Options), C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                      C.POINTER(C.c_int)]
    nv, nb, ng = C.c_int(), C.c_int(), C.c_int()
    _check(L.sevc_load_mesh_host(C.byref(opt), None, C.byref(nv), C.byref(nb), C.byref(ng)))
    sizes = {"v": nv.value, "v3": 3 * nv.value, "b": nb.value, "g": ng.value, "g100": MAXV * ng.value}
    arrs = {f: np.empty(sizes[k], dt) for f, k, dt in _MESH_FIELDS}
    mh = MeshHost(nv.value, nb.value, ng.value, *[arrs[f].ctypes.data for f, _, _ in _MESH_FIELDS])
    _check(L.sevc_load_mesh_host(C.byref(opt), C.byref(mh), None, None, None))
    return arrs


def mesh_host_of(arrs):
    """A MeshHost view of a dict of arrays (keys of get_state)."""
    nv, nb, ng = len(arrs["px"]), len(arrs["bini"]), len(arrs["gvlen"])
    return MeshHost(nv, nb, ng, *[np.ascontiguousarray(arrs[f]).ctypes.data for f, _, _ in _MESH_FIELDS])


def check_mesh(arrs):
    """check_data's violation count of a host mesh, counted on the device."""
    arrs = {f: np.ascontiguousarray(arrs[f], dt) for f, _, dt in _MESH_FIELDS}
    mh = mesh_host_of(arrs)
    n = C.c_int()
    L = lib()
    L.sevc_check_mesh.argtypes = [C.POINTER(MeshHost), C.POINTER(C.c_int)]
    _check(L.sevc_check_mesh(C.byref(mh), C.byref(n)))
    return n.value


def check_mesh_host(arrs):
    """The same count by the host restatement (no GPU)."""
    arrs = {f: np.ascontiguousarray(arrs[f], dt) for f, _, dt in _MESH_FIELDS}
    mh = mesh_host_of(arrs)
    L = lib()
    L.sevc_host_check.argtypes = [C.POINTER(MeshHost)]
    return int(L.sevc_host_check(C.byref(mh)))


def write_snapshot(arrs, opt, path, time):
    """The snapshot text (src/io.h:280-377) of a mesh held in host arrays
    (keys of get_state / load_mesh_host); host only."""
    arrs = {f: np.ascontiguousarray(arrs[f], dt) for f, _, dt in _MESH_FIELDS}
    mh = mesh_host_of(arrs)
    L = lib()
    L.sevc_write_snapshot.argtypes = [C.POINTER(MeshHost), C.POINTER(Options), C.c_char_p, C.c_double]
    _check(L.sevc_write_snapshot(C.byref(mh), C.byref(opt), path.encode(), float(time)))


def voronoi(n, seed, se_dist="uniform"):
    """Periodic Voronoi input of n grains from the library's C generator
    (sevc_voronoi_generate, voronoi.py's job): dict with xy (2n x 2),
    ridges (3n x 2), oris and se (n each; se U[0,1) or triangular(3,6,6))."""
    L = lib()
    L.sevc_voronoi_generate.argtypes = [C.c_int, C.c_uint64, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                        C.c_void_p]
    xy, ridges = np.empty((2 * n, 2)), np.empty((3 * n, 2), np.int32)
    oris, se = np.empty(n), np.empty(n)
    _check(L.sevc_voronoi_generate(n, seed, 1 if se_dist == "triangular" else 0, xy.ctypes.data, ridges.ctypes.data,
                                   oris.ctypes.data, se.ctypes.data))
    return {"xy": xy, "ridges": ridges, "oris": oris, "se": se, "n_grains": n}


def voronoi_write(inp, vertices, ridges, oris, se):
    """The four input files (voronoi.py's formats) of a voronoi() result."""
    L = lib()
    L.sevc_voronoi_write.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p] + [C.c_char_p] * 4
    a = {k: np.ascontiguousarray(inp[k]) for k in ("xy", "ridges", "oris", "se")}
    _check(L.sevc_voronoi_write(len(a["oris"]), a["xy"].ctypes.data, a["ridges"].ctypes.data, a["oris"].ctypes.data,
                                a["se"].ctypes.data, vertices.encode(), ridges.encode(), oris.encode(), se.encode()))


def measure_fp64_rate():
    """FP64 multiply-add thread operations per second of the current GPU."""
    r = C.c_double()
    L = lib()
    L.sevc_measure_fp64_rate.argtypes = [C.POINTER(C.c_double)]
    _check(L.sevc_measure_fp64_rate(C.byref(r)))
    return r.value


def selftest_arith(n, seed=1):
    """Bit-for-bit check of the certified division / square root behind
    the arclengths against the native operations on n random cases; a dict
    of the counts sevc_selftest_arith returns."""
    c = (C.c_longlong * 8)()
    L = lib()
    L.sevc_selftest_arith.argtypes = [C.c_longlong, C.c_ulonglong, C.POINTER(C.c_longlong)]
    _check(L.sevc_selftest_arith(int(n), int(seed), c))
    keys = ["div", "div_mismatch", "div_uncertified", "sqrt", "sqrt_mismatch", "sqrt_uncertified", "vmag",
            "vmag_mismatch"]
    return dict(zip(keys, list(c)))


def format_fixed16(x):
    """The snapshot writer's number text (printf "%.16f")."""
    buf = C.create_string_buffer(64)
    L = lib()
    L.sevc_format_fixed16.argtypes = [C.c_double, C.c_char_p]
    n = L.sevc_format_fixed16(float(x), buf)
    return buf.raw[:n].decode()


def rng_record(nstreams, ndraws):
    """First `ndraws` cuRAND draws of streams curand_init(32, tid, 0)."""
    out = np.empty((nstreams, ndraws), np.float64)
    _check(lib().sevc_rng_record(nstreams, ndraws, out.ctypes.data))
    return out


def rng_record_noalloc(nstreams, ndraws, d_out, stream=None):
    """Allocation-free record into caller-owned DEVICE memory `d_out`
    (an integer device address); asynchronous on `stream`."""
    L = lib()
    L.sevc_rng_record_noalloc.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_void_p]
    _check(L.sevc_rng_record_noalloc(nstreams, ndraws, C.c_void_p(d_out), C.c_void_p(stream)))


# fields of sevc_state_digest, in order (include/sevc.h)
DIGEST_FIELDS = ("px", "py", "vx", "vy", "ven", "vb", "vg", "bini", "bend", "benergy", "blen", "ben", "bcand",
                 "glist", "gvlen", "garea", "gori", "gse", "gen", "gtype")


class Engine:
    """One simulation on the GPU (an sevc_handle)."""

    def __init__(self, handle, opt):
        self._h = handle
        self.opt = opt
        nv, nb, ng = C.c_int(), C.c_int(), C.c_int()
        _check(lib().sevc_mesh_sizes(self._h, C.byref(nv), C.byref(nb), C.byref(ng)))
        self.nv, self.nb, self.ng = nv.value, nb.value, ng.value

    @classmethod
    def from_files(cls, opt):
        h = C.c_void_p()
        _check(lib().sevc_create(C.byref(opt), C.byref(h)))
        return cls(h, opt)

    @classmethod
    def from_arrays(cls, opt, xy, ridges, oris, se):
        xy = np.ascontiguousarray(xy, np.float64)
        ridges = np.ascontiguousarray(ridges, np.int32)
        oris = np.ascontiguousarray(oris, np.float64)
        se = np.ascontiguousarray(se, np.float64)
        h = C.c_void_p()
        _check(lib().sevc_create_from_arrays(C.byref(opt), len(xy), xy.ctypes.data, len(ridges), ridges.ctypes.data,
                                             len(oris), oris.ctypes.data, se.ctypes.data, C.byref(h)))
        return cls(h, opt)

    @classmethod
    def from_batch(cls, opt, meshes):
        """A batched handle over `meshes`, each a dict with xy, ridges, oris, se
        (the arrays of from_arrays)."""
        n = len(meshes)
        xy = [np.ascontiguousarray(m["xy"], np.float64) for m in meshes]
        rd = [np.ascontiguousarray(m["ridges"], np.int32) for m in meshes]
        ori = [np.ascontiguousarray(m["oris"], np.float64) for m in meshes]
        se = [np.ascontiguousarray(m["se"], np.float64) for m in meshes]
        ints = lambda v: (C.c_int * n)(*v)
        ptrs = lambda arrs: (C.c_void_p * n)(*[a.ctypes.data for a in arrs])
        L = lib()
        L.sevc_create_batch.argtypes = [C.POINTER(Options), C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                        C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(C.c_void_p)]
        h = C.c_void_p()
        _check(L.sevc_create_batch(C.byref(opt), n, ints([len(a) for a in xy]), ptrs(xy), ints([len(a) for a in rd]),
                                   ptrs(rd), ints([len(a) for a in ori]), ptrs(ori), ptrs(se), C.byref(h)))
        eng = cls(h, opt)
        eng._keep = (xy, rd, ori, se)
        return eng

    def instance_count(self):
        n = C.c_int()
        lib().sevc_instance_count.argtypes = [C.c_void_p, C.POINTER(C.c_int)]
        _check(lib().sevc_instance_count(self._h, C.byref(n)))
        return n.value

    def instance_ranges(self):
        """(voff, boff, goff), each ninst+1 int32 offsets."""
        n = self.instance_count()
        out = [np.zeros(n + 1, np.int32) for _ in range(3)]
        lib().sevc_instance_ranges.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        _check(lib().sevc_instance_ranges(self._h, *[a.ctypes.data for a in out]))
        return tuple(out)

    def instance_info(self, inst):
        info = StepInfo()
        lib().sevc_instance_info.argtypes = [C.c_void_p, C.c_int, C.POINTER(StepInfo)]
        _check(lib().sevc_instance_info(self._h, inst, C.byref(info)))
        return info

    def export_instance(self, inst, path, time):
        lib().sevc_export_instance_text.argtypes = [C.c_void_p, C.c_int, C.c_char_p, C.c_double]
        _check(lib().sevc_export_instance_text(self._h, inst, path.encode(), time))

    def instance_state(self, state, inst):
        """Instance `inst`'s part of a get_state() dict, in its own indices."""
        vo, bo, go = self.instance_ranges()
        v0, v1, b0, b1, g0, g1 = vo[inst], vo[inst + 1], bo[inst], bo[inst + 1], go[inst], go[inst + 1]
        sl = {"v": slice(v0, v1), "v3": slice(3 * v0, 3 * v1), "b": slice(b0, b1), "g": slice(g0, g1),
              "g100": slice(MAXV * g0, MAXV * g1)}
        shift = {"vb": b0, "vg": g0, "bini": v0, "bend": v0, "glist": v0}
        out = {}
        for f, k, _ in _MESH_FIELDS:
            a = state[f][sl[k]].copy()
            if f in shift:
                a = np.where(a >= 0, a - shift[f], a)
            out[f] = a
        return out

    def close(self):
        if self._h:
            lib().sevc_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def step(self):
        info = StepInfo()
        _check(lib().sevc_step(self._h, C.byref(info)))
        return info

    def run(self, n):
        """n steps (sevc_run: pipelined when the handle allows it); the list
        of their StepInfo"""
        infos = (StepInfo * max(n, 1))()
        done = C.c_int(0)
        rc = lib().sevc_run(self._h, n, infos, C.byref(done))
        out = [infos[k] for k in range(done.value)]
        _check(rc)
        return out

    def run_steps(self, n):
        info, done = StepInfo(), C.c_int()
        _check(lib().sevc_run_steps(self._h, n, C.byref(done), C.byref(info)))
        return done.value, info

    def should_continue(self):
        return bool(lib().sevc_should_continue(self._h))

    def export(self, path, time):
        _check(lib().sevc_export_text(self._h, path.encode(), time))

    def check_data(self):
        n = C.c_int()
        _check(lib().sevc_check_data(self._h, C.byref(n)))
        return n.value

    def check_data_host(self):
        n = C.c_int()
        lib().sevc_check_data_host.argtypes = [C.c_void_p, C.POINTER(C.c_int)]
        _check(lib().sevc_check_data_host(self._h, C.byref(n)))
        return n.value

    def get_state(self):
        """Full mesh as numpy arrays (keys as in sevc_mesh_host)."""
        sizes = {"v": self.nv, "v3": 3 * self.nv, "b": self.nb, "g": self.ng, "g100": MAXV * self.ng}
        arrs = {f: np.empty(sizes[k], dt) for f, k, dt in _MESH_FIELDS}
        mh = MeshHost(self.nv, self.nb, self.ng, *[arrs[f].ctypes.data for f, _, _ in _MESH_FIELDS])
        _check(lib().sevc_get_state(self._h, C.byref(mh)))
        return arrs

    def state_digest(self):
        """Per-field digests of the state computed on the device
        (sevc_state_digest), as a tuple of DIGEST_FIELDS Python ints."""
        out = (C.c_uint64 * len(DIGEST_FIELDS))()
        lib().sevc_state_digest.argtypes = [C.c_void_p, C.c_void_p]
        _check(lib().sevc_state_digest(self._h, out))
        return tuple(int(x) for x in out)

    # ---- checkpoint files, statistics ----
    def checkpoint_save(self, path):
        lib().sevc_checkpoint_save.argtypes = [C.c_void_p, C.c_char_p]
        _check(lib().sevc_checkpoint_save(self._h, path.encode()))

    def checkpoint_load(self, path):
        lib().sevc_checkpoint_load.argtypes = [C.c_void_p, C.c_char_p]
        _check(lib().sevc_checkpoint_load(self._h, path.encode()))

    def grain_stats(self, inst=-1):
        s = GrainStats()
        lib().sevc_grain_stats.argtypes = [C.c_void_p, C.c_int, C.POINTER(GrainStats)]
        _check(lib().sevc_grain_stats(self._h, inst, C.byref(s)))
        return {f: getattr(s, f) for f, _ in GrainStats._fields_}

    # ---- parameters and the adjoint ----
    def set_mobility(self, mu):
        lib().sevc_set_mobility.argtypes = [C.c_void_p, C.c_double]
        _check(lib().sevc_set_mobility(self._h, float(mu)))

    def set_gb_scaling(self, s):
        lib().sevc_set_gb_scaling.argtypes = [C.c_void_p, C.c_double]
        _check(lib().sevc_set_gb_scaling(self._h, float(s)))

    def set_stored_energy(self, se):
        se = np.ascontiguousarray(se, np.float64)
        assert se.shape == (self.ng,)
        lib().sevc_set_stored_energy.argtypes = [C.c_void_p, C.c_void_p]
        _check(lib().sevc_set_stored_energy(self._h, se.ctypes.data))

    def tape_start(self, checkpoint_every):
        lib().sevc_tape_start.argtypes = [C.c_void_p, C.c_int]
        _check(lib().sevc_tape_start(self._h, int(checkpoint_every)))

    def tape_stop(self):
        lib().sevc_tape_stop.argtypes = [C.c_void_p]
        _check(lib().sevc_tape_stop(self._h))

    def area_histogram(self, nbins, amax):
        out = np.zeros(nbins)
        lib().sevc_area_histogram.argtypes = [C.c_void_p, C.c_int, C.c_double, C.c_void_p]
        _check(lib().sevc_area_histogram(self._h, nbins, float(amax), out.ctypes.data))
        return out

    def adjoint_histogram(self, nbins, amax, dloss_dhist):
        """(dloss/dSE per grain, dloss/dGB_scaling, dloss/dmu) for the taped steps."""
        d = np.ascontiguousarray(dloss_dhist, np.float64)
        assert d.shape == (nbins,)
        gse = np.zeros(self.ng)
        ggb, gmu = C.c_double(), C.c_double()
        lib().sevc_adjoint_histogram.argtypes = [C.c_void_p, C.c_int, C.c_double, C.c_void_p, C.c_void_p,
                                                 C.POINTER(C.c_double), C.POINTER(C.c_double)]
        _check(lib().sevc_adjoint_histogram(self._h, nbins, float(amax), d.ctypes.data, gse.ctypes.data,
                                            C.byref(ggb), C.byref(gmu)))
        return gse, ggb.value, gmu.value

    def set_limits(self, polling_cap=0, worklist_cap=0):
        lib().sevc_set_limits.argtypes = [C.c_void_p, C.c_int, C.c_int]
        _check(lib().sevc_set_limits(self._h, polling_cap, worklist_cap))

    def set_exact_all(self, on):
        lib().sevc_set_exact_all.argtypes = [C.c_void_p, C.c_int]
        _check(lib().sevc_set_exact_all(self._h, 1 if on else 0))

    def autotune(self, steps=5):
        """Pick launch shapes by timing; returns (tpb_vertex, tpb_boundary,
        wide_sides, grain_occ)."""
        out = (C.c_int * 4)()
        lib().sevc_autotune.argtypes = [C.c_void_p, C.c_int, C.c_void_p]
        _check(lib().sevc_autotune(self._h, steps, out))
        return tuple(out)

    def set_graphs(self, on):
        lib().sevc_set_graphs.argtypes = [C.c_void_p, C.c_int]
        _check(lib().sevc_set_graphs(self._h, int(on) if not isinstance(on, bool) else (1 if on else 0)))

    def set_profiling(self, on):
        _check(lib().sevc_set_profiling(self._h, 1 if on else 0))

    def profile(self):
        cap = 64
        names = (C.c_char * 48 * cap)()
        ms = np.zeros(cap)
        launches = np.zeros(cap, np.int64)
        n = C.c_int()
        _check(lib().sevc_get_profile(self._h, cap, names, ms.ctypes.data, launches.ctypes.data, C.byref(n)))
        return {names[i].value.decode(): (float(ms[i]), int(launches[i])) for i in range(min(n.value, cap))}
