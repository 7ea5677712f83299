"""ctypes binding of the C oracle (TEST INFRASTRUCTURE ONLY).

Only tests/, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this module, to compare results against and to time
the host baseline.  The product (the CUDA library and its C ABI) never
loads the oracle.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
SRC = [os.path.join(HERE, "sevc_oracle.c")]

ORC_OK, ORC_ERR_IO, ORC_ERR_PARSE, ORC_ERR_CAPACITY, ORC_ERR_NONCONVERGED, ORC_ERR_TOPOLOGY, ORC_ERR_RNG = range(7)


def build(force=False):
    """Compile liboracle.so (gcc, no FMA contraction, OpenMP)."""
    newest = max(os.path.getmtime(p) for p in SRC + [os.path.join(HERE, "sevc_oracle.h"),
                                                      os.path.join(HERE, "synth_rng.h")])
    if not force and os.path.exists(LIB_PATH) and os.path.getmtime(LIB_PATH) >= newest:
        return LIB_PATH
    tmp = LIB_PATH + ".tmp%d" % os.getpid()
    subprocess.check_call(["gcc", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fopenmp", "-fPIC",
                           "-shared", "-o", tmp] + SRC + ["-lm"])
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


class Options(C.Structure):
    """struct orc_options (mirrors src/options.h:15-46)."""
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


class _State(C.Structure):
    _fields_ = [("opt", Options), ("nv", C.c_int), ("nb", C.c_int), ("ng", C.c_int)] + \
        [(n, C.c_void_p) for n in (
            "px py vx vy venergy vel_bnd_x vel_grn_x vel_bnd_y vel_grn_y nucl_r nucl_ori DeltaE nfactor "
            "ven vnucleate vb vg vmod voted bini bend benergy blen btext ben bcand bvotes bconf "
            "glist gvlen garea gdadt gori gse gen gcand gfix gtype").split()] + [
        ("n", C.c_int), ("prog", C.c_int), ("curr_n_grains", C.c_int), ("allow_nucleation", C.c_int),
        ("t", C.c_double), ("nucleated_area", C.c_double), ("cand_buf", C.c_void_p),
        ("vrt_id_candidate", C.c_int), ("vertex_buffer", C.c_int * 64), ("vrt_ids", C.c_int * 2),
        ("bnd_ids", C.c_int * 3), ("grn_id", C.c_int), ("polling_iters", C.c_int), ("polling_cap", C.c_int),
        ("last_two_three", C.c_int * 20), ("n_two_three_iters", C.c_int),
        ("rng_kind", C.c_int), ("rng_seed", C.c_uint64), ("rng_nstreams", C.c_int), ("rng_ndraws", C.c_int),
        ("rng_table", C.c_void_p), ("rng_pos", C.c_void_p),
        ("ev_flips", C.c_int), ("ev_removals", C.c_int), ("ev_two_three", C.c_int), ("ev_nucleations", C.c_int),
        ("status", C.c_int), ("nthreads_omp", C.c_int), ("ev_conflicts", C.c_int),
    ]


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        P = C.POINTER(_State)
        L.orc_parse_ini.argtypes = [C.c_char_p, C.POINTER(Options)]
        L.orc_default_options.argtypes = [C.POINTER(Options)]
        L.orc_finish_options.argtypes = [C.POINTER(Options)]
        L.orc_load_files.argtypes = [C.POINTER(Options), C.POINTER(P)]
        L.orc_load_arrays.argtypes = [C.POINTER(Options), C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_int,
                                      C.c_void_p, C.c_void_p, C.POINTER(P)]
        L.orc_free.argtypes = [P]
        L.orc_rng_synthetic.argtypes = [P, C.c_uint64]
        L.orc_rng_table.argtypes = [P, C.c_int, C.c_int, C.c_void_p]
        for f in ("orc_step", "orc_should_continue", "orc_should_export", "orc_finish_step", "orc_check_data",
                  "orc_current_n_grains"):
            getattr(L, f).argtypes = [P]
            getattr(L, f).restype = C.c_int
        L.orc_export.argtypes = [P, C.c_char_p, C.c_double]
        L.orc_field.argtypes = [P, C.c_char_p, C.POINTER(C.c_int64), C.POINTER(C.c_int)]
        L.orc_field.restype = C.c_void_p
        L.orc_clone.argtypes = [P]
        L.orc_clone.restype = P
        for f in ("orc_compute_boundary_arclengths", "orc_compute_grain_areas", "orc_compute_boundary_energies",
                  "orc_compute_vertex_energies", "orc_compute_vertex_velocities", "orc_compute_grain_dadts",
                  "orc_compute_t_ext"):
            getattr(L, f).argtypes = [P]
        L.orc_alloc_blank.argtypes = [C.POINTER(Options), C.c_int, C.c_int, C.c_int]
        L.orc_alloc_blank.restype = P
        L.orc_state_digest.argtypes = [P, C.c_void_p]
        L.orc_state_digest.restype = None
        L.orc_nucleated_fraction_area.argtypes = [P]
        L.orc_nucleated_fraction_area.restype = C.c_double
        _lib = L
    return _lib


_KIND = {0: np.float64, 1: np.int32, 2: np.uint8, 3: np.int64}


def default_options(**kw):
    o = Options()
    lib().orc_default_options(C.byref(o))
    for k, v in kw.items():
        setattr(o, k, v.encode() if isinstance(v, str) else v)
    return o


def finish_options(o):
    lib().orc_finish_options(C.byref(o))
    return o


def parse_ini(path):
    o = Options()
    rc = lib().orc_parse_ini(path.encode(), C.byref(o))
    if rc:
        raise OSError("orc_parse_ini(%s) failed: %d" % (path, rc))
    return o


class Oracle:
    """One reference-semantics simulation held by the C oracle."""

    def __init__(self, ptr, keep=()):
        self._p = ptr
        self._keep = list(keep)

    @classmethod
    def from_files(cls, opt):
        p = C.POINTER(_State)()
        rc = lib().orc_load_files(C.byref(opt), C.byref(p))
        if rc:
            raise RuntimeError("orc_load_files failed: %d" % rc)
        return cls(p)

    @classmethod
    def from_arrays(cls, opt, xy, ridges, oris, se):
        xy = np.ascontiguousarray(xy, np.float64)
        ridges = np.ascontiguousarray(ridges, np.int32)
        oris = np.ascontiguousarray(oris, np.float64)
        se = np.ascontiguousarray(se, np.float64)
        p = C.POINTER(_State)()
        rc = lib().orc_load_arrays(C.byref(opt), len(xy), xy.ctypes.data, len(ridges), ridges.ctypes.data,
                                   len(oris), oris.ctypes.data, se.ctypes.data, C.byref(p))
        if rc:
            raise RuntimeError("orc_load_arrays failed: %d" % rc)
        return cls(p)

    @classmethod
    def from_state(cls, opt, st, n=0, allow_nucleation=0, vrt_id_candidate=0):
        """An oracle holding a mesh taken in the middle of a run: st is a
        dict of arrays in the engine's sevc_get_state layout; the polling
        buffer starts as the candidate flags, the random stream at its
        beginning.  Used to time the reference's algorithm on a given
        state; the run from here is the reference's step logic, but not
        bit-identical to the run that produced st (its polling buffer and
        random streams are not carried over)."""
        nv, nb, ng = len(st["px"]), len(st["bini"]), len(st["gvlen"])
        o = cls(lib().orc_alloc_blank(C.byref(opt), nv, nb, ng))
        for f in ("px", "py", "vx", "vy", "venergy", "vel_bnd_x", "vel_grn_x", "vel_bnd_y", "vel_grn_y", "ven", "vb",
                  "vg", "bini", "bend", "benergy", "blen", "btext", "ben", "bcand", "glist", "gvlen", "garea", "gdadt",
                  "gori", "gse", "gen", "gtype"):
            o.field(f)[:] = st[f]
        o.field("cand_buf")[:] = st["bcand"] * st["ben"]
        s = o.s
        s.n = n
        s.t = n * opt.dt
        s.curr_n_grains = int(st["gen"].sum())
        s.allow_nucleation = allow_nucleation
        s.vrt_id_candidate = vrt_id_candidate
        return o

    def __del__(self):
        if getattr(self, "_p", None) and _lib is not None:
            _lib.orc_free(self._p)
            self._p = None

    @property
    def s(self):
        return self._p.contents

    def clone(self):
        return Oracle(lib().orc_clone(self._p), self._keep)

    def field(self, name):
        n, k = C.c_int64(), C.c_int()
        ptr = lib().orc_field(self._p, name.encode(), C.byref(n), C.byref(k))
        if not ptr:
            raise KeyError(name)
        if k.value == 4:
            return np.ctypeslib.as_array(C.cast(ptr, C.POINTER(C.c_int32)), shape=(n.value * 4,)).reshape(-1, 4)
        ct = {0: C.c_double, 1: C.c_int32, 2: C.c_uint8, 3: C.c_int64}[k.value]
        return np.ctypeslib.as_array(C.cast(ptr, C.POINTER(ct)), shape=(n.value,))

    def state_digest(self):
        """Per-field digests (the definition of the engine's sevc_state_digest)."""
        out = (C.c_uint64 * 20)()
        lib().orc_state_digest(self._p, out)
        return tuple(int(x) for x in out)

    def rng_synthetic(self, seed):
        lib().orc_rng_synthetic(self._p, seed)

    def rng_table(self, table):
        table = np.ascontiguousarray(table, np.float64)
        self._keep.append(table)
        lib().orc_rng_table(self._p, table.shape[0], table.shape[1], table.ctypes.data)

    def set_threads(self, n):
        self.s.nthreads_omp = int(n)

    def step(self):
        return lib().orc_step(self._p)

    def should_continue(self):
        return bool(lib().orc_should_continue(self._p))

    def should_export(self):
        return bool(lib().orc_should_export(self._p))

    def finish_step(self):
        return bool(lib().orc_finish_step(self._p))

    def export(self, path, time=None):
        return lib().orc_export(self._p, path.encode(), self.s.t if time is None else time)

    def check_data(self):
        return lib().orc_check_data(self._p)

    def run(self, out_dir, on_step=None):
        """The loop of src/main.cu:120-394: step, export when due, stop tests.

        Snapshots go to ``out_dir/%06d.txt`` with the reference's counter."""
        os.makedirs(out_dir, exist_ok=True)
        prog = 0
        while self.should_continue():
            rc = self.step()
            if rc:
                return rc
            if on_step:
                on_step(self)
            if self.should_export():
                if self.check_data():
                    return -1
                self.export(os.path.join(out_dir, "%06d.txt" % prog))
                prog += 1
            if not self.finish_step():
                break
        return 0
