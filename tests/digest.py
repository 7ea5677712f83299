"""numpy restatement of sevc_state_digest (include/sevc.h), used by the
tests to digest the oracle's state the way the engine digests its own.

digest of field f = sum over elements i of
    splitmix64_finaliser((f << 56) + i * 0x9E3779B97F4A7C15 + bits_i)  (mod 2**64)
with bits_i the IEEE-754 pattern of a double, the value of an int32 taken
as unsigned 32-bit, or the byte of a uint8.
"""
import numpy as np

K = np.uint64(0x9E3779B97F4A7C15)
C1 = np.uint64(0xBF58476D1CE4E5B9)
C2 = np.uint64(0x94D049BB133111EB)
FIELDS = ("px", "py", "vx", "vy", "ven", "vb", "vg", "bini", "bend", "benergy", "blen", "ben", "bcand",
          "glist", "gvlen", "garea", "gori", "gse", "gen", "gtype")


def _bits(a):
    a = np.ascontiguousarray(a)
    if a.dtype == np.float64:
        return a.view(np.uint64)
    if a.dtype == np.int32:
        return a.view(np.uint32).astype(np.uint64)
    if a.dtype == np.uint8:
        return a.astype(np.uint64)
    raise TypeError(a.dtype)


def field_digest(f, a):
    b = _bits(a).ravel()
    i = np.arange(b.size, dtype=np.uint64)
    with np.errstate(over="ignore"):
        z = (np.uint64(f) << np.uint64(56)) + i * K + b
        z = (z ^ (z >> np.uint64(30))) * C1
        z = (z ^ (z >> np.uint64(27))) * C2
        z = z ^ (z >> np.uint64(31))
        return int(np.sum(z, dtype=np.uint64))


def digest(get):
    """get(name) -> array in the layout of sevc_get_state (an oracle's
    field() or a get_state() dict's __getitem__)."""
    return tuple(field_digest(f, get(name)) for f, name in enumerate(FIELDS))
