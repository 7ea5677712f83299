"""Digests of snapshot files in the reference's text format (src/io.h:280-377).

full  sha256 of the file bytes;
topo  sha256 of the integer columns only (ids, enabled flags, connectivity,
      candidate flags, grain types, list lengths and vertex lists), which do
      not depend on the last bit of any transcendental function.
"""
import hashlib

import numpy as np


def parse(path):
    """Snapshot -> dict of numpy arrays (vertex, boundary, grain tables)."""
    with open(path) as f:
        lines = f.read().splitlines()
    hdr, i = {}, 0
    while not lines[i].startswith("#VERTEX"):
        k, v = lines[i].rsplit(" ", 1)
        hdr[k] = v
        i += 1
    nv, nb, ng = int(hdr["VERTICES"]), int(hdr["BOUNDARIES"]), int(hdr["GRAINS"])
    V = np.array([l.split() for l in lines[i + 1:i + 1 + nv]], dtype=object)
    i += 1 + nv
    B = np.array([l.split() for l in lines[i + 1:i + 1 + nb]], dtype=object)
    i += 1 + nb
    G = [l.split() for l in lines[i + 1:i + 1 + ng]]
    out = {"header": hdr}
    out["v_int"] = V[:, [0, 1, 11, 12, 13, 14, 15, 16]].astype(np.int64)
    out["v_float"] = V[:, 2:11].astype(np.float64)  # energy x y vx vy vbx vgx vby vgy
    out["b_int"] = B[:, [0, 1, 2, 3, 7]].astype(np.int64)
    out["b_float"] = B[:, 4:7].astype(np.float64)   # energy arclen t_ext
    out["g_int"] = np.array([[int(r[0]), int(r[1]), int(r[2]), int(r[7])] + [int(x) for x in r[8:]] for r in G],
                            dtype=np.int64)
    out["g_float"] = np.array([[float(x) for x in r[3:7]] for r in G], dtype=np.float64)  # ori se area dadt
    return out


def digests(path):
    with open(path, "rb") as f:
        full = hashlib.sha256(f.read()).hexdigest()
    s = parse(path)
    h = hashlib.sha256()
    for k in ("v_int", "b_int", "g_int"):
        h.update(np.ascontiguousarray(s[k]).tobytes())
    return full, h.hexdigest()
