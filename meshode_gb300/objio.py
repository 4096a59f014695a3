"""Wavefront OBJ reading and writing with the reference's conventions.

Mesh::ReadOBJ (src/lib/mesh.cc:14-44): only ``v`` and ``f`` records are read;
``v x y z`` is parsed as double; each ``f`` token keeps its leading digits
(``a/b/c`` -> ``a``), indices are 1-based, only the first three corners of a
polygon are kept; reading stops at the first line of 256 or more characters
(the reference reads lines into a 256-byte buffer with istream::getline).
Mesh::WriteOBJ (mesh.cc:46-64) prints coordinates with the default six
significant digits.
"""
import numpy as np


def _face_index(tok: bytes) -> int:
    i = 0
    for ch in tok:
        if ch == 0x2F:  # '/'
            break
        i = i * 10 + (ch - 48)
    return i - 1


def read_obj(path):
    """Returns (V float64 [n,3], F int64 [m,3]) exactly as Mesh::ReadOBJ."""
    V, F = [], []
    with open(path, "rb") as fh:
        for raw in fh:
            line = raw.rstrip(b"\r\n") if raw.endswith(b"\n") else raw
            if len(raw.rstrip(b"\n")) >= 256:
                break
            toks = line.split()
            if not toks:
                continue
            if toks[0] == b"v":
                if len(toks) < 4:
                    raise ValueError("malformed vertex record in %s: %r" % (path, raw))
                V.append((float(toks[1]), float(toks[2]), float(toks[3])))
            elif toks[0] == b"f":
                if len(toks) < 4:
                    raise ValueError("face record with fewer than 3 corners in %s: %r" % (path, raw))
                F.append((_face_index(toks[1]), _face_index(toks[2]), _face_index(toks[3])))
    return (np.asarray(V, np.float64).reshape(-1, 3), np.asarray(F, np.int64).reshape(-1, 3))


def write_obj(path, V, F):
    V = np.asarray(V, np.float64)
    F = np.asarray(F, np.int64)
    with open(path, "w") as fh:
        fh.writelines("v %g %g %g\n" % (v[0], v[1], v[2]) for v in V)
        fh.writelines("f %d %d %d\n" % (f[0] + 1, f[1] + 1, f[2] + 1) for f in F)
