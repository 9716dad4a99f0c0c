"""Reader for the "FVMRDUMP" files written by the reference harness
(oracle/ref/harness.cpp): a magic word followed by named arrays, each as a
32-byte name, a one-byte type code ('i' int32, 'd' float64), an int64 count
and the raw little-endian data.  Test infrastructure."""
import numpy as np


def read_dump(path):
    out = {}
    with open(path, "rb") as f:
        if f.read(8) != b"FVMRDUMP":
            raise ValueError(f"{path}: not an FVMRDUMP file")
        while True:
            name = f.read(32)
            if len(name) < 32:
                break
            code = f.read(1)
            count = int(np.frombuffer(f.read(8), dtype="<i8")[0])
            dt = {b"i": "<i4", b"d": "<f8"}[code]
            out[name.rstrip(b"\0").decode()] = np.frombuffer(f.read(count * np.dtype(dt).itemsize), dtype=dt).copy()
    n, e, v, nb = (int(x) for x in out["sizes"])
    shapes = {"node_xy": (2, v), "elem_nodes": (4, n), "elem_edges": (4, n), "elem_nbrs": (4, n),
              "elem_xy": (2, n), "edge_nodes": (2, e), "edge_xy": (2, e), "edge_normal": (2, e),
              "U0": (4, n), "U": (4, n), "rhs": (4, n), "grad_x": (4, n), "grad_y": (4, n)}
    for k, s in shapes.items():
        if k in out:
            out[k] = out[k].reshape(s)
    return out
