"""Pure-Python writer of the jittered periodic-square .su2 meshes (numpy only).

TEST INFRASTRUCTURE: the reference arm of bench.py and the oracle-side checks
make their meshes with it, so that a process timing the reference's CPU path
never loads the CUDA library.  Its output is byte for byte the file that the
library's own writer (fvgb_write_su2_periodic_square) produces for the same
arguments; tests/test_host.py checks that.

The mesh: (n + 1)^2 nodes on [0, L]^2 at spacing h = L / n, written as n x n
SU2 type-9 quads (counter-clockwise), interior nodes moved by
(2u - 1) jitter h in x and then y, u from splitmix64 (Steele, Lea and Flood,
"Fast splittable pseudorandom number generators", OOPSLA 2014) seeded with
`seed`, top 53 bits over 2^53.  Markers periodic_1 (x = 0 ascending y, x = L
descending y) and periodic_2 (y = L ascending x, y = 0 descending x), the
orientation of the reference's isentropic-vortex example.
"""
import numpy as np

_GAMMA = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


def splitmix_uniform(seed, count):
    """The first `count` uniforms in [0, 1) of splitmix64 started at `seed`."""
    with np.errstate(over="ignore"):
        k = np.arange(1, count + 1, dtype=np.uint64)
        z = np.uint64(seed) + k * _GAMMA
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
        z = z ^ (z >> np.uint64(31))
    return (z >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def periodic_square_text(n, L=10.0, jitter=0.0, seed=20261203):
    """The .su2 text of the n x n periodic square."""
    if n < 2 or not L > 0:
        raise ValueError("bad square mesh arguments")
    h = L / n
    nn = n + 1
    out = [f"% periodic square [0,{L:.17g}]^2, {n} x {n} quads, jitter {jitter:.17g} h, seed {seed}\nNDIME= 2\n",
           f"NELEM= {n * n}\n"]
    j, i = np.divmod(np.arange(n * n, dtype=np.int64), n)
    a = j * nn + i
    quads = np.stack([a, a + 1, a + nn + 1, a + nn, np.arange(n * n, dtype=np.int64)], axis=1)
    out.append("".join("9 %d %d %d %d %d\n" % tuple(q) for q in quads.tolist()))
    out.append(f"NPOIN= {nn * nn}\n")
    jj, ii = np.divmod(np.arange(nn * nn, dtype=np.int64), nn)
    x = ii.astype(np.float64) * h
    y = jj.astype(np.float64) * h
    x[ii == n] = L
    y[jj == n] = L
    if jitter > 0:
        inner = np.flatnonzero((ii > 0) & (ii < n) & (jj > 0) & (jj < n))
        u = splitmix_uniform(seed, 2 * inner.size)
        x[inner] += ((2.0 * u[0::2] - 1.0) * jitter) * h
        y[inner] += ((2.0 * u[1::2] - 1.0) * jitter) * h
    out.append("".join("%.17g %.17g %d\n" % t for t in zip(x.tolist(), y.tolist(), range(nn * nn))))
    out.append("NMARK= 4\n")
    rng = range(n)
    out.append(f"MARKER_TAG= periodic_1\nMARKER_ELEMS= {n}\n" + "".join(f"3 {k * nn} {(k + 1) * nn}\n" for k in rng))
    out.append(f"MARKER_TAG= periodic_1\nMARKER_ELEMS= {n}\n" +
               "".join(f"3 {k * nn + n} {(k - 1) * nn + n}\n" for k in range(n, 0, -1)))
    out.append(f"MARKER_TAG= periodic_2\nMARKER_ELEMS= {n}\n" +
               "".join(f"3 {n * nn + k} {n * nn + k + 1}\n" for k in rng))
    out.append(f"MARKER_TAG= periodic_2\nMARKER_ELEMS= {n}\n" + "".join(f"3 {k} {k - 1}\n" for k in range(n, 0, -1)))
    return "".join(out)


def write_periodic_square(path, n, L=10.0, jitter=0.0, seed=20261203):
    with open(path, "w") as f:
        f.write(periodic_square_text(n, L, jitter, seed))
    return path
