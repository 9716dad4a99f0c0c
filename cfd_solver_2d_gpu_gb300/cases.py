"""Benchmark and test workloads: synthetic meshes of the named shapes and the
input.toml text for each (same keys as the reference's input.toml,
FVMR/src/input/TomlFileManager.cpp:110-170, plus the [gpu] table).

    vortex_small   64 x 64 periodic vortex, 8,192 cells, Euler, Roe, first order, RK3, CFL 0.5
    vortex_large   1448 x 1448 jittered vortex, 4,193,408 cells, LSQ + Barth, Roe or LLF, SSP-RK3, CFL 0.8
    cylinder_ns    512 x 256 O-grid, 262,144 cells, Navier-Stokes, Ma 0.2, Re 100, LSQ, RK3
    vortex_adjoint 256 x 256 jittered vortex, 131,072 cells, LSQ + Barth, Roe, SSP-RK3
"""
import os
import re
import tempfile

from . import write_cylinder, write_periodic_square

JITTER_SEED = 20261203


def _num(x):
    """A float as TOML accepts it: no leading zeros in the exponent (1.79e-5, not 1.79e-05)."""
    s = repr(float(x))
    if "e" in s:
        mant, exp = s.split("e")
        sign = "-" if exp.startswith("-") else ""
        s = f"{mant}e{sign}{int(exp.lstrip('+-'))}"
    return s


def toml_text(*, equation=1, flux=2002, reconstruct=3001, gradient=1, limiter=1, time_advance=3103, CFL=0.5,
              T_end=1000.0, ic_type=2, vortex=(5.0, 5.0, 5.0), inf_mode=1, inf=(1.0, 1.0, 1.0, 1.0), Ma=0.2,
              AoA=0.0, Re=None, mu0=17.9e-6, Pr=0.72, ref_area=1.0, lsq_det="ref", wall_bc="ref", restrict="ref",
              renumber=1, filename="mesh", max_iteration=1000, inlet=None, outlet=None, shock_tube=None, dmr=None,
              steady=False, CFL_steady=0.8):
    """inlet / outlet: None (table left out, the reference's default state), (rho, u, v, p)
    (input_mode 1), (rho, u, angle_degree, p, "angle") (input_mode 3) or (Ma, AoA)
    (input_mode 0), as [boundaryCondition.2D.inlet|outlet].  shock_tube: (x, y, normal x,
    normal y) of [initialCondition.shockTube]; dmr: (x, y, angle) of
    [initialCondition.doubleShockReflection]."""
    lines = [
        "[basic]", "continue = false", "dimension = 2", f'filename = "{filename}"', 'meshFileType = "su2"',
        "useGPU = 1", "isDebugMode = false", "",
        "[constant]", "T0 = 288.16", "p0 = 101325.0", f"Pr = {_num(Pr)}", "gamma = 1.4", f"referenceArea = {_num(ref_area)}",
    ]
    if Re is not None:
        lines += [f"Re = {_num(Re)}", "calculate_mu0_by_Re = true"]
    else:
        lines += [f"mu0 = {_num(mu0)}", "calculate_mu0_by_Re = false"]
    lines += ["", "[initialCondition]", f"type = {ic_type}"]
    if ic_type == 2:
        lines += ["[initialCondition.isentropicVortex]", f"vortex_x = {_num(vortex[0])}", f"vortex_y = {_num(vortex[1])}",
                  f"vortex_strength = {_num(vortex[2])}"]
    if shock_tube is not None:
        lines += ["[initialCondition.shockTube]"] + [f"{k} = {_num(v)}" for k, v in zip(
            ("shock_x", "shock_y", "shock_normal_x", "shock_normal_y"), shock_tube)]
    if dmr is not None:
        lines += ["[initialCondition.doubleShockReflection]"] + [f"{k} = {_num(v)}" for k, v in zip(
            ("shock_x", "shock_y", "shock_angle_degree"), dmr)]
    lines += ["", "[boundaryCondition.2D.inf]"]
    if inf_mode == 1:
        lines += ["input_mode = 1", f"rho = {_num(inf[0])}", f"u = {_num(inf[1])}", f"v = {_num(inf[2])}", f"p = {_num(inf[3])}"]
    else:
        lines += ["input_mode = 0", f"Ma = {_num(Ma)}", f"AoA = {_num(AoA)}"]
    for name, bc in (("inlet", inlet), ("outlet", outlet)):
        if bc is None:
            continue
        lines += ["", f"[boundaryCondition.2D.{name}]"]
        if len(bc) == 4:
            lines += ["input_mode = 1"] + [f"{k} = {_num(v)}" for k, v in zip(("rho", "u", "v", "p"), bc)]
        elif len(bc) == 5:
            lines += ["input_mode = 3"] + [f"{k} = {_num(v)}" for k, v in zip(("rho", "u", "angle_degree", "p"), bc)]
        else:
            lines += ["input_mode = 0", f"Ma = {_num(bc[0])}", f"AoA = {_num(bc[1])}"]
    lines += ["", "[output]", "step_per_print = 50", "step_per_output_field = 100", "step_per_output_hist = 100",
              f"maxIteration = {max_iteration}", "tolerace_residual = 1e-7", "",
              "[physicsModel]", f"equation = {equation}", "",
              "[time]", f"is_steady = {1 if steady else 0}", "is_explicit = 1"] + (
                  [f"CFL = {_num(CFL)}"] if CFL is not None else []) + [
              f"CFL_steady = {_num(CFL_steady)}", f"max_physical_time = {_num(T_end)}",
              f"time_advance = {time_advance}", "",
              "[inviscid_flux_method]", f"flag_reconstruct = {reconstruct}", f"flag_gradient = {gradient}",
              f"flux_conservation_scheme = {flux}", f"flux_limiter = {limiter}", "",
              "[gpu]", f'lsq_det = "{lsq_det}"', f'wall_bc = "{wall_bc}"', f'restrict = "{restrict}"',
              f"renumber = {renumber}", ""]
    return "\n".join(lines)


def cache_dir(directory=None):
    d = directory or os.environ.get("FVGB_CACHE", os.path.join(tempfile.gettempdir(), "fvgb_meshes"))
    os.makedirs(d, exist_ok=True)
    return d


def square_mesh(n, jitter=0.0, L=10.0, seed=JITTER_SEED, directory=None):
    path = os.path.join(cache_dir(directory), f"square_{n}_{jitter:g}_{seed}.su2")
    if not os.path.exists(path):
        tmp = path + f".{os.getpid()}.tmp"
        write_periodic_square(tmp, n, L, jitter, seed)
        os.replace(tmp, path)
    return path


def mixed_mesh(su2_path, out_path, seed=5):
    """A copy of a quad mesh in which a seeded half of the quads are written as two
    triangles split along the other diagonal, (n0, n1, n2) + (n0, n2, n3), where the
    reader itself splits a quad into (n0, n1, n3) + (n3, n1, n2): a mesh of mixed
    element types and mixed diagonals."""
    import numpy as np
    rng = np.random.default_rng(seed)
    lines = open(su2_path).read().split("\n")
    out, i = [], 0
    while i < len(lines):
        ln = lines[i]
        if ln.startswith("NELEM="):
            n = int(ln.split("=")[1])
            elems = []
            for q in lines[i + 1:i + 1 + n]:
                f = q.split()
                if f[0] == "9" and rng.random() < 0.5:
                    a, b, c, d = f[1:5]
                    elems += [f"5 {a} {b} {c}", f"5 {a} {c} {d}"]
                else:
                    elems.append(" ".join(f[:-1]))
            out.append(f"NELEM= {len(elems)}")
            out += [f"{e} {k}" for k, e in enumerate(elems)]
            i += 1 + n
            continue
        out.append(ln)
        i += 1
    with open(out_path, "w") as fh:
        fh.write("\n".join(out))
    return out_path


def channel_mesh(n, jitter=0.0, L=10.0, seed=JITTER_SEED, directory=None):
    """The square of square_mesh with its four boundaries renamed: inlet (x = 0),
    outlet (x = L), symmetry (y = L) and wall (y = 0; slip for Euler, no-slip
    adiabatic for Navier-Stokes)."""
    path = os.path.join(cache_dir(directory), f"channel_{n}_{jitter:g}_{seed}.su2")
    if not os.path.exists(path):
        text = open(square_mesh(n, jitter, L, seed, directory)).read()
        tags = iter(("inlet", "outlet", "symmetry", "wall"))  # the square's marker order: left, right, top, bottom
        text = re.sub(r"MARKER_TAG= periodic_\d", lambda _: "MARKER_TAG= " + next(tags), text)
        tmp = path + f".{os.getpid()}.tmp"
        with open(tmp, "w") as f:
            f.write(text)
        os.replace(tmp, path)
    return path


def dmr_mesh(nx, jitter=0.0, wall="wall", seed=JITTER_SEED, directory=None):
    """The double-Mach-reflection domain [0, 4] x [0, 1] as nx x nx/4 quads (nx a
    multiple of 24, so that a node sits at x = 1/6).  Markers: "inlet" (x = 0, and
    y = 0 for x < 1/6), "outlet" (x = 4), "dsr" (y = 1) and `wall` (y = 0 from
    x = 1/6).  Interior nodes are moved by up to +-jitter h in x and y (seeded)."""
    import numpy as np
    if nx % 24:
        raise ValueError("nx must be a multiple of 24")
    ny = nx // 4
    path = os.path.join(cache_dir(directory), f"dmr_{nx}_{jitter:g}_{wall}_{seed}.su2")
    if os.path.exists(path):
        return path
    h = 4.0 / nx
    xs, ys = np.meshgrid(np.arange(nx + 1) * h, np.arange(ny + 1) * h)  # node (i, j) at index j (nx + 1) + i
    rng = np.random.default_rng(seed)
    d = rng.uniform(-jitter * h, jitter * h, (2, ny + 1, nx + 1))
    d[:, [0, -1], :] = 0.0
    d[:, :, [0, -1]] = 0.0
    xs, ys = xs + d[0], ys + d[1]
    nid = lambda i, j: j * (nx + 1) + i
    lines = ["%% double Mach reflection domain [0,4]x[0,1], %d x %d quads, jitter %g h, seed %d" % (nx, ny, jitter, seed),
             "NDIME= 2", "NELEM= %d" % (nx * ny)]
    k = 0
    for j in range(ny):
        for i in range(nx):
            lines.append("9 %d %d %d %d %d" % (nid(i, j), nid(i + 1, j), nid(i + 1, j + 1), nid(i, j + 1), k))
            k += 1
    lines.append("NPOIN= %d" % ((nx + 1) * (ny + 1)))
    for j in range(ny + 1):
        for i in range(nx + 1):
            lines.append("%.17g %.17g %d" % (xs[j, i], ys[j, i], nid(i, j)))
    i_w = nx // 24
    markers = [("inlet", [(nid(0, j + 1), nid(0, j)) for j in reversed(range(ny))] +
                [(nid(i, 0), nid(i + 1, 0)) for i in range(i_w)]),
               ("outlet", [(nid(nx, j), nid(nx, j + 1)) for j in range(ny)]),
               ("dsr", [(nid(i + 1, ny), nid(i, ny)) for i in reversed(range(nx))]),
               (wall, [(nid(i, 0), nid(i + 1, 0)) for i in range(i_w, nx)])]
    lines.append("NMARK= %d" % len(markers))
    for name, edges in markers:
        lines += ["MARKER_TAG= " + name, "MARKER_ELEMS= %d" % len(edges)] + ["3 %d %d" % e for e in edges]
    tmp = path + f".{os.getpid()}.tmp"
    with open(tmp, "w") as f:
        f.write("\n".join(lines) + "\n")
    os.replace(tmp, path)
    return path


def cylinder_mesh(n_theta, n_r, r0=0.5, r1=20.0, first_dr=1e-3, directory=None):
    path = os.path.join(cache_dir(directory), f"cyl_{n_theta}_{n_r}_{r0:g}_{r1:g}_{first_dr:g}.su2")
    if not os.path.exists(path):
        tmp = path + f".{os.getpid()}.tmp"
        write_cylinder(tmp, n_theta, n_r, r0, r1, first_dr)
        os.replace(tmp, path)
    return path


def wavy(mesh, U, L=10.0):
    """U with smooth multiplicative waves of period L on all four variables.

    Used where the initial field must be non-uniform in every cell: the
    isentropic vortex is uniform to ~1e-11 away from its core, where the Barth
    limiter and the time-step minimum switch branch under tiny perturbations."""
    import numpy as np
    x, y = mesh.array("elem_xy")
    k = 2 * np.pi / L
    f = 1 + 0.05 * np.sin(k * x + 0.3) * np.cos(k * y + 0.7) + 0.03 * np.sin(2 * k * (x + y))
    U = np.array(U, dtype=np.float64, copy=True)
    U[0] *= f
    U[1] *= 1 + 0.04 * np.cos(k * y)
    U[2] *= 1 - 0.04 * np.sin(k * x)
    U[3] *= f
    return U


def write_case(directory, name, toml, mesh_path):
    os.makedirs(directory, exist_ok=True)
    tp = os.path.join(directory, name + ".toml")
    with open(tp, "w") as f:
        f.write(toml)
    return tp, mesh_path


def vortex_small(directory, n=64, time_advance=3103, **kw):
    """64 x 64 periodic vortex (8,192 cells): Euler, Roe, first order, RK3, CFL 0.5."""
    args = dict(flux=2002, reconstruct=3001, gradient=1, limiter=1, time_advance=time_advance, CFL=0.5)
    args.update(kw)
    return write_case(directory, f"vortex_small_{n}", toml_text(**args), square_mesh(n))


def vortex_large(directory, n=1448, flux=2002, **kw):
    """1448 x 1448 jittered vortex (4,193,408 cells): LSQ + Barth, SSP-RK3, CFL 0.8."""
    args = dict(flux=flux, reconstruct=3002, gradient=1, limiter=1, time_advance=3104, CFL=0.8)
    args.update(kw)
    return write_case(directory, f"vortex_large_{n}_{flux}", toml_text(**args), square_mesh(n, jitter=0.2))


def cylinder_ns(directory, n_theta=512, n_r=256, **kw):
    """Laminar cylinder, Ma 0.2, Re 100 (diameter), Pr 0.72, LSQ + Barth, RK3."""
    args = dict(equation=2, flux=2002, reconstruct=3002, gradient=1, limiter=1, time_advance=3103, CFL=0.5,
                ic_type=1, inf_mode=0, Ma=0.2, AoA=0.0, Re=100.0, Pr=0.72, ref_area=1.0)
    args.update(kw)
    return write_case(directory, f"cylinder_ns_{n_theta}_{n_r}", toml_text(**args), cylinder_mesh(n_theta, n_r))


def cylinder_batch(directory, n=256, n_min=5000, n_max=200000, seed=20261203, first_dr=1e-3, **kw):
    """Batched cylinder instances: cell counts log-uniform in [n_min, n_max]
    (n_r = round(sqrt(N/4)), n_theta = 2 n_r), freestream Mach uniform in
    [0.1, 0.6]; inviscid (the wall is a slip wall), Roe, LSQ + Barth, RK3.
    Returns a list of (toml path, su2 path, Mach)."""
    import numpy as np
    rng = np.random.default_rng(seed)
    sizes = np.exp(rng.uniform(np.log(n_min), np.log(n_max), n))
    machs = rng.uniform(0.1, 0.6, n)
    out = []
    for i, (sz, ma) in enumerate(zip(sizes, machs)):
        nr = max(2, int(round(np.sqrt(sz / 4.0))))
        args = dict(equation=1, flux=2002, reconstruct=3002, gradient=1, limiter=1, time_advance=3103, CFL=0.5,
                    ic_type=1, inf_mode=0, Ma=float(ma), AoA=0.0, T_end=1e9)
        args.update(kw)
        tp, sp = write_case(directory, f"batch_{i}", toml_text(**args),
                            cylinder_mesh(2 * nr, nr, first_dr=first_dr, directory=directory))
        out.append((tp, sp, float(ma)))
    return out
