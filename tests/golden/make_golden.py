"""Generates the golden fixtures under tests/golden/ by running the reference
itself: the reference's CPU step path compiled from its own sources with
myfloat = double (oracle/ref, binary oracle/_ref/fvmr_ref_f64).

Run here, where the reference sources are present:
    make -C oracle/ref && python tests/golden/make_golden.py [fixture names]

Each fixture is one compressed .npz with the case's input.toml text, the mesh
(.su2 text, compressed), the reference's mesh arrays, its initial field, one
residual evaluation (rhs, limited gradients, dt), the state after a few
steps, and the reference's residual norms (get_residual_host: L-infinity, L1
and L2) of the rhs evaluation and of the last residual of the steps.  Test
infrastructure.
"""
import gzip
import io
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

from cfd_solver_2d_gpu_gb300 import cases  # noqa: E402
from fvmrdump import read_dump  # noqa: E402

REF = os.path.join(ROOT, "oracle", "_ref", "fvmr_ref_f64")
REF32 = os.path.join(ROOT, "oracle", "_ref", "fvmr_ref_f32")

MESH_KEYS = ["node_xy", "elem_nodes", "elem_edges", "elem_nbrs", "elem_xy", "elem_vol", "edge_nodes", "edge_L",
             "edge_R", "edge_set", "edge_pair", "edge_len", "edge_xy", "edge_normal", "bc_type", "U0"]


def golden_cases(d):
    """(name, toml text, su2 path, stepping mode, steps) of every fixture."""
    sq16 = cases.square_mesh(16, directory=d)
    sq24j = cases.square_mesh(24, jitter=0.2, directory=d)
    sq64 = cases.square_mesh(64, directory=d)
    cyl = cases.cylinder_mesh(32, 16, directory=d)
    ch24j = cases.channel_mesh(24, jitter=0.2, directory=d)
    dmr48 = cases.dmr_mesh(48, jitter=0.2, directory=d)
    T = cases.toml_text
    # the double Mach reflection of the reference's own example (2D_double_shock_reflect/input.toml):
    # shock at (1/6, 0), 60 degrees; post-shock inlet (8, 8.25 at -30 degrees, 116.5), still gas ahead
    dmr = dict(ic_type=4, dmr=(1.0 / 6.0, 0.0, 60.0), inlet=(8.0, 8.25, -30.0, 116.5, "angle"),
               outlet=(1.4, 0.0, 0.0, 1.0, "angle"))
    sod = dict(ic_type=3, inlet=(1.0, 0.0, 0.0, 1.0), outlet=(0.125, 0.0, 0.0, 0.1))
    return [
        # the small plain config: 64x64 vortex, Roe, first order, Kutta RK3, CFL 0.5, 1000 steps
        ("vortex64_roe_o1_rk3", T(flux=2002, reconstruct=3001, gradient=1, limiter=1, time_advance=3103, CFL=0.5),
         sq64, "rk3", 1000),
        ("vortex16_roe_o1_euler", T(flux=2002, reconstruct=3001, gradient=1, limiter=1, time_advance=3101, CFL=0.5),
         sq16, "euler", 20),
        ("vortex16_llf_o1_rk3", T(flux=2001, reconstruct=3001, gradient=1, limiter=1, time_advance=3103, CFL=0.5),
         sq16, "rk3", 20),
        # second order on a jittered mesh: LSQ (reference determinant guard) + Barth, SSP-RK3
        ("jvortex24_roe_lsq_barth_ssp", T(flux=2002, reconstruct=3002, gradient=1, limiter=1, time_advance=3104,
                                          CFL=0.8), sq24j, "ssprk3", 10),
        ("jvortex24_llf_lsq_barth_ssp", T(flux=2001, reconstruct=3002, gradient=1, limiter=1, time_advance=3104,
                                          CFL=0.8), sq24j, "ssprk3", 10),
        ("jvortex24_roe_gg_barth_euler", T(flux=2002, reconstruct=3002, gradient=2, limiter=1, time_advance=3101,
                                           CFL=0.8), sq24j, "euler", 10),
        ("jvortex24_roe_lsq_nolim_euler", T(flux=2002, reconstruct=3002, gradient=1, limiter=0, time_advance=3101,
                                            CFL=0.2), sq24j, "euler", 3),
        # laminar cylinder: no-slip wall, far field, Sutherland, Kutta RK3
        ("cylinder32_ns_lsq_barth_rk3", T(equation=2, flux=2002, reconstruct=3002, gradient=1, limiter=1,
                                          time_advance=3103, CFL=0.5, ic_type=1, inf_mode=0, Ma=0.2, Re=100.0),
         cyl, "rk3", 5),
        # inviscid cylinder: slip wall, far field
        ("cylinder32_euler_roe_lsq_rk3", T(equation=1, flux=2002, reconstruct=3002, gradient=1, limiter=1,
                                           time_advance=3103, CFL=0.5, ic_type=1, inf_mode=0, Ma=0.5), cyl, "rk3", 5),
        # channel: inlet (x = 0), outlet (x = 10), symmetry (y = 10), wall (y = 0); the vortex sits
        # near two of them so that their edges see a non-uniform state
        # subsonic inflow and outflow, slip wall
        ("jchannel24_roe_lsq_barth_ssp", T(flux=2002, reconstruct=3002, gradient=1, limiter=1, time_advance=3104,
                                           CFL=0.8, vortex=(2.5, 7.0, 5.0), inf=(1.0, 1.0, 0.3, 1.0),
                                           inlet=(1.0, 1.0, 0.3, 1.0), outlet=(1.0, 1.0, 0.0, 0.9)),
         ch24j, "ssprk3", 10),
        # supersonic inflow and outflow (Mach 2.1)
        ("jchannel24_llf_lsq_barth_rk3_mach2", T(flux=2001, reconstruct=3002, gradient=1, limiter=1,
                                                 time_advance=3103, CFL=0.5, vortex=(7.0, 3.0, 3.0),
                                                 inf=(1.0, 2.5, 0.2, 1.0), inlet=(1.0, 2.5, 0.2, 1.0),
                                                 outlet=(1.0, 2.5, 0.0, 1.0)), ch24j, "rk3", 10),
        # laminar: no-slip adiabatic wall, Green-Gauss gradients, viscous fluxes on every boundary kind
        ("jchannel24_ns_gg_barth_rk3", T(equation=2, flux=2002, reconstruct=3002, gradient=2, limiter=1,
                                         time_advance=3103, CFL=0.5, vortex=(5.0, 2.5, 5.0), inf=(1.0, 1.0, 0.3, 1.0),
                                         Re=100.0, inlet=(1.0, 1.0, 0.3, 1.0), outlet=(1.0, 1.0, 0.0, 0.9)),
         ch24j, "rk3", 5),
        # double Mach reflection: the "dsr" edges switch from the inlet to the outlet state where the
        # moving shock crosses the top boundary, at each stage's time; the runs are long enough
        # (t > 0.0042) for the crossing to pass one edge midpoint
        ("dmr48_roe_gg_barth_euler", T(flux=2002, reconstruct=3002, gradient=2, limiter=1, time_advance=3101,
                                       CFL=0.5, **dmr), dmr48, "euler", 40),
        ("dmr48_llf_lsq_barth_ssp", T(flux=2001, reconstruct=3002, gradient=1, limiter=1, time_advance=3104,
                                      CFL=0.5, **dmr), dmr48, "ssprk3", 25),
        ("dmr48_ns_lsq_barth_rk3", T(equation=2, flux=2002, reconstruct=3002, gradient=1, limiter=1,
                                     time_advance=3103, CFL=0.5, Re=1000.0, **dmr), dmr48, "rk3", 25),
        # shock tubes (Sod states): the normal along +x, and a tilted one
        ("sod_channel24_roe_o1_rk3", T(flux=2002, reconstruct=3001, gradient=1, limiter=1, time_advance=3103,
                                       CFL=0.5, shock_tube=(5.0, 0.0, 1.0, 0.0), **sod), ch24j, "rk3", 20),
        ("sod_tilted_channel24_llf_lsq_barth_ssp", T(flux=2001, reconstruct=3002, gradient=1, limiter=1,
                                                     time_advance=3104, CFL=0.5, shock_tube=(5.0, 5.0, 0.6, 0.8),
                                                     **sod), ch24j, "ssprk3", 10),
        # steady runs (local time stepping through iteration_host): the cylinder with time.CFL given,
        # the channel without it (the reference's default CFL 0.6; time.CFL_steady is not used)
        ("cylinder32_euler_roe_lsq_steady", T(equation=1, flux=2002, reconstruct=3002, gradient=1, limiter=1,
                                              time_advance=3101, CFL=0.8, steady=True, ic_type=1, inf_mode=0,
                                              Ma=0.5), cyl, "euler", 30),
        ("jchannel24_llf_o1_steady", T(flux=2001, reconstruct=3001, gradient=1, limiter=1, time_advance=3101,
                                       CFL=None, steady=True, CFL_steady=0.3, vortex=(2.5, 7.0, 5.0),
                                       inf=(1.0, 1.0, 0.3, 1.0), inlet=(1.0, 1.0, 0.3, 1.0),
                                       outlet=(1.0, 1.0, 0.0, 0.9)), ch24j, "euler", 30),
    ]


CONTINUE_DIR = os.path.join(HERE, "continue")
REF_MESH_KEYS = MESH_KEYS + ["edge_dist"]


def continue_cases(d):
    """(name, toml text, su2 path, equation) of the continue-file fixtures."""
    T = cases.toml_text
    return [
        ("jsquare12", T(equation=1, filename="jsquare12"), cases.square_mesh(12, jitter=0.2, directory=d), 1),
        ("cylinder16_ns", T(equation=2, filename="cylinder16_ns", ic_type=1, inf_mode=0, Ma=0.2, Re=100.0),
         cases.cylinder_mesh(16, 8, directory=d), 2),
    ]


def make_continue(d):
    """Continue files written by this library (fvgb_write_continue, seeded state) and the
    arrays the reference's ContinueFileReader builds from them (oracle/_ref, continue mode)."""
    import cfd_solver_2d_gpu_gb300 as fv
    os.makedirs(CONTINUE_DIR, exist_ok=True)
    for name, toml, su2, eq in continue_cases(d):
        m = fv.Mesh.read_su2(su2, equation=eq)
        U = np.random.default_rng(20261203).uniform(0.5, 2.0, (4, m.N))
        folder = os.path.join(d, "cont_" + name)
        os.makedirs(folder, exist_ok=True)
        path = os.path.join(folder, f"pause_{name}[0042].dat")
        m.write_continue(path, U, 0.123456789012345678, 42, 0.8)
        tp = os.path.join(folder, "input.toml")
        with open(tp, "w") as f:
            f.write(toml)
        ref = run_ref(REF, tp, folder, "continue", 0, os.path.join(d, name + "_cont.bin"))
        out = {k: ref[k] for k in REF_MESH_KEYS}
        out.update(continue_info=ref["continue"],
                   toml=np.frombuffer(toml.encode(), dtype=np.uint8),
                   pause_gz=np.frombuffer(gzip.compress(open(path, "rb").read(), mtime=0), dtype=np.uint8),
                   equation=np.array([eq]))
        dst = os.path.join(CONTINUE_DIR, name + ".npz")
        np.savez_compressed(dst, **out)
        print(f"{dst}: N={ref['sizes'][0]} ({os.path.getsize(dst) // 1024} KiB)")


OUTPUT_DIR = os.path.join(HERE, "output")


def output_cases(d):
    """(name, toml text, su2 path, forward-Euler steps) of the field-output fixtures."""
    T = cases.toml_text
    return [
        ("cylinder32_ns", T(equation=2, flux=2002, reconstruct=3002, gradient=1, limiter=1, time_advance=3101,
                            CFL=0.5, ic_type=1, inf_mode=0, Ma=0.3, AoA=4.0, Re=100.0, ref_area=2.0),
         cases.cylinder_mesh(32, 16, directory=d), 5),
        ("jvortex24", T(flux=2002, reconstruct=3002, gradient=1, limiter=1, time_advance=3101, CFL=0.5,
                        inf=(1.0, 1.0, 0.3, 1.0)), cases.square_mesh(24, jitter=0.2, directory=d), 3),
    ]


def make_output(d):
    """The reference's own field output (FieldWriter: node values, Tecplot volume and boundary
    files, one hist line) after a few forward-Euler steps (oracle/_ref, output mode)."""
    os.makedirs(OUTPUT_DIR, exist_ok=True)
    for name, toml, su2, steps in output_cases(d):
        tp = os.path.join(d, name + "_out.toml")
        with open(tp, "w") as f:
            f.write(toml)
        base = os.path.join(d, name + "_out.bin")
        ref = run_ref(REF, tp, su2, "output", steps, base)
        gz = lambda path: np.frombuffer(gzip.compress(open(path, "rb").read(), mtime=0), dtype=np.uint8)
        out = dict(U=ref["U"], t=ref["t"], node_ruvp=ref["node_ruvp"], node_Cp=ref["node_Cp"],
                   node_Ma=ref["node_Ma"], volume_gz=gz(base + ".volume.dat"), boundary_gz=gz(base + ".boundary.dat"),
                   hist=np.frombuffer(open(base + ".hist.dat", "rb").read(), dtype=np.uint8),
                   toml=np.frombuffer(toml.encode(), dtype=np.uint8),
                   su2_gz=np.frombuffer(gzip.compress(open(su2, "rb").read(), mtime=0), dtype=np.uint8),
                   steps=np.array([steps]))
        dst = os.path.join(OUTPUT_DIR, name + ".npz")
        np.savez_compressed(dst, **out)
        print(f"{dst}: N={ref['sizes'][0]} ({os.path.getsize(dst) // 1024} KiB)")


def run_ref(binary, toml_path, su2, mode, steps, out):
    r = subprocess.run([binary, toml_path, su2, mode, str(steps), out], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"{binary} {mode} failed: {r.stderr[-400:]}")
    return read_dump(out)


def main(only=()):
    """Makes every fixture, or with names on the command line only the step fixtures of
    those names (existing files are then left as they are)."""
    if not os.path.exists(REF):
        sys.exit("build the reference first: make -C oracle/ref")
    with tempfile.TemporaryDirectory() as d:
        for name, toml, su2, mode, steps in golden_cases(d):
            if only and name not in only:
                continue
            tp = os.path.join(d, name + ".toml")
            with open(tp, "w") as f:
                f.write(toml)
            rhs = run_ref(REF, tp, su2, "rhs", 0, os.path.join(d, name + "_rhs.bin"))
            stp = run_ref(REF, tp, su2, mode, steps, os.path.join(d, name + "_step.bin"))
            out = {k: rhs[k] for k in MESH_KEYS}
            out.update(rhs=rhs["rhs"], grad_x=rhs["grad_x"], grad_y=rhs["grad_y"], dt=rhs["dt"],
                       U=stp["U"], dts=stp["dts"], t=stp["t"], steps=np.array([steps]),
                       toml=np.frombuffer(toml.encode(), dtype=np.uint8),
                       su2_gz=np.frombuffer(gzip.compress(open(su2, "rb").read(), mtime=0), dtype=np.uint8),
                       mode=np.frombuffer(mode.encode(), dtype=np.uint8),
                       # the reference's get_residual_host norms (rows L-inf, L1, L2) of the rhs
                       # evaluation and of the last residual the steps evaluated
                       residual_rhs=rhs["residual_norms"].reshape(3, 4),
                       residual_step=stp["residual_norms"].reshape(3, 4))
            if os.path.exists(REF32):  # the reference as shipped (float), for the record
                s32 = run_ref(REF32, tp, su2, mode, steps, os.path.join(d, name + "_f32.bin"))
                out["U_f32"] = s32["U"]
            path = os.path.join(HERE, name + ".npz")
            np.savez_compressed(path, **out)
            print(f"{path}: N={rhs['sizes'][0]} {mode} x{steps} ({os.path.getsize(path) // 1024} KiB)")
        if not only:
            make_continue(d)
            make_output(d)


def load(name):
    """Loads a fixture and materialises its input.toml and .su2 in a temp directory."""
    z = np.load(os.path.join(HERE, name + ".npz"))
    d = tempfile.mkdtemp(prefix="fvgb_golden_")
    tp, sp = os.path.join(d, name + ".toml"), os.path.join(d, name + ".su2")
    with open(tp, "wb") as f:
        f.write(z["toml"].tobytes())
    with open(sp, "wb") as f:
        f.write(gzip.decompress(z["su2_gz"].tobytes()))
    data = {k: z[k] for k in z.files}
    data["mode"] = z["mode"].tobytes().decode()
    return tp, sp, data


def names():
    return sorted(f[:-4] for f in os.listdir(HERE) if f.endswith(".npz"))


if __name__ == "__main__":
    main(tuple(sys.argv[1:]))
