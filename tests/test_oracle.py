"""The oracle (oracle/fvm_oracle.c) against the golden fixtures made by the
reference itself (tests/golden/make_golden.py), and, where the reference was
compiled here (oracle/_ref), against live reference runs.  CPU only."""
import os
import subprocess
import sys

import numpy as np
import pytest

from golden import make_golden
from oracle.pyoracle import Oracle

NAMES = make_golden.names()
MESH = {"node_xy": "node_xy", "elem_nodes": "elem_nodes", "elem_edges": "elem_edges", "elem_nbrs": "elem_nbrs",
        "elem_xy": "elem_xy", "elem_vol": "elem_vol", "edge_nodes": "edge_nodes", "edge_L": "edge_L",
        "edge_R": "edge_R", "edge_set": "edge_set", "edge_pair": "edge_pair", "edge_len": "edge_len",
        "edge_xy": "edge_xy", "edge_normal": "edge_normal", "bc_type": "bc_type"}
MODE_CODE = {"euler": 3101, "rk3": 3103, "ssprk3": 3104}


def rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


@pytest.fixture(scope="module", params=NAMES)
def case(request):
    tp, sp, g = make_golden.load(request.param)
    return request.param, Oracle(tp, sp), g


def test_mesh_bit_exact(case):
    name, o, g = case
    for k, v in MESH.items():
        a = o.array(v)
        assert np.array_equal(a, g[k].reshape(a.shape)), f"{name}: {k} differs from the reference"


def test_initial_field(case):
    name, o, g = case
    # exp/pow of the platform's libm: equal on x86, within a few ulp elsewhere
    assert rel(o.init_field(), g["U0"]) <= 1e-15


def test_residual_gradient_dt(case):
    name, o, g = case
    R, gx, gy = o.rhs(g["U0"])
    assert rel(R, g["rhs"]) <= 1e-14, name
    assert rel(gx, g["grad_x"]) <= 1e-14 and rel(gy, g["grad_y"]) <= 1e-14, name
    dt, _ = o.dt(g["U0"])
    assert abs(dt - g["dt"][0]) <= 1e-15 * g["dt"][0]


def test_steps(case):
    name, o, g = case
    if int(g["steps"][0]) > 100:
        pytest.skip("long run covered by the GPU parity test")
    o.params.time_advance = MODE_CODE[g["mode"]]
    U, t, dts, _ = o.run(g["U0"], int(g["steps"][0]))
    assert rel(U, g["U"]) <= 1e-13, name
    assert abs(t - g["t"][0]) <= 1e-14 * abs(g["t"][0])


def test_bit_exact_on_x86(case):
    """On the machine the fixtures were made on, the oracle is the reference bit for bit."""
    import platform
    if platform.machine() not in ("x86_64", "AMD64"):
        pytest.skip("libm differs across architectures")
    name, o, g = case
    R, gx, gy = o.rhs(g["U0"])
    assert np.array_equal(R, g["rhs"]) and np.array_equal(gx, g["grad_x"]), name


def test_planted_mistake_is_caught():
    """A checker that cannot fail checks nothing: plant a change in the oracle's
    parameters (gamma 1.4 -> 1.4 + 1e-9) and the residual no longer matches."""
    tp, sp, g = make_golden.load("jvortex24_roe_lsq_barth_ssp")
    o = Oracle(tp, sp)
    o.params.gamma = 1.4 + 1e-9
    R, _, _ = o.rhs(g["U0"])
    assert rel(R, g["rhs"]) > 1e-12


REF = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle", "_ref", "fvmr_ref_f64")


@pytest.mark.skipif(not os.path.exists(REF), reason="reference not compiled here (oracle/_ref)")
def test_live_reference_larger_mesh(tmp_path):
    """A 96x96 jittered second-order case run by the reference binary and the oracle."""
    from cfd_solver_2d_gpu_gb300 import cases
    from fvmrdump import read_dump
    su2 = cases.square_mesh(96, jitter=0.2, directory=str(tmp_path))
    tp = tmp_path / "c.toml"
    tp.write_text(cases.toml_text(flux=2002, reconstruct=3002, gradient=1, limiter=1, time_advance=3104, CFL=0.8))
    out = tmp_path / "r.bin"
    subprocess.run([REF, str(tp), su2, "ssprk3", "3", str(out)], check=True, capture_output=True)
    ref = read_dump(str(out))
    o = Oracle(str(tp), su2)
    U, t, _, _ = o.run(o.init_field(), 3)
    assert np.array_equal(U, ref["U"])


REF_CASES = os.path.join(os.path.dirname(REF), "quick_start", "U2NITS-10.0")
# the reference's example cases (folder, mesh) and what each exercises
EXAMPLES = [
    ("2D_isentropic_vortex", "ivortex50.su2"),        # periodic vortex, Green-Gauss, Roe
    ("2D_cylinder", "cylinder_allfar_50.su2"),       # laminar cylinder, no-slip wall, far field
    ("1D_shocktube", "shocktube_100.su2"),           # shock tube along x
    ("2D_Neuvillette_shock", "neuvillette.su2"),     # shock tube with the normal along y, laminar
    ("2D_double_shock_reflect", "dsr131new_slippery.su2"),  # "dsr" boundary, input_mode 3, laminar
]


@pytest.mark.skipif(not (os.path.exists(REF) and os.path.isdir(REF_CASES)),
                    reason="the reference (sources and oracle/_ref build) is only in the build container")
@pytest.mark.parametrize("folder,mesh", EXAMPLES)
def test_live_reference_own_examples(tmp_path, folder, mesh):
    """The reference's own example cases as shipped (mesh and input.toml), their mesh
    arrays, initial field and 5 forward-Euler steps run by the reference binary and by the
    oracle: identical bits; and this library's reader, input.toml and initial field on
    the same files."""
    from fvmrdump import read_dump
    su2 = os.path.join(REF_CASES, folder, mesh)
    tp = os.path.join(REF_CASES, folder, "input.toml")
    out = tmp_path / "r.bin"
    subprocess.run([REF, tp, su2, "euler", "5", str(out)], check=True, capture_output=True)
    ref = read_dump(str(out))
    o = Oracle(tp, su2)
    for k, v in MESH.items():
        assert np.array_equal(o.array(v), np.asarray(ref[k]).reshape(o.array(v).shape)), k
    U0 = o.init_field()
    assert np.array_equal(U0, ref["U0"].reshape(U0.shape))
    o.params.time_advance = 3101
    U, t, _, _ = o.run(U0, 5)
    assert np.array_equal(U, ref["U"].reshape(U.shape)) and t == ref["t"][0]
    import cfd_solver_2d_gpu_gb300 as fv
    p = fv.Params.from_toml(tp)
    m = fv.Mesh.read_su2(su2, p)
    for ours, theirs in (("edge_xy", "edge_xy"), ("edge_normal", "edge_normal"), ("elem_neighbors", "elem_nbrs"),
                         ("boundary_type", "bc_type")):
        assert np.array_equal(m.array(ours).ravel(), o.array(theirs).ravel()), ours
    assert np.array_equal(fv.initial_field(m, p), U0)
