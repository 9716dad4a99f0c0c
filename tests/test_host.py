"""Host side of the library (no GPU needed): the C ABI exports, input.toml
reading, .su2 reading and assembly against the reference's arrays, the
initial field, the synthetic mesh writers and the error paths."""
import ctypes
import os
import re

import numpy as np
import pytest

import cfd_solver_2d_gpu_gb300 as fv
from cfd_solver_2d_gpu_gb300 import cases
from golden import make_golden
from oracle.pyoracle import params_from_toml

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
MESH = {"node_xy": "node_xy", "elem_nodes": "elem_nodes", "elem_edges": "elem_edges",
        "elem_neighbors": "elem_nbrs", "elem_xy": "elem_xy", "elem_volume": "elem_vol", "edge_nodes": "edge_nodes",
        "edge_L": "edge_L", "edge_R": "edge_R", "edge_setID": "edge_set", "edge_periodicPair": "edge_pair",
        "edge_length": "edge_len", "edge_xy": "edge_xy", "edge_normal": "edge_normal", "boundary_type": "bc_type"}


def declared_symbols():
    names = set()
    for h in os.listdir(os.path.join(ROOT, "include")):
        if h.endswith(".h"):
            text = open(os.path.join(ROOT, "include", h)).read()
            names |= set(re.findall(r"\b(fvgb_\w+)\s*\(", text))
    return sorted(names)


def test_library_exports_every_declared_symbol():
    L = fv.lib()
    missing = [n for n in declared_symbols() if not hasattr(L, n)]
    assert not missing, missing
    assert fv.lib().fvgb_version().decode().startswith("fvgb")


@pytest.mark.parametrize("name", make_golden.names())
def test_mesh_matches_reference(name):
    tp, sp, g = make_golden.load(name)
    p = fv.Params.from_toml(tp)
    m = fv.Mesh.read_su2(sp, p)
    for k, v in MESH.items():
        a = m.array(k)
        assert np.array_equal(a, g[v].reshape(a.shape)), f"{name}: {k}"
    U0 = fv.initial_field(m, p)
    assert np.max(np.abs(U0 - g["U0"])) <= 1e-15 * np.max(np.abs(g["U0"]))


@pytest.mark.parametrize("name", make_golden.names())
def test_toml_matches_reference_semantics(name):
    tp, _, _ = make_golden.load(name)
    p = fv.Params.from_toml(tp)
    q, info = params_from_toml(tp)
    for k in ("equation", "flux_scheme", "reconstruct", "gradient", "limiter", "time_advance", "steady"):
        assert getattr(p, k) == getattr(q, k), k
    for k in ("gamma", "R", "Pr", "mu0", "T0", "CFL", "T_end"):
        assert getattr(p, k) == pytest.approx(getattr(q, k), rel=1e-15), k
    for k in ("inf", "inlet", "outlet"):
        assert np.allclose(list(getattr(p, k)), list(getattr(q, k)), rtol=1e-15, atol=0), k


# the reference's example cases, reached through the link the oracle recipe (oracle/ref) makes
# next to the reference build where the reference tree is mounted
REF_TOML = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle", "_ref", "quick_start",
                        "U2NITS-10.0")


@pytest.mark.skipif(not os.path.isdir(REF_TOML), reason="reference tree not mounted")
@pytest.mark.parametrize("case", ["2D_isentropic_vortex", "2D_cylinder", "1D_shocktube"])
def test_reads_the_references_own_input_toml(case):
    p = fv.Params.from_toml(os.path.join(REF_TOML, case, "input.toml"))
    assert p.mesh_name
    assert p.flux_scheme in (2001, 2002) and p.time_advance in (3101, 3103)


def test_su2_writers(tmp_path):
    sq = str(tmp_path / "sq.su2")
    fv.write_periodic_square(sq, 8, 10.0, 0.2, 7)
    m = fv.Mesh.read_su2(sq)
    assert (m.N, m.E, m.V) == (128, (3 * 128 + 32) // 2, 81)  # E = (3N + boundary edges) / 2
    # periodic edges all have a partner whose partner is the edge itself
    pair = m.array("edge_periodicPair")
    ids = np.nonzero(pair >= 0)[0]
    assert len(ids) == 32 and np.array_equal(pair[pair[ids]], ids)
    # jitter stays inside +-0.2 h and boundary nodes are not moved
    xy = m.array("node_xy")
    h = 10.0 / 8
    gx, gy = np.meshgrid(np.arange(9) * h, np.arange(9) * h)
    assert np.max(np.abs(xy[0] - gx.ravel())) <= 0.2 * h + 1e-12
    onb = (gx.ravel() == 0) | (gx.ravel() == 10) | (gy.ravel() == 0) | (gy.ravel() == 10)
    assert np.all(xy[0][onb] == gx.ravel()[onb])
    cy = str(tmp_path / "cy.su2")
    fv.write_cylinder(cy, 16, 4)
    m = fv.Mesh.read_su2(cy, equation=2)
    assert m.N == 128 and sorted(m.array("boundary_type")) == [6002, 6013]
    r = np.hypot(*m.array("node_xy"))
    assert np.isclose(r.min(), 0.5) and np.isclose(r.max(), 20.0)


@pytest.mark.parametrize("n,jitter,seed", [(8, 0.2, 7), (24, 0.2, 20261203), (5, 0.0, 1), (2, 0.3, 3)])
def test_python_square_writer_is_byte_identical(tmp_path, n, jitter, seed):
    """oracle/meshgen.py (numpy only; the reference arm of bench.py makes its mesh with it,
    so that it never loads the CUDA library) writes the library writer's exact bytes."""
    from oracle import meshgen
    a, b = str(tmp_path / "lib.su2"), str(tmp_path / "py.su2")
    fv.write_periodic_square(a, n, 10.0, jitter, seed)
    meshgen.write_periodic_square(b, n, 10.0, jitter, seed)
    assert open(a, "rb").read() == open(b, "rb").read()


def test_errors_are_codes_not_exits(tmp_path):
    bad = tmp_path / "bad.su2"
    bad.write_text("NDIME= 3\n")
    with pytest.raises(fv.FvgbError) as e:
        fv.Mesh.read_su2(str(bad))
    assert e.value.code == -3
    with pytest.raises(fv.FvgbError) as e:
        fv.Mesh.read_su2(str(tmp_path / "missing.su2"))
    assert e.value.code == -2
    odd = tmp_path / "odd.su2"  # a periodic marker without its pair
    odd.write_text("NDIME= 2\nNELEM= 1\n5 0 1 2 0\nNPOIN= 3\n0 0 0\n1 0 1\n0 1 2\nNMARK= 1\n"
                   "MARKER_TAG= periodic_1\nMARKER_ELEMS= 1\n3 0 1\n")
    with pytest.raises(fv.FvgbError) as e:
        fv.Mesh.read_su2(str(odd))
    assert e.value.code == -4
    t = tmp_path / "x.toml"
    t.write_text("[constant]\ngamma = 1.4\n")
    with pytest.raises(fv.FvgbError) as e:
        fv.Params.from_toml(str(t))
    assert "missing" in str(e.value)


def test_cases_write_valid_toml(tmp_path):
    tp, sp = cases.vortex_small(str(tmp_path), n=8)
    p = fv.Params.from_toml(tp)
    assert (p.time_advance, p.reconstruct, p.CFL) == (3103, 3001, 0.5)


def test_channel_boundaries_and_inlet_tables(tmp_path):
    """Boundary names to types (BoundaryManager.cpp:15-48: "wall" is slip for Euler, no-slip
    adiabatic for Navier-Stokes) and the inlet / outlet tables in both input modes
    (TomlFileManager.cpp:200-265), against the oracle's reading of the same file."""
    sp = cases.channel_mesh(6, directory=str(tmp_path))
    assert list(fv.Mesh.read_su2(sp, equation=1).array("boundary_type")) == [6011, 6012, 6021, 6001]
    assert list(fv.Mesh.read_su2(sp, equation=2).array("boundary_type")) == [6011, 6012, 6021, 6002]
    tp = tmp_path / "ch.toml"
    tp.write_text(cases.toml_text(inlet=(0.4, 10.0), outlet=(1.2, 0.5, -0.1, 0.8)))
    p = fv.Params.from_toml(str(tp))
    q, _ = params_from_toml(str(tp))
    assert list(p.outlet) == [1.2, 0.5, -0.1, 0.8]
    assert np.allclose(list(p.inlet), list(q.inlet), rtol=1e-15, atol=0)
    # (Ma, AoA) with T0, p0 the stagnation state: flow at 10 degrees, static pressure below p0
    assert np.degrees(np.arctan2(p.inlet[2], p.inlet[1])) == pytest.approx(10.0, rel=1e-12)
    assert p.inlet[3] < 101325.0


def test_double_mach_reflection_and_shock_tube_inputs(tmp_path):
    """[initialCondition.doubleShockReflection] is required for type 4 and its angle must lie in
    [0, 90] (FieldInitializer.cpp:93-105); the shock tube's normal defaults to +x
    (FieldInitializer.h:23-26); both initial fields equal the oracle's."""
    from oracle.pyoracle import Oracle
    dmr = dict(ic_type=4, inlet=(8.0, 8.25, -30.0, 116.5, "angle"), outlet=(1.4, 0.0, 0.0, 1.0))
    tp = tmp_path / "dmr.toml"
    tp.write_text(cases.toml_text(**dmr))
    with pytest.raises(fv.FvgbError) as e:
        fv.Params.from_toml(str(tp))
    assert e.value.code == -3 and "doubleShockReflection" in str(e.value)
    tp.write_text(cases.toml_text(dmr=(0.2, 0.0, 95.0), **dmr))
    with pytest.raises(fv.FvgbError) as e:
        fv.Params.from_toml(str(tp))
    assert "shock_angle_degree" in str(e.value)
    sp = cases.dmr_mesh(24, jitter=0.2, directory=str(tmp_path))
    for angle in (60.0, 90.0, 35.0):
        tp.write_text(cases.toml_text(dmr=(1.0 / 6.0, 0.0, angle), **dmr))
        p = fv.Params.from_toml(str(tp))
        U = fv.initial_field(fv.Mesh.read_su2(sp, p), p)
        assert np.array_equal(U, Oracle(str(tp), sp).init_field()), angle
        assert 0 < np.count_nonzero(U[0] == 8.0) < U.shape[1]
    sod = dict(ic_type=3, inlet=(1.0, 0.0, 0.0, 1.0), outlet=(0.125, 0.0, 0.0, 0.1))
    sp = cases.channel_mesh(12, jitter=0.2, directory=str(tmp_path))
    for shock in (None, (4.0, 0.0, 0.0, 0.0), (5.0, 5.0, -0.6, 0.8)):
        tp.write_text(cases.toml_text(shock_tube=shock, **sod))
        p = fv.Params.from_toml(str(tp))
        U = fv.initial_field(fv.Mesh.read_su2(sp, p), p)
        assert np.array_equal(U, Oracle(str(tp), sp).init_field()), shock
    tp.write_text(cases.toml_text(**sod))
    p = fv.Params.from_toml(str(tp))
    assert list(p.shock) == [0.0, 0.0, 1.0, 0.0]
    U = fv.initial_field(fv.Mesh.read_su2(sp, p), p)
    assert np.all(U[0] == 0.125)  # every centroid lies at x > 0: downstream of the default shock


def test_steady_inputs(tmp_path):
    """time.is_steady = 1 (TomlFileManager.cpp:158-160): time.CFL_steady is required and
    time.CFL optional (default 0.6), and the step uses time.CFL, as the reference does;
    the batched form and the adjoint step in time only."""
    tp = tmp_path / "s.toml"
    tp.write_text(cases.toml_text(steady=True, CFL=None, CFL_steady=0.3))
    p = fv.Params.from_toml(str(tp))
    assert (p.steady, p.CFL, p.CFL_steady) == (1, 0.6, 0.3)
    q, _ = params_from_toml(str(tp))
    assert (q.steady, q.CFL) == (1, 0.6)
    tp.write_text(cases.toml_text(steady=True, CFL=0.45).replace("CFL_steady = 0.8\n", ""))
    with pytest.raises(fv.FvgbError) as e:
        fv.Params.from_toml(str(tp))
    assert "time.CFL_steady" in str(e.value)
    tp.write_text(cases.toml_text(CFL=None))
    with pytest.raises(fv.FvgbError) as e:
        fv.Params.from_toml(str(tp))
    assert "time.CFL" in str(e.value)
    tp.write_text(cases.toml_text(steady=True, CFL=0.45))
    p = fv.Params.from_toml(str(tp))
    assert (p.steady, p.CFL) == (1, 0.45)
    m = fv.Mesh.read_su2(cases.square_mesh(8, directory=str(tmp_path)), p)
    with pytest.raises(fv.FvgbError) as e:
        fv.Batch([m], [p])
    assert "is_steady" in str(e.value)


@pytest.mark.parametrize("base", ["channel", "square"])
def test_mixed_element_mesh_matches_the_oracle_reader(tmp_path, base):
    """Triangles and quads in one file (half of the quads written as two triangles on the
    other diagonal): this library's O(N) reader gives the oracle's arrays, which follow the
    reference's legacy assembly, bit for bit."""
    from oracle.pyoracle import Oracle
    src = (cases.channel_mesh if base == "channel" else cases.square_mesh)(10, jitter=0.2, directory=str(tmp_path))
    su2 = cases.mixed_mesh(src, str(tmp_path / f"mixed_{base}.su2"))
    assert "\n5 " in open(su2).read() and "\n9 " in open(su2).read()
    tp, _ = cases.vortex_small(str(tmp_path), n=4)
    p = fv.Params.from_toml(tp)
    m = fv.Mesh.read_su2(su2, p)
    o = Oracle(tp, su2)
    assert (m.N, m.E) == (o.N, o.E)
    for mine, theirs in (("elem_edges", "elem_edges"), ("elem_nodes", "elem_nodes"),
                         ("elem_neighbors", "elem_nbrs"), ("edge_L", "edge_L"), ("edge_R", "edge_R"),
                         ("edge_setID", "edge_set"), ("elem_volume", "elem_vol"), ("elem_xy", "elem_xy")):
        a, b = np.asarray(m.array(mine)), o.array(theirs)
        assert np.array_equal(a.reshape(b.shape), b), mine


def test_create_refuses_bad_meshes_on_the_host(tmp_path):
    """fvgb_create checks the caller's mesh before it looks for a device: an empty mesh,
    a NULL array and an index outside the mesh are FVGB_ERR_MESH (-4) here, without a
    GPU; a good mesh gets as far as the device check (-10 without a GPU)."""
    L = fv.lib()
    tp, su2 = cases.vortex_small(str(tmp_path), n=6)
    p = fv.Params.from_toml(tp)
    m = fv.Mesh.read_su2(su2, p)

    def create(soa):
        h = ctypes.c_void_p()
        rc = L.fvgb_create(ctypes.byref(soa), ctypes.byref(p), ctypes.byref(h))
        if rc == 0:
            L.fvgb_destroy(h)
        return rc, L.fvgb_last_error().decode()

    def copy():
        soa = fv.MeshSoA()
        ctypes.memmove(ctypes.byref(soa), ctypes.byref(m.soa), ctypes.sizeof(soa))
        return soa

    empty = fv.MeshSoA()
    assert create(empty) == (-4, "mesh has no cells")
    soa = copy()
    soa.edge_normal = None
    assert create(soa) == (-4, "a mesh array is NULL")
    keep = []
    for name, index, value in (("edge_L", 3, m.N), ("edge_R", 0, -2), ("edge_setID", m.E - 1, m.NB + 1),
                               ("elem_edges", 5, m.E), ("elem_neighbors", 2, m.N)):
        arr = np.ascontiguousarray(m.array(name)).copy()
        arr.reshape(-1)[index] = value
        keep.append(arr)
        soa = copy()
        setattr(soa, name, arr.ctypes.data)
        rc, msg = create(soa)
        assert rc == -4 and "outside" in msg, (name, rc, msg)
    if not torch_cuda_available():
        assert create(copy())[0] == -10


def torch_cuda_available():
    try:
        import torch
        return torch.cuda.is_available()
    except ImportError:
        return False


def test_rhs_noalloc_refuses_null_mesh_arrays():
    """fvgb_rhs_noalloc reads the caller's device arrays; a NULL among them is refused on the
    host before anything is launched (no GPU needed to see it)."""
    L = fv.lib()
    L.fvgb_rhs_noalloc.restype = ctypes.c_int
    L.fvgb_rhs_noalloc.argtypes = [ctypes.POINTER(fv.MeshSoA), ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                   ctypes.c_void_p]
    p = fv.Params.default()
    p.reconstruct, p.equation, p.flux_scheme = 3001, 1, 2002
    soa = fv.MeshSoA()
    soa.num_element, soa.num_edge, soa.num_boundary = 4, 6, 1
    dummy = ctypes.c_double()
    rc = L.fvgb_rhs_noalloc(ctypes.byref(soa), ctypes.addressof(p), ctypes.addressof(dummy), ctypes.addressof(dummy),
                            None)
    assert rc == -1 and "NULL" in L.fvgb_last_error().decode()


class _RoutineControllerStatement:
    """The reference's adaptive CFL, restated from its rules (RoutineController.cpp:13-90)."""

    def __init__(self):
        self.calls, self.record = 0, 10.0
        self.last = {"inc": 0, "dec": 0}
        self.cold = {"inc": 1000, "dec": 500}

    def _try(self, which, cfl, step, factor):
        if step - self.last[which] >= self.cold[which]:
            self.last[which] = step
            return cfl * factor, True
        return cfl, False

    def apply(self, res, step, cfl):
        ok = False
        if self.calls == 0:
            self.record = res
        else:
            if step > 1000 and res > self.record * 10.0:
                cfl, a = self._try("dec", cfl, step, 0.75)
                ok |= a
            if step > 5000 and res < self.record * 0.5:
                cfl, a = self._try("inc", cfl, step, 1.1)
                if a:
                    self.record *= 0.9
                ok |= a
            if step > 5000:
                cfl, a = self._try("inc", cfl, step, 1.05)
                ok |= a
            cfl = max(cfl, 0.5)
        self.calls += 1
        return cfl, ok


def test_adaptive_cfl_controller_follows_the_reference_rules():
    L = fv.lib()
    L.fvgb_cfl_controller_create.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)]
    L.fvgb_cfl_controller_apply.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_int,
                                            ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int)]
    L.fvgb_cfl_controller_destroy.argtypes = [ctypes.c_void_p]
    L.fvgb_cfl_controller_destroy.restype = None
    rng = np.random.default_rng(4)
    for trial in range(6):
        c = ctypes.c_void_p()
        assert L.fvgb_cfl_controller_create(1, ctypes.byref(c)) == 0
        ref = _RoutineControllerStatement()
        cfl = ctypes.c_double(0.8)
        cfl_ref, changes = 0.8, 0
        res = 1e-2
        for step in [1] + list(range(50, 12001, 50)):
            # residual histories that fall, jump up by orders of magnitude, and stall
            res *= float(np.exp(rng.normal(-0.02, 0.3))) * (30.0 if rng.random() < 0.02 else 1.0)
            applied = ctypes.c_int()
            assert L.fvgb_cfl_controller_apply(c, res, step, ctypes.byref(cfl), ctypes.byref(applied)) == 0
            cfl_ref, ok = ref.apply(res, step, cfl_ref)
            assert cfl.value == cfl_ref and bool(applied.value) == ok, (trial, step)
            changes += ok
        assert changes > 3
        L.fvgb_cfl_controller_destroy(c)
    c = ctypes.c_void_p()
    assert L.fvgb_cfl_controller_create(0, ctypes.byref(c)) == 0  # strategy 0 never changes CFL
    cfl = ctypes.c_double(0.8)
    for step in range(1, 20000, 97):
        L.fvgb_cfl_controller_apply(c, 1e3 * step, step, ctypes.byref(cfl), None)
    assert cfl.value == 0.8
    L.fvgb_cfl_controller_destroy(c)
    assert L.fvgb_cfl_controller_create(2, ctypes.byref(c)) == -1


def test_time_strategy_key(tmp_path):
    tp = tmp_path / "s.toml"
    tp.write_text(cases.toml_text().replace("[time]\n", "[time]\nstrategy = 1\n"))
    assert fv.run_config(str(tp))["time_strategy"] == 1
    tp.write_text(cases.toml_text().replace("[time]\n", "[time]\nstrategy = 3\n"))
    with pytest.raises(fv.FvgbError):
        fv.run_config(str(tp))


def test_dimension_other_than_2_is_refused(tmp_path):
    tp = tmp_path / "d.toml"
    tp.write_text(cases.toml_text().replace("dimension = 2", "dimension = 3"))
    with pytest.raises(fv.FvgbError) as e:
        fv.Params.from_toml(str(tp))
    assert "dimension" in str(e.value)
