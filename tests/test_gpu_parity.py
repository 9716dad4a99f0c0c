"""Parity of the CUDA path (through the C ABI) with the reference: against the
golden fixtures the reference produced, against the oracle on the same inputs
at larger sizes, and through size-independent properties at full size.

Tolerances are relative L-infinity norms, ||a - b||_inf / ||b||_inf, in FP64:
  residual, gradients, dt of one evaluation     1e-12 (gradients: relative to the
                                                larger of ||b||_inf and max|U| / h)
  state after <= 20 steps                       1e-12
  state after 1000 steps (64x64 vortex)         1e-9
  second-order limited runs (<= 10 steps)       1e-10
  second-order limited runs (200 steps)         1e-9 (measured 5e-15 .. 7e-15)
"""
import numpy as np
import pytest

import cfd_solver_2d_gpu_gb300 as fv
from cfd_solver_2d_gpu_gb300 import cases
from golden import make_golden
from oracle.pyoracle import Oracle

pytestmark = pytest.mark.gpu
NAMES = make_golden.names()


def rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def rel_grad(a, b, U, vol):
    """Gradients relative to the larger of their own maximum and the field's scale
    max|U| / sqrt(mean cell area): where every gradient is limited away or the field is
    piecewise uniform, both sides hold round-off alone (the reference's Green-Gauss sums
    leave ~1e-14 where this library's give exact zeros)."""
    scale = max(np.max(np.abs(b)), np.max(np.abs(U)) / np.sqrt(np.mean(vol)))
    return float(np.max(np.abs(a - b)) / scale)


def make(tp, sp, renumber=1):
    p = fv.Params.from_toml(tp)
    p.renumber = renumber
    m = fv.Mesh.read_su2(sp, p)
    return fv.GPUSolver2(m, p), p, m


@pytest.fixture(scope="module", params=NAMES)
def golden(request):
    return request.param, make_golden.load(request.param)


def test_residual_matches_reference(golden):
    name, (tp, sp, g) = golden
    s, p, m = make(tp, sp)
    R, gx, gy = s.rhs(g["U0"], gradients=True)
    assert rel(R, g["rhs"]) <= 1e-12, name
    if p.reconstruct == 3002 or p.equation == 2:
        assert rel_grad(gx, g["grad_x"], g["U0"], g["elem_vol"]) <= 1e-12, name
        assert rel_grad(gy, g["grad_y"], g["U0"], g["elem_vol"]) <= 1e-12, name
    s.set_state(g["U0"])
    assert abs(s.dt() - g["dt"][0]) <= 1e-12 * g["dt"][0], name


def test_steps_match_reference(golden):
    name, (tp, sp, g) = golden
    s, p, m = make(tp, sp)
    s.set_state(g["U0"])
    n = int(g["steps"][0])
    t = s.step(0.0, p.T_end, n)
    U = s.get_state()
    tol = 1e-9 if n >= 1000 else (1e-10 if p.reconstruct == 3002 else 1e-12)
    assert rel(U, g["U"]) <= tol, (name, rel(U, g["U"]))
    assert abs(t - g["t"][0]) <= 1e-11 * g["t"][0]


def test_residual_norms_match_reference(golden):
    """fvgb_residual, the replacement of GPUSolver2::updateResidualVector over
    get_residual_host (FVMR/src/output/residual/Residual.cpp:4-43), against the
    reference's own norms (L-infinity, L1, L2) stored in the fixture: of one residual
    evaluation, at 1e-12; and of the last residual of the fixture's steps (Euler, Kutta
    RK3, SSP-RK3 and steady runs), at the tolerance of the state after those steps scaled
    by the residual's sensitivity (the residual of a state that differs by d differs by
    about d / h), and against the oracle's norms of the oracle's last residual, which the
    oracle computes the reference's way, at the same tolerance."""
    name, (tp, sp, g) = golden
    s, p, m = make(tp, sp)
    s.rhs(g["U0"])
    for norm in (0, 1, 2):
        assert rel(s.update_residual_vector(norm), g["residual_rhs"][norm]) <= 1e-12, (name, norm)
    n = int(g["steps"][0])
    s.set_state(g["U0"])
    s.step(0.0, p.T_end, n)
    o = Oracle(tp, sp)
    _, _, _, last = o.run(g["U0"], n)
    tol = 1e-7 if n >= 1000 else (1e-8 if p.reconstruct == 3002 else 1e-10)
    for norm in (0, 1, 2):
        got = s.update_residual_vector(norm)
        assert rel(got, g["residual_step"][norm]) <= tol, (name, norm, rel(got, g["residual_step"][norm]))
        assert np.array_equal(o.residual(last, norm), g["residual_step"][norm]) or \
            rel(o.residual(last, norm), g["residual_step"][norm]) <= 1e-14, (name, norm)


def test_residual_norm_is_nan_when_a_residual_is(tmp_path):
    """A NaN anywhere in the residual makes the L-infinity norm NaN, whichever cell holds it,
    so that the driver's NaN stop (CDriver.cpp:235-263) fires; L1 and L2 sums carry it too."""
    tp, su2 = cases.vortex_small(str(tmp_path), n=32)
    s, p, m = make(tp, su2)
    U = s.get_state()
    for cell in (0, m.N // 2, m.N - 1):
        V = U.copy()
        V[1, cell] = np.nan
        s.rhs(V)
        for norm in (0, 1, 2):
            assert np.isnan(s.update_residual_vector(norm)[1]), (cell, norm)
    s.rhs(U)
    assert np.all(np.isfinite(s.update_residual_vector(0)))


def test_connectivity_maps_back_bit_exact(golden):
    name, (tp, sp, g) = golden
    s, p, m = make(tp, sp, renumber=1)
    ee, nb, eL, eR = s.layout_connectivity()
    N = m.N
    ref_ee = g["elem_edges"].reshape(4, N)[:3]
    ref_nb = g["elem_nbrs"].reshape(4, N)[:3]
    assert np.array_equal(ee, ref_ee)
    compact = np.full_like(ref_nb, -1)  # the device keeps valid neighbours first, in slot order
    for c in range(N):
        v = ref_nb[:, c][ref_nb[:, c] >= 0]
        compact[: len(v), c] = v
    assert np.array_equal(nb, compact)
    assert np.array_equal(eL, g["edge_L"]) and np.array_equal(eR, g["edge_R"])
    perm = s.cell_permutation()
    assert np.array_equal(np.sort(perm), np.arange(N))


def test_renumbering_does_not_change_the_answer():
    tp, sp, g = make_golden.load("jvortex24_roe_lsq_barth_ssp")
    a, p, _ = make(tp, sp, renumber=0)
    b, _, _ = make(tp, sp, renumber=1)
    for s in (a, b):
        s.set_state(g["U0"])
        s.step(0.0, p.T_end, 5)
    assert rel(a.get_state(), b.get_state()) <= 1e-12


def test_deterministic_bitwise():
    tp, sp, g = make_golden.load("cylinder32_ns_lsq_barth_rk3")
    s, p, _ = make(tp, sp)
    out = []
    for _ in range(2):
        s.set_state(g["U0"])
        s.step(0.0, p.T_end, 5)
        out.append(s.get_state())
    assert np.array_equal(out[0], out[1])


@pytest.mark.parametrize("cfg", [
    dict(flux=2002, reconstruct=3002, gradient=1, limiter=1, time_advance=3104, CFL=0.8),
    dict(flux=2001, reconstruct=3002, gradient=1, limiter=1, time_advance=3104, CFL=0.8),
    dict(flux=2002, reconstruct=3002, gradient=1, limiter=1, time_advance=3104, CFL=0.8, lsq_det="fixed"),
    dict(flux=2002, reconstruct=3002, gradient=2, limiter=1, time_advance=3103, CFL=0.8),
])
def test_against_oracle_128(tmp_path, cfg):
    """128x128 jittered vortex (32,768 cells): oracle and CUDA path on the same inputs."""
    su2 = cases.square_mesh(128, jitter=0.2, directory=str(tmp_path))
    tp = tmp_path / "c.toml"
    tp.write_text(cases.toml_text(**cfg))
    o = Oracle(str(tp), su2)
    s, p, _ = make(str(tp), su2)
    U0 = o.init_field()
    R, gx, _ = o.rhs(U0)
    Rg, gxg, _ = s.rhs(U0, gradients=True)
    assert rel(Rg, R) <= 1e-12 and rel(gxg, gx) <= 1e-12
    U, t, _, _ = o.run(U0, 3)
    s.set_state(U0)
    s.step(0.0, p.T_end, 3)
    assert rel(s.get_state(), U) <= 1e-10


def vortex_density(xy, t, gamma=1.4, chi=5.0, L=10.0):
    """The isentropic vortex of strength chi started at (5, 5), carried by the freestream
    (1, 1) to time t on the periodic L x L square (nearest image), at the points xy[2][N]."""
    d = [(xy[k] - (5.0 + t)) for k in (0, 1)]
    d = [di - L * np.round(di / L) for di in d]
    r2 = d[0] ** 2 + d[1] ** 2
    T = 1.0 - (gamma - 1.0) * chi ** 2 / (8.0 * gamma * np.pi ** 2) * np.exp(1.0 - r2)
    return T ** (1.0 / (gamma - 1.0))


@pytest.mark.parametrize("flux", [2002, 2001])
def test_second_order_200_steps(tmp_path, flux):
    """64x64 jittered vortex, LSQ + Barth, SSP-RK3, CFL 0.8, 200 steps: the state's drift
    from the oracle stays at round-off level (measured on a GB300: 6.5e-15 Roe, 5.2e-15 LLF;
    the bound, 1e-9, leaves room for a limiter branch that round-off flips), and both
    sides have the same error against the exact vortex (3.5e-3 Roe, 3.4e-3 LLF, L1 of
    density at t = 0.344)."""
    su2 = cases.square_mesh(64, jitter=0.2, directory=str(tmp_path))
    tp = tmp_path / "c.toml"
    tp.write_text(cases.toml_text(flux=flux, reconstruct=3002, gradient=1, limiter=1, time_advance=3104, CFL=0.8))
    o = Oracle(str(tp), su2)
    s, p, m = make(str(tp), su2)
    U0 = o.init_field()
    U, t, _, _ = o.run(U0, 200)
    s.set_state(U0)
    tg = s.step(0.0, p.T_end, 200)
    Ug = s.get_state()
    drift = rel(Ug, U)
    print(f"flux {flux}: t = {t:.6f}, drift after 200 steps {drift:.3e}")
    assert abs(tg - t) <= 1e-11 * t
    assert drift <= 1e-9, drift
    vol, xy = m.array("elem_volume"), m.array("elem_xy")
    exact = vortex_density(xy, t)
    err_o = float(np.sum(np.abs(U[0] - exact) * vol) / np.sum(vol))
    err_g = float(np.sum(np.abs(Ug[0] - exact) * vol) / np.sum(vol))
    print(f"flux {flux}: L1 density error against the exact vortex: oracle {err_o:.6e}, CUDA {err_g:.6e}")
    assert abs(err_g - err_o) <= 1e-9 * err_o
    assert err_g < 1e-2


@pytest.mark.parametrize("size", [(128, 64), (512, 256)])
def test_against_oracle_cylinder_ns(tmp_path, size):
    """Laminar cylinder O-grid at Re 100, Ma 0.2, LSQ + Barth, Kutta RK3: 128 x 64 and the
    full 512 x 256 (262,144 cells) workload of the Navier-Stokes bench line."""
    import os
    from oracle import pyoracle
    tp, su2 = cases.cylinder_ns(str(tmp_path), *size)
    o = Oracle(tp, su2)
    s, p, _ = make(tp, su2)
    U0 = o.init_field()
    assert rel(s.rhs(U0), o.rhs(U0)[0]) <= 1e-12
    before = pyoracle.set_threads(0)
    pyoracle.set_threads(os.cpu_count() or 1)
    try:
        U, t, _, _ = o.run(U0, 3)
    finally:
        pyoracle.set_threads(before)
    s.set_state(U0)
    s.step(0.0, p.T_end, 3)
    assert rel(s.get_state(), U) <= 1e-11


def test_positivity_pass_matches_oracle(tmp_path):
    """A cell whose density is out of range is replaced by the neighbour mean, as the reference does."""
    tp, sp, g = make_golden.load("vortex16_roe_o1_euler")
    o = Oracle(tp, sp)
    s, p, m = make(tp, sp)
    U0 = g["U0"].copy()
    U0[:, 100] = [1e-12, 0.0, 0.0, 1.0]   # rho below RHO_MIN
    U0[:, 101] = [500.0, 0.0, 0.0, 1e3]   # rho above RHO_MAX, a neighbour of 100
    U, _, _, _ = o.run(U0, 1)
    s.set_state(U0)
    s.step(0.0, p.T_end, 1)
    assert rel(s.get_state(), U) <= 1e-12
    assert s.device_status()[0] >= 1


def test_nan_is_an_error_code_not_a_crash():
    tp, sp, g = make_golden.load("vortex16_roe_o1_euler")
    s, p, _ = make(tp, sp)
    U0 = g["U0"].copy()
    U0[0, 7] = np.nan
    s.set_state(U0)
    with pytest.raises(fv.FvgbError) as e:
        s.step(0.0, p.T_end, 1)
    assert e.value.code == -6
    s.set_state(g["U0"])  # the handle stays usable
    s.step(0.0, p.T_end, 1)


def test_full_size_step_matches_the_oracle(tmp_path):
    """The bench workload itself, 1448x1448 jittered vortex (4,193,408 cells), LSQ + Barth,
    Roe, SSP-RK3, CFL 0.8: the residual and one step against the oracle on the same
    inputs (the oracle's loops on all host threads, a few seconds)."""
    import os
    from oracle import pyoracle
    tp, su2 = cases.vortex_large(str(tmp_path))
    before = pyoracle.set_threads(0)  # 0 only reads the count
    pyoracle.set_threads(os.cpu_count() or 1)
    try:
        o = Oracle(tp, su2)
        s, p, m = make(tp, su2)
        U0 = o.init_field()
        assert rel(s.rhs(U0), o.rhs(U0)[0]) <= 1e-12
        U, t, _, _ = o.run(U0, 1)
    finally:
        pyoracle.set_threads(before)
    s.set_state(U0)
    tg = s.step(0.0, p.T_end, 1)
    assert abs(tg - t) <= 1e-12 * t
    assert rel(s.get_state(), U) <= 1e-12


@pytest.mark.parametrize("flux", [2002, 2001])
def test_full_size_200_steps_match_the_oracle(tmp_path, flux):
    """The large plain configuration at its own horizon: 1448x1448 jittered vortex
    (4,193,408 cells), LSQ + Barth, Roe and LLF, SSP-RK3, CFL 0.8, 200 steps on the GPU
    against 200 steps of the oracle on all host threads (about a minute on 16 cores).
    The bound is the 1000-step tolerance, 1e-9; the measured drift is printed."""
    import os
    from oracle import pyoracle
    tp, su2 = cases.vortex_large(str(tmp_path), flux=flux)
    before = pyoracle.set_threads(0)
    pyoracle.set_threads(os.cpu_count() or 1)
    try:
        o = Oracle(tp, su2)
        U0 = o.init_field()
        U, t, _, _ = o.run(U0, 200)
    finally:
        pyoracle.set_threads(before)
    s, p, m = make(tp, su2)
    s.set_state(U0)
    tg = s.step(0.0, p.T_end, 200)
    drift = rel(s.get_state(), U)
    print(f"1448^2 flux {flux}: t = {t:.6f}, drift after 200 steps {drift:.3e}")
    assert abs(tg - t) <= 1e-11 * t
    assert drift <= 1e-9, drift


def test_large_mesh_properties(tmp_path):
    """1448x1448 jittered vortex (4,193,408 cells), second order, SSP-RK3: total mass
    and energy are conserved on the periodic domain and the residual is finite."""
    tp, su2 = cases.vortex_large(str(tmp_path))
    s, p, m = make(tp, su2)
    vol = m.array("elem_volume")
    U0 = s.get_state()
    mass0 = np.dot(vol, U0[0])
    s.step(0.0, p.T_end, 3)
    U = s.get_state()
    assert np.all(np.isfinite(U))
    assert abs(np.dot(vol, U[0]) - mass0) <= 1e-12 * mass0
    assert abs(np.dot(vol, U[3]) - np.dot(vol, U0[3])) <= 1e-12 * np.dot(vol, U0[3])
    res = s.update_residual_vector()
    assert np.all(np.isfinite(res)) and res[0] > 0


def test_pinned_host_buffers_match_pageable(tmp_path):
    """fvgb_set_state / fvgb_get_state with page-locked buffers (read and written by the
    permuting kernels directly over the host link) give the same state as pageable ones."""
    torch = pytest.importorskip("torch")
    tp, su2 = cases.vortex_small(str(tmp_path), n=32)
    p = fv.Params.from_toml(tp)
    m = fv.Mesh.read_su2(su2, p)
    a, b = fv.GPUSolver2(m, p), fv.GPUSolver2(m, p)
    U0 = a.get_state() * np.random.default_rng(3).uniform(0.99, 1.01, (4, m.N))  # the vortex, perturbed
    pin = torch.from_numpy(U0.copy()).pin_memory()
    a.set_state(U0)
    b.set_state_ptr(pin.data_ptr())
    pin.zero_()  # set_state returned: the buffer may be reused at once
    a.step(0.0, p.T_end, 3)
    b.step(0.0, p.T_end, 3)
    out = torch.empty((4, m.N), dtype=torch.float64).pin_memory()
    b.get_state_ptr(out.data_ptr())
    assert np.array_equal(a.get_state(), out.numpy())


def test_bad_mesh_indices_are_refused(tmp_path):
    """Indices outside the caller's arrays (an edge's cell, a cell's edge, a boundary set) are
    refused with FVGB_ERR_MESH before anything is built or launched."""
    import ctypes
    tp, su2 = cases.vortex_small(str(tmp_path), n=6)
    p = fv.Params.from_toml(tp)
    m = fv.Mesh.read_su2(su2, p)
    for name, index, value in (("edge_L", 3, m.N), ("edge_R", 0, -2), ("edge_setID", m.E - 1, m.NB + 1),
                               ("elem_edges", 5, m.E)):
        arr = np.ascontiguousarray(m.array(name)).copy()
        arr.reshape(-1)[index] = value
        soa = fv.MeshSoA()
        ctypes.memmove(ctypes.byref(soa), ctypes.byref(m.soa), ctypes.sizeof(soa))
        setattr(soa, name, arr.ctypes.data)
        h = ctypes.c_void_p()
        rc = fv.lib().fvgb_create(ctypes.byref(soa), ctypes.byref(p), ctypes.byref(h))
        assert rc == -4 and "outside" in fv.lib().fvgb_last_error().decode(), name


@pytest.mark.parametrize("base,scheme", [("channel", "euler_lsq_roe"), ("square", "euler_lsq_roe"),
                                         ("channel", "ns_gg_llf"), ("square", "ns_lsq_roe")])
def test_mixed_element_mesh_matches_the_oracle(tmp_path, base, scheme):
    """Triangles and quads in one file (half of the quads written as two triangles on the
    other diagonal): residual and 5 SSP-RK3 steps, second order, against the oracle; Euler
    and laminar Navier-Stokes (Re 100), least squares and Green-Gauss, Roe and LLF."""
    src = (cases.channel_mesh if base == "channel" else cases.square_mesh)(16, jitter=0.2, directory=str(tmp_path))
    su2 = cases.mixed_mesh(src, str(tmp_path / f"mixed_{base}.su2"))
    tp = str(tmp_path / "mixed.toml")
    extra = dict(vortex=(2.5, 7.0, 3.0), inf=(1.0, 1.0, 0.3, 1.0), inlet=(1.0, 1.0, 0.3, 1.0),
                 outlet=(1.0, 1.0, 0.0, 0.9)) if base == "channel" else {}
    extra.update({"euler_lsq_roe": dict(flux=2002, gradient=1),
                  "ns_gg_llf": dict(equation=2, Re=100.0, flux=2001, gradient=2),
                  "ns_lsq_roe": dict(equation=2, Re=100.0, flux=2002, gradient=1)}[scheme])
    with open(tp, "w") as f:
        f.write(cases.toml_text(reconstruct=3002, limiter=1, time_advance=3104, CFL=0.6, **extra))
    s, p, m = make(tp, su2)
    o = Oracle(tp, su2)
    U0 = cases.wavy(m, o.init_field())
    assert rel(s.rhs(U0), o.rhs(U0)[0]) <= 1e-12
    U, _, _, _ = o.run(U0, 5)
    s.set_state(U0)
    s.step(0.0, p.T_end, 5)
    assert rel(s.get_state(), U) <= 1e-10


@pytest.mark.parametrize("kind", ["square2", "square3", "channel2"])
@pytest.mark.parametrize("second_order", [False, True])
def test_tiny_meshes_match_the_oracle(tmp_path, kind, second_order):
    """The smallest meshes the writers make: 8 and 18 triangles on the periodic square (a
    cell's periodic faces wrap onto cells it also meets inside) and the 8-triangle channel,
    every cell of which touches a boundary."""
    n = int(kind[-1])
    su2 = (cases.square_mesh if kind.startswith("square") else cases.channel_mesh)(n, directory=str(tmp_path))
    tp = str(tmp_path / "tiny.toml")
    with open(tp, "w") as f:
        f.write(cases.toml_text(flux=2002, reconstruct=3002 if second_order else 3001, gradient=1, limiter=1,
                                time_advance=3104, CFL=0.5))
    s, p, m = make(tp, su2)
    o = Oracle(tp, su2)
    U0 = cases.wavy(m, o.init_field())
    s.set_state(U0)
    s.step(0.0, p.T_end, 4)
    o.params.time_advance = 3104
    Uo, _, _, _ = o.run(U0, 4)
    assert rel(s.get_state(), Uo) <= 1e-12
