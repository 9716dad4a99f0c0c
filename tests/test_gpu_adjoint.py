"""The discrete adjoint (fvgb_adjoint_forward / fvgb_adjoint_backward) against
central finite differences of the same forward map (step 1e-6, random unit
directions), against finite differences of the oracle's forward map (the
reference gradient), under different checkpoint counts, and through the
torch.autograd.Function wrapper.

Loss: L = 1/2 sum_c (rho_K(c) - rho_target(c))^2, the target being the
forward solution from a perturbed initial state (vortex strength and centre
shifted by seeded amounts).

The forward map is only piecewise smooth: the Barth limiter's min(1, .) and
its choice of vertex, and the argmin cell of the global time step, switch
branch where two candidates tie. The isentropic vortex is uniform to ~1e-11
away from its core and a regular mesh gives equal time steps in many cells,
so a finite-difference step of 1e-6 crosses branches there and the difference
quotient is no derivative. The test states therefore carry a smooth wave on
top of the vortex everywhere, and the meshes are jittered."""
import numpy as np
import pytest

import cfd_solver_2d_gpu_gb300 as fv
from cfd_solver_2d_gpu_gb300 import adjoint_backward, adjoint_forward, cases
from oracle.pyoracle import Oracle

pytestmark = pytest.mark.gpu
H = 1e-6


def setup_case(tmp_path, n=24, jitter=0.2, time_advance=3104, reconstruct=3002, limiter=1, walls=False, CFL=0.8,
               flux=2002, gradient=1):
    su2 = cases.square_mesh(n, jitter=jitter, directory=str(tmp_path))
    if walls:  # periodic left/right, slip walls top and bottom
        text = open(su2).read().replace("MARKER_TAG= periodic_2", "MARKER_TAG= wall")
        su2 = str(tmp_path / f"channel_{n}.su2")
        open(su2, "w").write(text)
    tp = str(tmp_path / f"adj_{n}_{time_advance}_{reconstruct}_{limiter}_{walls}_{flux}_{gradient}.toml")
    with open(tp, "w") as f:
        f.write(cases.toml_text(flux=flux, reconstruct=reconstruct, gradient=gradient, limiter=limiter,
                                time_advance=time_advance, CFL=CFL))
    p = fv.Params.from_toml(tp)
    mesh = fv.Mesh.read_su2(su2, p)
    solver = fv.GPUSolver2(mesh, p)
    U0 = cases.wavy(mesh, solver.get_state())
    # target: vortex strength 5 (1 + 0.02 r1), centre (5 + 0.1 r2, 5 + 0.1 r3)
    rng = np.random.default_rng(7)
    r = rng.uniform(-1, 1, 3)
    pt = fv.Params.from_toml(tp)
    pt.vortex[0], pt.vortex[1], pt.vortex[2] = 5 + 0.1 * r[1], 5 + 0.1 * r[2], 5 * (1 + 0.02 * r[0])
    Ut0 = cases.wavy(mesh, fv.initial_field(mesh, pt))
    return tp, su2, p, mesh, solver, U0, Ut0


def forward(solver, p, U0, K):
    solver.set_state(U0)
    solver.step(0.0, p.T_end, K)
    return solver.get_state()


def loss_seed(UK, rho_t):
    d = UK[0] - rho_t
    seed = np.zeros_like(UK)
    seed[0] = d
    return 0.5 * float(np.dot(d, d)), seed


def fd_check(solver, p, U0, rho_t, K, ndir, seed_rng=11, nck=None):
    UK, _ = adjoint_forward(solver, U0, K, nck)
    L0, seed = loss_seed(UK, rho_t)
    g, _ = adjoint_backward(solver, seed)
    rng = np.random.default_rng(seed_rng)
    errs = []
    for _ in range(ndir):
        d = rng.standard_normal(U0.shape)
        d /= np.linalg.norm(d)
        Lp, _ = loss_seed(forward(solver, p, U0 + H * d, K), rho_t)
        Lm, _ = loss_seed(forward(solver, p, U0 - H * d, K), rho_t)
        fd = (Lp - Lm) / (2 * H)
        ad = float(np.sum(g * d))
        errs.append(abs(fd - ad) / max(abs(fd), 1e-30))
    return np.array(errs), g


def test_adjoint_matches_fd_second_order_ssp(tmp_path):
    tp, su2, p, mesh, solver, U0, Ut0 = setup_case(tmp_path)
    K = 10
    rho_t = forward(solver, p, Ut0, K)[0]
    errs, _ = fd_check(solver, p, U0, rho_t, K, 8)
    print(f"FD relative errors: median {np.median(errs):.2e} max {errs.max():.2e} over {len(errs)} directions")
    assert np.median(errs) <= 1e-6 and errs.max() <= 2e-5, errs  # measured: median 1.3e-7, max 2.3e-6


def test_adjoint_matches_fd_first_order_euler(tmp_path):
    tp, su2, p, mesh, solver, U0, Ut0 = setup_case(tmp_path, n=16, time_advance=3101, reconstruct=3001, CFL=0.5)
    K = 8
    rho_t = forward(solver, p, Ut0, K)[0]
    errs, _ = fd_check(solver, p, U0, rho_t, K, 6)
    print(f"FD relative errors: median {np.median(errs):.2e} max {errs.max():.2e} over {len(errs)} directions")
    assert errs.max() <= 1e-6, errs


def test_adjoint_slip_walls(tmp_path):
    tp, su2, p, mesh, solver, U0, Ut0 = setup_case(tmp_path, n=16, walls=True, limiter=0, CFL=0.5)
    K = 6
    rho_t = forward(solver, p, Ut0, K)[0]
    errs, _ = fd_check(solver, p, U0, rho_t, K, 6)
    print(f"FD relative errors: median {np.median(errs):.2e} max {errs.max():.2e} over {len(errs)} directions")
    assert np.median(errs) <= 1e-7 and errs.max() <= 1e-6, errs  # measured: median 8.5e-9, max 1.6e-8


def test_checkpoints_do_not_change_the_gradient(tmp_path):
    tp, su2, p, mesh, solver, U0, Ut0 = setup_case(tmp_path, n=16)
    K = 9
    rho_t = forward(solver, p, Ut0, K)[0]
    grads = []
    for nck in (1, 3, 9):
        UK, _ = adjoint_forward(solver, U0, K, nck)
        _, seed = loss_seed(UK, rho_t)
        g, _ = adjoint_backward(solver, seed)
        grads.append(g)
    assert np.array_equal(grads[0], grads[1]) and np.array_equal(grads[1], grads[2])


@pytest.mark.parametrize("kind", ["ssp_lsq_barth", "kutta_gg", "euler_o1", "ns_vortex"])
def test_overlapped_sweep_is_bitwise_the_sequential_one(tmp_path, kind):
    """The backward sweep with each segment's recomputation on the solver's stream beside the
    reverse of the next segment (two sets of records, one graph with two branches) against the
    sweep that recomputes and reverses one after the other: the same kernels on the same data,
    so the gradient is bitwise equal.  Seven steps in segments of 3, 3 and 1; a second backward
    after the first (the forward's last segment no longer kept) gives the same gradient."""
    from cfd_solver_2d_gpu_gb300 import adjoint_overlap
    if kind == "ns_vortex":
        su2 = cases.square_mesh(16, jitter=0.2, directory=str(tmp_path))
        text = cases.toml_text(equation=2, flux=2002, reconstruct=3002, gradient=1, limiter=1, time_advance=3104,
                               CFL=0.6, Re=100.0)
        p, solver, U0, Ut0 = boundary_case(tmp_path, kind, text, su2)
    else:
        ta, rc, gr, lim = {"ssp_lsq_barth": (3104, 3002, 1, 1), "kutta_gg": (3103, 3002, 2, 1),
                           "euler_o1": (3101, 3001, 1, 0)}[kind]
        tp, su2, p, mesh, solver, U0, Ut0 = setup_case(tmp_path, n=16, time_advance=ta, reconstruct=rc, gradient=gr,
                                                       limiter=lim)
    K = 7
    rho_t = forward(solver, p, Ut0, K)[0]
    out = {}
    for mode in (1, 0):
        adjoint_overlap(solver, mode)
        UK, _ = adjoint_forward(solver, U0, K, 3)
        assert adjoint_overlap(solver) == bool(mode)
        _, seed = loss_seed(UK, rho_t)
        g1, _ = adjoint_backward(solver, seed)
        g2, _ = adjoint_backward(solver, seed)
        assert np.all(np.isfinite(g1))
        assert np.array_equal(g1, g2)
        out[mode] = (UK, g1)
    adjoint_overlap(solver, 1)
    assert np.array_equal(out[0][0], out[1][0])
    assert np.array_equal(out[0][1], out[1][1])


def test_workspace_reuse(tmp_path):
    """A forward with the same steps, checkpoints, overlap mode and CFL reuses the previous
    forward's workspace and the backward sweep's captured graphs: the gradients equal those of
    a fresh workspace bitwise, for other initial states and seeds, and after a CFL change (which
    lays the workspace out again)."""
    tp, su2, p, mesh, solver, U0, Ut0 = setup_case(tmp_path, n=16)
    K, nck = 7, 3
    rng = np.random.default_rng(12)
    U0b = U0 * (1 + 1e-3 * rng.standard_normal(U0.shape))
    seed_a, seed_b = rng.standard_normal(U0.shape), rng.standard_normal(U0.shape)

    def run(U, seed, fresh):
        if fresh:
            fv.lib().fvgb_adjoint_release(solver._h)
        UK, _ = adjoint_forward(solver, U, K, nck)
        return UK, adjoint_backward(solver, seed)[0]

    a1 = run(U0, seed_a, True)
    b_reused = run(U0b, seed_b, False)
    a_reused = run(U0, seed_a, False)
    b_fresh = run(U0b, seed_b, True)
    for x, y in ((a1, a_reused), (b_reused, b_fresh)):
        assert np.array_equal(x[0], y[0]) and np.array_equal(x[1], y[1])
    assert not np.array_equal(a1[1], b_fresh[1])
    solver.set_cfl(0.6)
    c_after = run(U0, seed_a, False)
    c_fresh = run(U0, seed_a, True)
    assert np.array_equal(c_after[1], c_fresh[1])
    assert not np.array_equal(c_after[1], a1[1])


def test_against_oracle_finite_differences(tmp_path):
    """The reference gradient: central differences of the oracle's forward map (CPU)."""
    tp, su2, p, mesh, solver, U0, Ut0 = setup_case(tmp_path, n=12)
    K = 5
    o = Oracle(tp, su2)
    rho_t = o.run(Ut0, K)[0][0]
    UK, _ = adjoint_forward(solver, U0, K)
    _, seed = loss_seed(UK, rho_t)
    g, _ = adjoint_backward(solver, seed)
    rng = np.random.default_rng(3)
    for _ in range(4):
        d = rng.standard_normal(U0.shape)
        d /= np.linalg.norm(d)
        Lp, _ = loss_seed(o.run(U0 + H * d, K)[0], rho_t)
        Lm, _ = loss_seed(o.run(U0 - H * d, K)[0], rho_t)
        fd = (Lp - Lm) / (2 * H)
        print(f"oracle FD relative error {abs(fd - np.sum(g * d)) / abs(fd):.2e}")
        assert abs(fd - np.sum(g * d)) <= 1e-6 * abs(fd)  # measured: 7e-10 .. 2.2e-8


def test_torch_autograd_function(tmp_path):
    torch = pytest.importorskip("torch")
    from cfd_solver_2d_gpu_gb300.autograd import steps
    tp, su2, p, mesh, solver, U0, Ut0 = setup_case(tmp_path, n=12)
    K = 4
    rho_t = torch.from_numpy(forward(solver, p, Ut0, K)[0])
    x = torch.from_numpy(U0.copy()).requires_grad_(True)
    UK = steps(x, solver, K)
    loss = 0.5 * ((UK[0] - rho_t) ** 2).sum()
    loss.backward()
    UK2, _ = adjoint_forward(solver, U0, K)
    _, seed = loss_seed(UK2, rho_t.numpy())
    g, _ = adjoint_backward(solver, seed)
    assert np.allclose(x.grad.numpy(), g, rtol=0, atol=1e-14 * np.abs(g).max())


def test_torch_autograd_rhs(tmp_path):
    """The residual's wrapper: torch's backward through R(U) is fvgb_rhs_vjp, and the
    directional derivative it gives matches a central difference of R."""
    torch = pytest.importorskip("torch")
    from cfd_solver_2d_gpu_gb300.autograd import rhs
    tp, su2, p, mesh, solver, U0, Ut0 = setup_case(tmp_path, n=12)
    w = torch.from_numpy(np.random.default_rng(2).standard_normal(U0.shape))
    x = torch.from_numpy(U0.copy()).requires_grad_(True)
    (rhs(x, solver) * w).sum().backward()
    assert np.array_equal(x.grad.numpy(), solver.rhs_vjp(U0, w.numpy()))
    d = np.random.default_rng(3).standard_normal(U0.shape)
    d /= np.linalg.norm(d)
    fd = float(np.sum(w.numpy() * (solver.rhs(U0 + H * d) - solver.rhs(U0 - H * d)))) / (2 * H)
    assert abs(fd - float(np.sum(x.grad.numpy() * d))) <= 1e-6 * abs(fd)


def test_adjoint_matches_fd_kutta_rk3(tmp_path):
    """Kutta RK3 (3103): the stages' seeds s3 = L3/6, s2 = 2/3 L3 + 2 L2, s1 = L3/6 - L2 + L1/2."""
    tp, su2, p, mesh, solver, U0, Ut0 = setup_case(tmp_path, n=16, time_advance=3103, CFL=0.6)
    K = 8
    rho_t = forward(solver, p, Ut0, K)[0]
    errs, _ = fd_check(solver, p, U0, rho_t, K, 6)
    print(f"FD relative errors: median {np.median(errs):.2e} max {errs.max():.2e} over {len(errs)} directions")
    assert np.median(errs) <= 1e-7 and errs.max() <= 1e-6, errs  # measured: median 9.4e-9, max 2.2e-8


@pytest.mark.parametrize("flux,gradient", [(2001, 1), (2002, 2), (2001, 2)])
def test_adjoint_llf_and_green_gauss(tmp_path, flux, gradient):
    """The LLF flux's reverse (llf_rev) and the Green-Gauss gradient's transpose, periodic faces
    included (the cell beyond a periodic face is its partner's), with the Barth limiter."""
    tp, su2, p, mesh, solver, U0, Ut0 = setup_case(tmp_path, n=16, flux=flux, gradient=gradient)
    K = 8
    rho_t = forward(solver, p, Ut0, K)[0]
    errs, _ = fd_check(solver, p, U0, rho_t, K, 6)
    print(f"FD relative errors: median {np.median(errs):.2e} max {errs.max():.2e} over {len(errs)} directions")
    assert np.median(errs) <= 1e-7 and errs.max() <= 2e-6, errs  # measured: medians <= 2.9e-8, max <= 1.0e-7


def boundary_case(tmp_path, name, text, su2):
    tp = str(tmp_path / f"{name}.toml")
    with open(tp, "w") as f:
        f.write(text)
    p = fv.Params.from_toml(tp)
    mesh = fv.Mesh.read_su2(su2, p)
    solver = fv.GPUSolver2(mesh, p)
    # a smooth wave with no mirror symmetry on every variable: the O-grid is symmetric about
    # both axes, and a field even in x or y there gives neighbours exactly equal values, where
    # the limiter's choice of bound ties and the map has a kink
    x, y = mesh.array("elem_xy")
    U0 = solver.get_state()
    for v, ph in enumerate((0.2, 1.1, 2.3, 0.7)):
        U0[v] *= 1 + 0.03 * np.sin(0.37 * x + 0.61 * y + ph) + 0.02 * np.cos(0.53 * x - 0.29 * y + 2 * ph)
    Ut0 = U0.copy()
    Ut0[0] *= 1 + 0.02 * np.cos(0.7 * x + 0.3 * y)  # target: the forward solution from a reshaped density
    Ut0[3] *= 1 + 0.02 * np.cos(0.7 * x + 0.3 * y)
    return p, solver, U0, Ut0


@pytest.mark.parametrize("kind", ["cylinder_far_field", "channel_subsonic", "channel_mach2", "channel_gg_llf",
                                  "channel_dsr"])
def test_adjoint_far_field_inlet_outlet(tmp_path, kind):
    """Far-field, inlet and outlet ghosts (ghost_farfield_vjp, all four sub/supersonic
    branches between the three cases), with slip walls and symmetry edges, against central
    finite differences of the same forward map."""
    d = str(tmp_path)
    if kind == "cylinder_far_field":  # slip wall + far field, uniform flow at Mach 0.34
        # first order: in the wall cells of the O-grid the limiter's choices switch within a
        # finite-difference step of 1e-6, so the difference quotient is no derivative there, and
        # the unlimited reconstruction does not stay finite (the channel cases keep the limiter)
        su2 = cases.cylinder_mesh(16, 8, directory=d)
        text = cases.toml_text(flux=2002, reconstruct=3001, gradient=1, limiter=1, time_advance=3104, CFL=0.6,
                               ic_type=1, inf=(1.0, 0.4, 0.05, 1.0))
    elif kind == "channel_subsonic":
        su2 = cases.channel_mesh(12, jitter=0.2, directory=d)
        text = cases.toml_text(flux=2002, reconstruct=3002, gradient=1, limiter=1, time_advance=3103, CFL=0.6,
                               vortex=(2.5, 7.0, 3.0), inf=(1.0, 1.0, 0.3, 1.0), inlet=(1.0, 1.0, 0.3, 1.0),
                               outlet=(1.0, 1.0, 0.0, 0.9))
    elif kind == "channel_dsr":  # the top boundary as "dsr": inlet state left of the moving shock, outlet right
        text0 = open(cases.channel_mesh(12, jitter=0.2, directory=d)).read()
        su2 = str(tmp_path / "channel_dsr.su2")
        open(su2, "w").write(text0.replace("MARKER_TAG= symmetry", "MARKER_TAG= dsr"))
        text = cases.toml_text(flux=2002, reconstruct=3002, gradient=1, limiter=1, time_advance=3104, CFL=0.6,
                               vortex=(2.5, 7.0, 3.0), inf=(1.0, 1.0, 0.3, 1.0), inlet=(1.0, 1.0, 0.3, 1.0),
                               outlet=(1.0, 1.0, 0.0, 0.9))
    elif kind == "channel_gg_llf":  # Green-Gauss boundary faces (the cell's own value), LLF
        su2 = cases.channel_mesh(12, jitter=0.2, directory=d)
        text = cases.toml_text(flux=2001, reconstruct=3002, gradient=2, limiter=1, time_advance=3103, CFL=0.6,
                               vortex=(2.5, 7.0, 3.0), inf=(1.0, 1.0, 0.3, 1.0), inlet=(1.0, 1.0, 0.3, 1.0),
                               outlet=(1.0, 1.0, 0.0, 0.9))
    else:
        su2 = cases.channel_mesh(12, jitter=0.2, directory=d)
        text = cases.toml_text(flux=2002, reconstruct=3002, gradient=1, limiter=0, time_advance=3101, CFL=0.5,
                               vortex=(7.0, 3.0, 2.0), inf=(1.0, 2.5, 0.2, 1.0), inlet=(1.0, 2.5, 0.2, 1.0),
                               outlet=(1.0, 2.5, 0.0, 1.0))
    p, solver, U0, Ut0 = boundary_case(tmp_path, kind, text, su2)
    K = 6
    rho_t = forward(solver, p, Ut0, K)[0]
    errs, g = fd_check(solver, p, U0, rho_t, K, 6)
    assert np.all(np.isfinite(g))
    print(f"FD relative errors: median {np.median(errs):.2e} max {errs.max():.2e} over {len(errs)} directions")
    # measured maxima: cylinder 3.8e-7, channels 5.4e-9 .. 1.4e-7, double Mach reflection 5.9e-6 (its
    # moving shock switches "dsr" edges between the inlet and outlet states near the FD step)
    bound = 5e-5 if kind == "channel_dsr" else 5e-6
    assert np.median(errs) <= 1e-7 and errs.max() <= bound, errs


@pytest.mark.parametrize("kind", ["vortex_ns", "channel_ns_gg", "channel_ns_o1_mirror"])
def test_adjoint_navier_stokes(tmp_path, kind):
    """The laminar viscous flux's reverse (viscous_vjp: the averaged state and the gradients it
    reads, through the gradient and limiter transposes), the no-slip wall's ghost in both of
    its forms, and the viscous term of the time step, at Re = 100."""
    d = str(tmp_path)
    if kind == "vortex_ns":  # periodic, LSQ + Barth, Roe, SSP-RK3
        su2 = cases.square_mesh(16, jitter=0.2, directory=d)
        text = cases.toml_text(equation=2, flux=2002, reconstruct=3002, gradient=1, limiter=1, time_advance=3104,
                               CFL=0.6, Re=100.0)
    elif kind == "channel_ns_gg":  # no-slip wall (the reference's ghost), symmetry, inlet, outlet
        su2 = cases.channel_mesh(12, jitter=0.2, directory=d)
        text = cases.toml_text(equation=2, flux=2002, reconstruct=3002, gradient=2, limiter=1, time_advance=3103,
                               CFL=0.6, Re=100.0, vortex=(2.5, 7.0, 3.0), inf=(1.0, 1.0, 0.3, 1.0),
                               inlet=(1.0, 1.0, 0.3, 1.0), outlet=(1.0, 1.0, 0.0, 0.9))
    else:  # constant reconstruction (the viscous flux still reads gradients), mirrored wall ghost, LLF
        su2 = cases.channel_mesh(12, jitter=0.2, directory=d)
        text = cases.toml_text(equation=2, flux=2001, reconstruct=3001, gradient=1, limiter=1, time_advance=3101,
                               CFL=0.5, Re=100.0, vortex=(2.5, 7.0, 3.0), inf=(1.0, 1.0, 0.3, 1.0),
                               inlet=(1.0, 1.0, 0.3, 1.0), outlet=(1.0, 1.0, 0.0, 0.9), wall_bc="mirror")
    p, solver, U0, Ut0 = boundary_case(tmp_path, kind, text, su2)
    K = 6
    rho_t = forward(solver, p, Ut0, K)[0]
    errs, g = fd_check(solver, p, U0, rho_t, K, 6)
    assert np.all(np.isfinite(g))
    print(f"FD relative errors: median {np.median(errs):.2e} max {errs.max():.2e} over {len(errs)} directions")
    # measured: vortex_ns median 9.5e-7, max 1.0e-5 (limiter branches of the viscous vortex near the
    # FD step); the channels' maxima 6.1e-8 and 1.1e-7
    if kind == "vortex_ns":
        assert np.median(errs) <= 1e-6 and errs.max() <= 1e-4, errs
    else:
        assert np.median(errs) <= 1e-7 and errs.max() <= 2e-6, errs


@pytest.mark.parametrize("kind", ["vortex_lsq_barth_roe", "vortex_gg_llf", "vortex_o1", "channel_subsonic",
                                  "vortex_ns", "channel_ns_gg", "vortex_steady", "channel_mixed"])
def test_rhs_vjp_matches_fd(tmp_path, kind):
    """fvgb_rhs_vjp, (dR/dU)^T seed, against central finite differences of fvgb_rhs
    (seed . (R(U + h d) - R(U - h d)) / 2h against d . grad, random unit directions d)."""
    d = str(tmp_path)
    channel = dict(vortex=(2.5, 7.0, 3.0), inf=(1.0, 1.0, 0.3, 1.0), inlet=(1.0, 1.0, 0.3, 1.0),
                   outlet=(1.0, 1.0, 0.0, 0.9))
    if kind.startswith("vortex"):
        su2 = cases.square_mesh(16, jitter=0.2, directory=d)
    else:
        su2 = cases.channel_mesh(12, jitter=0.2, directory=d)
    if kind == "channel_mixed":  # triangles and quads in one file
        su2 = cases.mixed_mesh(su2, str(tmp_path / "mixed.su2"))
    cfg = {"vortex_lsq_barth_roe": dict(flux=2002, reconstruct=3002, gradient=1, limiter=1),
           "vortex_gg_llf": dict(flux=2001, reconstruct=3002, gradient=2, limiter=1),
           "vortex_o1": dict(flux=2002, reconstruct=3001, gradient=1, limiter=1),
           "channel_subsonic": dict(flux=2002, reconstruct=3002, gradient=1, limiter=1, **channel),
           "vortex_ns": dict(equation=2, flux=2002, reconstruct=3002, gradient=1, limiter=1, Re=100.0),
           "channel_ns_gg": dict(equation=2, flux=2002, reconstruct=3002, gradient=2, limiter=1, Re=100.0, **channel),
           "vortex_steady": dict(flux=2002, reconstruct=3002, gradient=1, limiter=1, steady=1),
           "channel_mixed": dict(flux=2002, reconstruct=3002, gradient=1, limiter=1, **channel)}[kind]
    text = cases.toml_text(time_advance=3104, CFL=0.6, **cfg)
    p, solver, U0, _ = boundary_case(tmp_path, kind, text, su2)
    rng = np.random.default_rng(5)
    lam = rng.standard_normal(U0.shape)
    g = solver.rhs_vjp(U0, lam)
    assert np.all(np.isfinite(g))
    assert np.array_equal(solver.get_state(), U0)  # the handle's state is U, as after rhs
    assert np.array_equal(solver.rhs_vjp(U0, lam), g)  # the cached workspace: same bits again
    errs = []
    for _ in range(6):
        dU = rng.standard_normal(U0.shape)
        dU /= np.linalg.norm(dU)
        fd = float(np.sum(lam * (solver.rhs(U0 + H * dU) - solver.rhs(U0 - H * dU)))) / (2 * H)
        ad = float(np.sum(g * dU))
        errs.append(abs(fd - ad) / max(abs(fd), 1e-30))
    errs = np.array(errs)
    print(f"FD relative errors: median {np.median(errs):.2e} max {errs.max():.2e} over {len(errs)} directions")
    assert np.median(errs) <= 1e-7 and errs.max() <= 1e-6, errs  # measured: maxima 5.2e-9 .. 4.1e-8


def test_handles_in_parallel_threads(tmp_path):
    """Two handles driven from two host threads at once (ctypes releases the GIL during
    each call): the adjoint's and the residual VJP's per-handle workspaces are registered
    concurrently, and each thread's results equal the same calls made one after another."""
    import threading
    tp, su2, p, mesh, a, U0, Ut0 = setup_case(tmp_path, n=16)
    b = fv.GPUSolver2(mesh, p)
    lam = np.random.default_rng(4).standard_normal(U0.shape)
    seed = np.random.default_rng(6).standard_normal(U0.shape)

    def work_a(out):
        for _ in range(3):
            UK, _ = adjoint_forward(a, U0, 5, 2)
            out.append(adjoint_backward(a, seed)[0])
            fv.lib().fvgb_adjoint_release(a._h)

    def work_b(out):
        for _ in range(6):
            out.append(b.rhs_vjp(U0, lam))
            fv.lib().fvgb_adjoint_release(b._h)

    ra, rb = [], []
    ta, tb = threading.Thread(target=work_a, args=(ra,)), threading.Thread(target=work_b, args=(rb,))
    ta.start(); tb.start(); ta.join(); tb.join()
    adjoint_forward(a, U0, 5, 2)
    ga = adjoint_backward(a, seed)[0]
    gb = b.rhs_vjp(U0, lam)
    assert len(ra) == 3 and len(rb) == 6
    assert all(np.array_equal(g, ga) for g in ra)
    assert all(np.array_equal(g, gb) for g in rb)
