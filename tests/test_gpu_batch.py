"""The batched form (fvgb_batch_*): instances of uneven size packed into one
persistent launch per Runge-Kutta stage give, bit for bit, what each instance
gives when stepped alone through the plain path; the autotuner leaves the state
untouched."""
import numpy as np
import pytest

import cfd_solver_2d_gpu_gb300 as fv
from cfd_solver_2d_gpu_gb300 import cases

pytestmark = pytest.mark.gpu


def load(tp, sp):
    p = fv.Params.from_toml(tp)
    return fv.Mesh.read_su2(sp, p), p


def cylinders(tmp_path, nrs, machs, **kw):
    out = []
    for i, (nr, ma) in enumerate(zip(nrs, machs)):
        args = dict(equation=1, flux=2002, reconstruct=3002, gradient=1, limiter=1, time_advance=3103, CFL=0.5,
                    ic_type=1, inf_mode=0, Ma=ma, AoA=0.0, T_end=1e9)
        args.update(kw)
        tp, sp = cases.write_case(str(tmp_path), f"c{i}", cases.toml_text(**args),
                                  cases.cylinder_mesh(2 * nr, nr, directory=str(tmp_path)))
        out.append(load(tp, sp))
    return out


def plain_run(mesh, p, steps):
    s = fv.GPUSolver2(mesh, p)
    t = s.step(0.0, p.T_end, steps)
    return s.get_state(), t


def test_batch_matches_plain_cylinders(tmp_path):
    inst = cylinders(tmp_path, [6, 9, 12, 7, 10], [0.15, 0.3, 0.45, 0.55, 0.2])
    b = fv.Batch([m for m, _ in inst], [p for _, p in inst])
    t = b.step(4)
    info = b.info()
    assert info["instances"] == 5 and info["launches"] == 12
    for i, (m, p) in enumerate(inst):
        U, tp = plain_run(m, p, 4)
        assert np.array_equal(b.get_state(i), U), i
        assert t[i] == tp


def test_batch_matches_plain_vortex_ssp_gg_llf(tmp_path):
    inst = []
    for n in (8, 16, 12):
        tp, sp = cases.write_case(str(tmp_path), f"v{n}", cases.toml_text(
            flux=2001, reconstruct=3002, gradient=2, limiter=1, time_advance=3104, CFL=0.8),
            cases.square_mesh(n, jitter=0.2, directory=str(tmp_path)))
        inst.append(load(tp, sp))
    b = fv.Batch([m for m, _ in inst], [p for _, p in inst])
    b.step(3)
    for i, (m, p) in enumerate(inst):
        U, _ = plain_run(m, p, 3)
        assert np.array_equal(b.get_state(i), U), i


def test_batch_matches_plain_mixed_elements(tmp_path):
    """Instances whose meshes mix triangles and quads (half of the quads written as two
    triangles on the other diagonal) next to plain quad meshes."""
    inst = []
    for i, (n, mixed) in enumerate(((10, True), (14, False), (12, True))):
        src = cases.channel_mesh(n, jitter=0.2, directory=str(tmp_path))
        sp = cases.mixed_mesh(src, str(tmp_path / f"mx{i}.su2"), seed=i) if mixed else src
        tp, _ = cases.write_case(str(tmp_path), f"mx{i}", cases.toml_text(
            flux=2002, reconstruct=3002, gradient=1, limiter=1, time_advance=3104, CFL=0.6, vortex=(2.5, 7.0, 3.0),
            inf=(1.0, 1.0, 0.3, 1.0), inlet=(1.0, 1.0, 0.3, 1.0), outlet=(1.0, 1.0, 0.0, 0.9)), sp)
        inst.append(load(tp, sp))
    b = fv.Batch([m for m, _ in inst], [p for _, p in inst])
    t = b.step(3)
    for i, (m, p) in enumerate(inst):
        U, tp = plain_run(m, p, 3)
        assert np.array_equal(b.get_state(i), U), i
        assert t[i] == tp


def test_batch_matches_plain_channels(tmp_path):
    """Inlet, outlet, symmetry and slip-wall edges, each instance with its own inflow and
    outflow states (one supersonic)."""
    inst = []
    for i, (n, inlet, outlet) in enumerate(((8, (1.0, 1.0, 0.3, 1.0), (1.0, 1.0, 0.0, 0.9)),
                                            (16, (1.0, 2.5, 0.2, 1.0), (1.0, 2.5, 0.0, 1.0)),
                                            (12, (1.2, 0.6, -0.1, 1.1), (0.9, 0.5, 0.0, 1.0)))):
        tp, sp = cases.write_case(str(tmp_path), f"ch{i}", cases.toml_text(
            flux=2002, reconstruct=3002, gradient=1, limiter=1, time_advance=3103, CFL=0.5, vortex=(2.5, 7.0, 3.0),
            inf=inlet, inlet=inlet, outlet=outlet), cases.channel_mesh(n, jitter=0.2, directory=str(tmp_path)))
        inst.append(load(tp, sp))
    b = fv.Batch([m for m, _ in inst], [p for _, p in inst])
    t = b.step(3)
    for i, (m, p) in enumerate(inst):
        U, tp = plain_run(m, p, 3)
        assert np.array_equal(b.get_state(i), U), i
        assert t[i] == tp


def test_batch_matches_plain_double_mach_reflection(tmp_path):
    """"dsr" edges on each instance's own clock, evaluated at each stage's time: the runs
    are long enough for the shock to pass an edge midpoint on the top boundary."""
    inst = []
    for i, (n, cfl) in enumerate(((24, 0.4), (48, 0.5), (24, 0.3))):
        tp, sp = cases.write_case(str(tmp_path), f"dmr{i}", cases.toml_text(
            flux=2002, reconstruct=3002, gradient=1, limiter=1, time_advance=3103, CFL=cfl, ic_type=4,
            dmr=(1.0 / 6.0, 0.0, 60.0), inlet=(8.0, 8.25, -30.0, 116.5, "angle"), outlet=(1.4, 0.0, 0.0, 1.0)),
            cases.dmr_mesh(n, jitter=0.2, directory=str(tmp_path)))
        inst.append(load(tp, sp))
    b = fv.Batch([m for m, _ in inst], [p for _, p in inst])
    t = b.step(25)
    assert t[1] > 0.0042  # past the crossing of the 48-cell instance's tenth top edge
    for i, (m, p) in enumerate(inst):
        U, tp = plain_run(m, p, 25)
        assert np.array_equal(b.get_state(i), U), i
        assert t[i] == tp


@pytest.mark.parametrize("reconstruct,gradient", [(3002, 1), (3001, 2)])
def test_batch_matches_plain_navier_stokes(tmp_path, reconstruct, gradient):
    """Laminar cylinders (no-slip wall, far field; one viscosity law for the batch), second
    order with least squares, and first order with Green-Gauss gradients for the viscous flux."""
    inst = cylinders(tmp_path, [6, 9, 12], [0.2, 0.3, 0.45], equation=2, reconstruct=reconstruct, gradient=gradient)
    b = fv.Batch([m for m, _ in inst], [p for _, p in inst])
    t = b.step(4)
    for i, (m, p) in enumerate(inst):
        U, tp = plain_run(m, p, 4)
        assert np.array_equal(b.get_state(i), U), i
        assert t[i] == tp
    other = cylinders(tmp_path, [5], [0.2], equation=2, mu0=2e-5)[0]
    with pytest.raises(fv.FvgbError):
        fv.Batch([inst[0][0], other[0]], [inst[0][1], other[1]])


def test_autotuner_keeps_state_and_result(tmp_path):
    inst = cylinders(tmp_path, [8, 14, 5], [0.1, 0.4, 0.6])
    b = fv.Batch([m for m, _ in inst], [p for _, p in inst])
    before = [b.get_state(i) for i in range(3)]
    report = b.tune(1)
    assert report.count("ms/step") >= 4 and "chosen" in report
    for i in range(3):
        assert np.array_equal(b.get_state(i), before[i])
    b.step(2)
    for i, (m, p) in enumerate(inst):
        U, _ = plain_run(m, p, 2)
        assert np.array_equal(b.get_state(i), U), i


def test_batch_rejects_mixed_schemes(tmp_path):
    a = cylinders(tmp_path, [5], [0.2])[0]
    c = cylinders(tmp_path, [5], [0.2], flux=2001)[0]
    with pytest.raises(fv.FvgbError):
        fv.Batch([a[0], c[0]], [a[1], c[1]])


def test_bounded_barrier_gives_up_and_reports():
    """A block that never arrives makes the others' bounded wait run out: they set the error
    word and return (no hang, no fault), and the GPU stays usable."""
    import time
    t0 = time.perf_counter()
    timed_out, passed = fv.barrier_selftest(blocks=8, absent_block=3, spin_limit=200000)
    assert timed_out and passed == 0
    assert time.perf_counter() - t0 < 5.0
    timed_out, passed = fv.barrier_selftest(blocks=8, absent_block=-1, spin_limit=200000)
    assert not timed_out and passed == 8
