"""The headless driver (fvgb_run, csrc/driver/fvgb_run.cpp) on the GPU: its loop
gives the same state as stepping through the C ABI directly, a run stopped and
restarted from its pause file ends bit for bit where an unbroken run ends, and a
NaN ends the run with status 2 and a nan_ continue file (as CDriver::start's
signal packs, FVMR/src/drivers/CDriver.cpp:202-263)."""
import ctypes
import os
import shutil
import subprocess

import numpy as np
import pytest

import cfd_solver_2d_gpu_gb300 as fv
from cfd_solver_2d_gpu_gb300 import cases
from oracle.pyoracle import Oracle

pytestmark = pytest.mark.gpu
EXE = os.path.join(os.path.dirname(fv.__file__), "fvgb_run")


def make_case(d, max_iteration, cont=False):
    os.makedirs(d, exist_ok=True)
    text = cases.toml_text(flux=2002, reconstruct=3002, gradient=1, limiter=1, time_advance=3104, CFL=0.8,
                           filename="jv", max_iteration=max_iteration)
    text = text.replace("step_per_print = 50", "step_per_print = 10").replace(
        "step_per_output_hist = 100", "step_per_output_hist = 5")
    if cont:
        text = text.replace("continue = false", "continue = true")
    tp = os.path.join(d, "input.toml")
    with open(tp, "w") as f:
        f.write(text)
    shutil.copy(cases.square_mesh(24, jitter=0.2), os.path.join(d, "jv.su2"))
    return tp


def run(tp, out):
    fv.lib()
    return subprocess.run([EXE, tp, "--output", out], capture_output=True, text=True)


def test_driver_matches_direct_stepping(tmp_path):
    d = str(tmp_path / "case")
    tp = make_case(d, 30)
    r = run(tp, os.path.join(d, "out"))
    assert r.returncode == 0, r.stderr
    mesh, U, t, istep, cfl = fv.Mesh.read_continue(os.path.join(d, "out", "pause_jv[0030].dat"))
    assert istep == 30 and cfl == 0.8
    p = fv.Params.from_toml(tp)
    m = fv.Mesh.read_su2(os.path.join(d, "jv.su2"), p)
    s = fv.GPUSolver2(m, p)
    t2 = s.step(0.0, p.T_end, 30)
    assert np.array_equal(s.get_state(), U) and t2 == t
    hist = open(os.path.join(d, "out", "jv_hist.dat")).read().split("\n")
    assert hist[0] == 'title= "tecplot hist file"' and hist[1].startswith('variables= "Iteration"')
    assert hist[2].startswith("zone")
    rows = [l.split() for l in hist[3:] if l]
    assert [int(r[0]) for r in rows] == [1, 5, 10, 15, 20, 25, 30] and all(len(r) == 8 for r in rows)
    # the residual columns: the L-infinity norms of updateResidualVector (GPUSolver2.cpp:294-296),
    # against the oracle's get_residual_host of its own last residual after 30 steps, to the
    # precision of the file's %e (6 significant decimals)
    o = Oracle(tp, os.path.join(d, "jv.su2"))
    _, _, _, last = o.run(o.init_field(), 30)
    assert np.allclose([float(x) for x in rows[-1][2:6]], o.residual(last, 0), rtol=1e-6, atol=0)
    assert "step = 10" in r.stdout and "step = 30" in r.stdout
    # Tecplot volume files at step 1 and at the stop, the boundary file overwritten in place
    out = os.path.join(d, "out")
    for f in ("jv[0001].dat", "jv[0030].dat", "jv_tec_boundary.dat"):
        assert os.path.getsize(os.path.join(out, f)) > 0, f
    vol = open(os.path.join(out, "jv[0030].dat")).read().split("\n")
    assert vol[1] == 'variables= "x", "y", "rho", "u", "v", "p", "Ma"' and f"nodes= {m.V}" in vol[2]
    assert np.allclose([float(x) for x in vol[3].split()[2:6]], s.node_field()[:4, 0], rtol=1e-6)


def test_restart_continues_bit_for_bit(tmp_path):
    one = str(tmp_path / "one")
    assert run(make_case(one, 30), os.path.join(one, "out")).returncode == 0
    two = str(tmp_path / "two")
    out = os.path.join(two, "out")
    assert run(make_case(two, 12), out).returncode == 0
    r = run(make_case(two, 30, cont=True), out)  # basic.continue: resumes from pause_jv[0012].dat
    assert r.returncode == 0 and "continue from" in r.stdout, r.stdout + r.stderr
    _, Ua, ta, ia, _ = fv.Mesh.read_continue(os.path.join(one, "out", "pause_jv[0030].dat"))
    _, Ub, tb, ib, _ = fv.Mesh.read_continue(os.path.join(out, "pause_jv[0030].dat"))
    assert ia == ib == 30 and ta == tb and np.array_equal(Ua, Ub)


def test_nan_stops_with_status_2(tmp_path):
    d = str(tmp_path / "nan")
    out = os.path.join(d, "out")
    assert run(make_case(d, 3), out).returncode == 0
    mesh, U, t, istep, cfl = fv.Mesh.read_continue(os.path.join(out, "pause_jv[0003].dat"))
    U[:, 17] = np.nan
    os.remove(os.path.join(out, "pause_jv[0003].dat"))
    mesh.write_continue(os.path.join(out, "pause_jv[0004].dat"), U, t, 4, cfl)
    r = run(make_case(d, 20, cont=True), out)
    assert r.returncode == 2, (r.returncode, r.stdout, r.stderr)
    assert any(f.startswith("nan_jv[") for f in os.listdir(out))


def test_driver_adaptive_cfl(tmp_path):
    """time.strategy = 1: past step 5000 the driver raises CFL at its print events as
    RoutineController does (x 1.1 or x 1.05 with a 1000-step cool-down); the steps after a
    change equal a solver created with the new CFL, and the pause file keeps it."""
    d = str(tmp_path / "case")
    os.makedirs(d)
    text = cases.toml_text(flux=2002, reconstruct=3001, gradient=1, limiter=1, time_advance=3101, CFL=0.5,
                           filename="sq", max_iteration=5060)
    text = text.replace("[time]\n", "[time]\nstrategy = 1\n").replace(
        "step_per_output_field = 100", "step_per_output_field = 100000")
    tp = os.path.join(d, "input.toml")
    with open(tp, "w") as f:
        f.write(text)
    shutil.copy(cases.square_mesh(8), os.path.join(d, "sq.su2"))
    r = run(tp, os.path.join(d, "out"))
    assert r.returncode == 0, r.stderr
    changes = [l for l in r.stdout.split("\n") if "CFL = " in l]
    assert len(changes) == 1 and changes[0].startswith("step = 5050"), changes
    new = float(changes[0].split("CFL = ")[1])
    assert new in (0.5 * 1.1, 0.5 * 1.05)
    _, U, t, istep, cfl = fv.Mesh.read_continue(os.path.join(d, "out", "pause_sq[5060].dat"))
    assert istep == 5060 and cfl == new
    # the same run through the C ABI: 5050 steps at 0.5, then 10 at the new CFL
    p = fv.Params.from_toml(tp)
    m = fv.Mesh.read_su2(os.path.join(d, "sq.su2"), p)
    s = fv.GPUSolver2(m, p)
    t1 = s.step(0.0, p.T_end, 5050)
    assert fv.lib().fvgb_set_cfl(s._h, ctypes.c_double(new)) == 0
    t2 = s.step(t1, p.T_end, 10)
    assert np.array_equal(s.get_state(), U) and t2 == t


def test_driver_wall_time_snapshots(tmp_path):
    """The reference writes a pause file whenever 30 minutes of wall time have passed since the
    last one (CDriver.cpp:227-232); with the cool-down at 0 s every event writes one, each the
    state of its step."""
    d = str(tmp_path / "case")
    tp = make_case(d, 20)
    out = os.path.join(d, "out")
    fv.lib()
    r = subprocess.run([EXE, tp, "--output", out, "--snapshot-seconds", "0"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    pauses = sorted(f for f in os.listdir(out) if f.startswith("pause_"))
    assert pauses == ["pause_jv[%04d].dat" % k for k in (1, 5, 10, 15, 20)], pauses
    p = fv.Params.from_toml(tp)
    m = fv.Mesh.read_su2(os.path.join(d, "jv.su2"), p)
    s = fv.GPUSolver2(m, p)
    t = s.step(0.0, p.T_end, 10)
    _, U, t10, istep, _ = fv.Mesh.read_continue(os.path.join(out, "pause_jv[0010].dat"))
    assert istep == 10 and t10 == t and np.array_equal(U, s.get_state())
    d2 = str(tmp_path / "case2")
    r = run(make_case(d2, 20), os.path.join(d2, "out"))  # the default cool-down: only the stop writes one
    assert r.returncode == 0 and [f for f in os.listdir(os.path.join(d2, "out")) if f.startswith("pause_")] == \
        ["pause_jv[0020].dat"]


def test_driver_stops_on_a_signal(tmp_path):
    """SIGINT plays the reference's ESC key (CDriver.cpp:244-249): the run stops at its next
    event and writes the pause file of that step."""
    import signal
    d = str(tmp_path / "case")
    tp = make_case(d, 10_000_000)
    out = os.path.join(d, "out")
    fv.lib()
    proc = subprocess.Popen([EXE, tp, "--output", out], stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True)
    try:
        for line in proc.stdout:
            if line.startswith("step = 200\t"):
                proc.send_signal(signal.SIGINT)
                break
        rest, err = proc.communicate(timeout=60)
    finally:
        if proc.poll() is None:
            proc.kill()
            proc.wait()
    assert proc.returncode == 0, err
    pauses = [f for f in os.listdir(out) if f.startswith("pause_")]
    assert len(pauses) == 1
    _, U, t, istep, _ = fv.Mesh.read_continue(os.path.join(out, pauses[0]))
    assert 200 <= istep < 10_000_000 and "stopped by a signal" in rest
    p = fv.Params.from_toml(tp)
    s = fv.GPUSolver2(fv.Mesh.read_su2(os.path.join(d, "jv.su2"), p), p)
    t2 = s.step(0.0, p.T_end, istep)
    assert np.array_equal(s.get_state(), U) and t2 == t
