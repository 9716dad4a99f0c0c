"""Continue ("pause") files and the driver's configuration, on the host (no GPU).

The reference restarts from pause_<filename>[n].dat files written by
FieldWriter::writeContinueFile_1 (FVMR/src/output/FieldWriter.cpp:264-326) and
read by ContinueFileReader::readContinueFile_1 (FVMR/src/input/ContinueFileReader.cpp:
19-158, 457-494), which rebuilds the whole mesh from the file.  Pins:
  - golden fixtures (tests/golden/continue/): files written by this library
    and the arrays the reference's own reader built from them
    (make_golden.py, oracle/_ref in continue mode);
  - where the reference is present, its own shipped pause file read by both;
  - round trips through this library's writer and reader.
"""
import gzip
import os
import shutil
import subprocess
import sys

import numpy as np
import pytest

import cfd_solver_2d_gpu_gb300 as fv
from cfd_solver_2d_gpu_gb300 import cases

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, HERE)
from fvmrdump import read_dump  # noqa: E402

GOLDEN = os.path.join(HERE, "golden", "continue")
REF_BIN = os.path.join(ROOT, "oracle", "_ref", "fvmr_ref_f64")
# the reference's example cases, linked there by the oracle/ref recipe
REF_PAUSE_DIR = os.path.join(ROOT, "oracle", "_ref", "quick_start", "U2NITS-10.0", "2D_cylinder")

# this library's array name -> the reference dump's
ARRAYS = {"node_xy": "node_xy", "elem_nodes": "elem_nodes", "elem_edges": "elem_edges",
          "elem_neighbors": "elem_nbrs", "elem_xy": "elem_xy", "elem_volume": "elem_vol",
          "edge_nodes": "edge_nodes", "edge_L": "edge_L", "edge_R": "edge_R", "edge_setID": "edge_set",
          "edge_periodicPair": "edge_pair", "edge_length": "edge_len", "edge_distance": "edge_dist",
          "edge_xy": "edge_xy", "edge_normal": "edge_normal", "boundary_type": "bc_type"}


def assert_same_mesh(mesh, ref):
    for ours, theirs in ARRAYS.items():
        a = mesh.array(ours)
        b = np.asarray(ref[theirs])
        assert np.array_equal(a.reshape(b.shape), b), ours


@pytest.mark.parametrize("name", ["jsquare12", "cylinder16_ns"])
def test_reader_matches_reference_reader(name, tmp_path):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    path = tmp_path / f"pause_{name}[0042].dat"
    path.write_bytes(gzip.decompress(z["pause_gz"].tobytes()))
    mesh, U, t, istep, cfl = fv.Mesh.read_continue(str(path), equation=int(z["equation"][0]))
    assert_same_mesh(mesh, z)
    assert np.array_equal(U, z["U0"])
    t_ref, istep_ref, cfl_ref = z["continue_info"]
    assert (t, istep, cfl) == (t_ref, int(istep_ref), cfl_ref)


@pytest.mark.parametrize("kind", ["square", "cylinder"])
def test_write_then_read_is_exact(kind, tmp_path):
    if kind == "square":
        su2, eq = cases.square_mesh(10, jitter=0.2, directory=str(tmp_path)), 1
    else:
        su2, eq = cases.cylinder_mesh(12, 6, directory=str(tmp_path)), 2
    m = fv.Mesh.read_su2(su2, equation=eq)
    U = np.random.default_rng(5).normal(1.0, 0.3, (4, m.N))
    path = str(tmp_path / "pause_x[0007].dat")
    m.write_continue(path, U, np.pi, 7, 0.65)
    m2, U2, t, istep, cfl = fv.Mesh.read_continue(path, equation=eq)
    for k in ARRAYS:
        assert np.array_equal(m.array(k), m2.array(k)), k
    assert np.array_equal(U, U2) and t == np.pi and istep == 7 and cfl == 0.65
    # a mesh read from a continue file writes the same file again
    again = str(tmp_path / "again.dat")
    m2.write_continue(again, U2, t, istep, cfl)
    assert open(path).read() == open(again).read()


def test_file_layout_follows_the_reference_writer(tmp_path):
    su2 = cases.cylinder_mesh(12, 6, directory=str(tmp_path))
    m = fv.Mesh.read_su2(su2, equation=1)
    path = str(tmp_path / "p.dat")
    m.write_continue(path, np.ones((4, m.N)), 1.5, 3, 0.5)
    lines = open(path).read().split("\n")
    assert lines[0] == "t, istep, CFL" and lines[1].split() == ["1.5", "3", "0.5"]
    assert lines[2] == "nodes: ID, x, y"
    i = lines.index("elements: ID, nodes, U")
    assert i == 3 + m.V
    j = lines.index("boundaries: ID, name; edgeIDs")
    assert j == i + 1 + m.N
    assert lines[i + 1].split()[0] == "1" and len(lines[i + 1].split()) == 8
    # edge IDs ten to a line after each "ID name" line
    assert lines[j + 1].split()[1] in ("wall", "farfield")
    assert all(len(l.split()) <= 10 for l in lines[j + 1:])


def test_find_continue_file_rule(tmp_path):
    for f in ("pause_run[0000].dat", "pause_run[0005].dat", "pause_run[0012].dat", "pause_run[x].dat",
              "pause_other[0099].dat", "nan_run[0100].dat", "pause_run[0003].txt"):
        (tmp_path / f).write_text("")
    assert fv.find_continue_file(str(tmp_path), "run") == str(tmp_path / "pause_run[0012].dat")
    assert fv.find_continue_file(str(tmp_path), "nothing") is None
    only0 = tmp_path / "z"
    only0.mkdir()
    (only0 / "pause_run[0000].dat").write_text("")
    assert fv.find_continue_file(str(only0), "run") is None  # n = 0 is never chosen (ContinueFileReader.cpp:46)


def test_malformed_continue_file_is_an_error(tmp_path):
    p = tmp_path / "bad.dat"
    p.write_text("nodes: ID, x, y\n1 0 0\n")
    with pytest.raises(fv.FvgbError) as e:
        fv.Mesh.read_continue(str(p))
    assert e.value.code == -3  # FVGB_ERR_FORMAT
    with pytest.raises(fv.FvgbError) as e:
        fv.Mesh.read_continue(str(tmp_path / "missing.dat"))
    assert e.value.code == -2  # FVGB_ERR_IO


@pytest.mark.skipif(not (os.path.exists(REF_BIN) and os.path.isdir(REF_PAUSE_DIR)),
                    reason="the reference (sources and oracle/_ref build) is only in the build container")
def test_reads_the_references_own_pause_file(tmp_path):
    """The pause file the reference ships (6 significant digits, NS cylinder), read by the
    reference's ContinueFileReader and by this library: identical arrays and state."""
    out = str(tmp_path / "ref.bin")
    r = subprocess.run([REF_BIN, os.path.join(REF_PAUSE_DIR, "input.toml"), REF_PAUSE_DIR, "continue", "0", out],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-300:]
    ref = read_dump(out)
    path = fv.find_continue_file(REF_PAUSE_DIR, "cylinder_allfar_50")
    mesh, U, t, istep, cfl = fv.Mesh.read_continue(path, equation=2)
    assert_same_mesh(mesh, ref)
    assert np.array_equal(U, ref["U0"])
    assert (t, istep, cfl) == tuple(ref["continue"][:1]) + (int(ref["continue"][1]), ref["continue"][2])


def test_run_config_keys(tmp_path):
    tp = tmp_path / "in.toml"
    tp.write_text(cases.toml_text(filename="abc", max_iteration=77))
    c = fv.run_config(str(tp))
    assert c["filename"] == "abc" and c["max_iteration"] == 77 and c["continue_run"] == 0
    assert (c["step_per_print"], c["step_per_output_field"], c["step_per_output_hist"]) == (50, 100, 100)
    assert c["tolerance_residual"] == 1e-7 and c["mesh_file_type"] == "su2"


def test_driver_cli_without_a_gpu(tmp_path):
    exe = os.path.join(ROOT, "cfd_solver_2d_gpu_gb300", "fvgb_run")
    fv.lib()  # builds the library and the driver
    r = subprocess.run([exe, "--help"], capture_output=True, text=True)
    assert r.returncode == 1 and "usage" in r.stderr
    tp, su2 = cases.vortex_small(str(tmp_path), n=8)
    shutil.copy(su2, str(tmp_path / "mesh.su2"))
    r = subprocess.run([exe, tp, "--output", str(tmp_path / "out"), "--quiet"], capture_output=True, text=True)
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if not has_gpu:
        # no device: a clean error from fvgb_create, never a crash
        assert r.returncode == 1 and "fvgb_create" in r.stderr, (r.returncode, r.stderr)
