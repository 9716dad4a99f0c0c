"""Field output on the GPU against the oracle (oracle/fvm_oracle.c), which restates
the reference's writers operation by operation:
  node values   FieldWriter::update_nodeField (FVMR/src/output/FieldWriter.cpp:364-453)
  forces        ReferenceData::calculate_edgeSet_force (FieldWriter.cpp:175-210)
  Tecplot text  write_tecplot_volume_file / write_tecplot_boundary_file (FieldWriter.cpp:44-172)
  colouring     CudaGrid_kernels.cu:24-130 (the GUI path, into a device buffer)
Node values, forces and colours are compared bit for bit, the files as text."""
import os

import numpy as np
import pytest

import cfd_solver_2d_gpu_gb300 as fv
from cfd_solver_2d_gpu_gb300 import cases
from oracle import pyoracle

pytestmark = pytest.mark.gpu


def make(tmp_path, kind):
    d = str(tmp_path)
    if kind == "vortex":
        su2 = cases.square_mesh(24, jitter=0.2, directory=d)
        text = cases.toml_text(flux=2002, reconstruct=3002, gradient=1, limiter=1, time_advance=3104, CFL=0.8,
                               inf=(1.0, 1.0, 0.3, 1.0))
    else:
        su2 = cases.cylinder_mesh(32, 16, directory=d)
        text = cases.toml_text(equation=2, flux=2002, reconstruct=3002, gradient=1, limiter=1, time_advance=3103,
                               CFL=0.5, ic_type=1, inf_mode=0, Ma=0.3, AoA=4.0, Re=100.0, ref_area=2.0)
    tp = os.path.join(d, kind + ".toml")
    with open(tp, "w") as f:
        f.write(text)
    p = fv.Params.from_toml(tp)
    m = fv.Mesh.read_su2(su2, p)
    s = fv.GPUSolver2(m, p)
    s.step(0.0, p.T_end, 7)
    return p, m, s


def oracle_node_field(p, m, s):
    return pyoracle.node_field(m.array("elem_nodes"), s.get_state(), m.V, p.gamma, list(p.inf))


@pytest.mark.parametrize("kind", ["vortex", "cylinder"])
def test_node_field_bit_exact(tmp_path, kind):
    p, m, s = make(tmp_path, kind)
    assert np.array_equal(s.node_field(), oracle_node_field(p, m, s))


@pytest.mark.parametrize("kind", ["vortex", "cylinder"])
def test_boundary_forces_bit_exact(tmp_path, kind):
    p, m, s = make(tmp_path, kind)
    f = oracle_node_field(p, m, s)
    want = pyoracle.boundary_forces(m.array("set_edge_offsets"), m.array("set_edge_list"), m.array("boundary_type"),
                                    m.array("edge_nodes"), m.array("edge_normal"), m.array("edge_length"), f[4],
                                    p.ref_area)
    got = s.boundary_forces(m.NB)
    assert np.array_equal(got[0], want[0]) and np.array_equal(got[1], want[1])
    assert got[2:] == want[2:]
    if kind == "cylinder":
        assert got[2] != 0.0  # the wall carries a pressure force


def _line(vals):
    return " ".join("%e" % v for v in vals) + "\n"


def _cols(f, xy, n, preset):
    V = f.shape[1]
    vals = [xy[0, n], xy[1, n], f[0, n], f[1, n], f[2, n], f[3, n]]
    if preset == 1:
        vals.append(f[4, n])
    elif preset == 2:
        vals.append(f[5, n])
    return vals


NAMES = {0: '"x", "y", "rho", "u", "v", "p"', 1: '"x", "y", "rho", "u", "v", "p", "Cp"',
         2: '"x", "y", "rho", "u", "v", "p", "Ma"'}


@pytest.mark.parametrize("preset", [0, 1, 2])
def test_tecplot_volume_text(tmp_path, preset):
    p, m, s = make(tmp_path, "cylinder")
    path = str(tmp_path / "vol.dat")
    s.write_tecplot_volume(path, 0.25, title="cyl", preset=preset)
    f = oracle_node_field(p, m, s)
    xy = m.array("node_xy")
    en = m.array("elem_nodes")
    want = ('title= "cyl"\nvariables= %s\nzone t= "volume field", nodes= %d, elements= %d, datapacking= point, '
            "zonetype= fequadrilateral, solutiontime= %e\n" % (NAMES[preset], m.V, m.N, 0.25))
    want += "".join(_line(_cols(f, xy, n, preset)) for n in range(m.V))
    want += "".join("%d %d %d %d\n" % (en[0, c] + 1, en[1, c] + 1, en[2, c] + 1, en[2, c] + 1) for c in range(m.N))
    assert open(path).read() == want


def test_tecplot_boundary_text(tmp_path):
    p, m, s = make(tmp_path, "cylinder")
    path = str(tmp_path / "bnd.dat")
    s.write_tecplot_boundary(path, 0.5, preset=1)
    f = oracle_node_field(p, m, s)
    xy = m.array("node_xy")
    off, lst, ed = m.array("set_edge_offsets"), m.array("set_edge_list"), m.array("edge_nodes")
    names = ["wall", "farfield"]
    want = 'title= "tecplot boundary file"\nvariables= %s\n' % NAMES[1]
    for b in range(m.NB):
        want += ('zone t= "boundary %d %s", solutiontime= %e, strandid= 0, i= %d, j= 1, f= point\n'
                 % (b + 1, names[b], 0.5, off[b + 1] - off[b]))
        n1_old = -1
        for e in lst[off[b]:off[b + 1]]:
            n0, n1 = ed[0, e], ed[1, e]
            if n0 != n1_old:
                want += _line(_cols(f, xy, n0, 1))
            want += _line(_cols(f, xy, n1, 1))
            n1_old = n1
    assert open(path).read() == want


@pytest.mark.parametrize("rng", [(0.5, 1.5), (0.9, 1.1), (1.0, 1.0)])
def test_colouring_bit_exact(tmp_path, rng):
    p, m, s = make(tmp_path, "vortex")
    rgb, val, dev = s.colour_nodes(*rng)
    want_rgb, want_val = pyoracle.colour_nodes(m.array("elem_nodes"), s.get_state(), m.V, *rng)
    assert dev and np.array_equal(val, want_val) and np.array_equal(rgb, want_rgb)
    assert rgb.min() >= 0.0 and rgb.max() <= 1.0


def test_colouring_full_mesh_deterministic():
    with_dir = cases.cache_dir()
    tp, su2 = cases.vortex_large(with_dir)
    p = fv.Params.from_toml(tp)
    s = fv.GPUSolver2(fv.Mesh.read_su2(su2, p), p)
    s.step(0.0, p.T_end, 2)
    a = s.colour_nodes(0.5, 1.05)
    b = s.colour_nodes(0.5, 1.05)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    assert np.isfinite(a[1]).all() and a[1].min() > 0.3
