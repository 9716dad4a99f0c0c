"""Field output pinned against the reference's own FieldWriter (compiled from source into
oracle/_ref, output mode; fixtures by tests/golden/make_golden.py): node values
(update_nodeField, FVMR/src/output/FieldWriter.cpp:364-453), the Tecplot volume and
boundary files (44-172) and the wall forces of the hist line (175-262).

CPU tests check the oracle's restatement against the fixtures; the -m gpu tests
check the library (device node values, host writers) against the same fixtures."""
import gzip
import os
import tempfile

import numpy as np
import pytest

import cfd_solver_2d_gpu_gb300 as fv
from oracle import pyoracle

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "golden", "output")
NAMES = sorted(f[:-4] for f in os.listdir(OUT) if f.endswith(".npz"))


def load(name):
    z = np.load(os.path.join(OUT, name + ".npz"))
    d = tempfile.mkdtemp(prefix="fvgb_out_")
    tp, sp = os.path.join(d, "case.toml"), os.path.join(d, "case.su2")
    open(tp, "wb").write(z["toml"].tobytes())
    open(sp, "wb").write(gzip.decompress(z["su2_gz"].tobytes()))
    p = fv.Params.from_toml(tp)
    return z, p, fv.Mesh.read_su2(sp, p)


def ref_forces(z):
    last = [l for l in z["hist"].tobytes().decode().split("\n") if l][-1].split()
    return last[6], last[7]  # C_L, C_D as the reference printed them


@pytest.mark.parametrize("name", NAMES)
def test_oracle_node_field_matches_reference(name):
    z, p, m = load(name)
    f = pyoracle.node_field(m.array("elem_nodes"), z["U"], m.V, p.gamma, list(p.inf))
    assert np.array_equal(f[:4], z["node_ruvp"].reshape(4, m.V))
    assert np.array_equal(f[4], z["node_Cp"]) and np.array_equal(f[5], z["node_Ma"])


@pytest.mark.parametrize("name", NAMES)
def test_oracle_forces_match_reference(name):
    z, p, m = load(name)
    f = pyoracle.node_field(m.array("elem_nodes"), z["U"], m.V, p.gamma, list(p.inf))
    _, _, cdw, clw = pyoracle.boundary_forces(m.array("set_edge_offsets"), m.array("set_edge_list"),
                                              m.array("boundary_type"), m.array("edge_nodes"),
                                              m.array("edge_normal"), m.array("edge_length"), f[4], p.ref_area)
    assert ("%e" % clw, "%e" % cdw) == ref_forces(z)


@pytest.mark.gpu
@pytest.mark.parametrize("name", NAMES)
def test_library_output_matches_reference(name, tmp_path):
    z, p, m = load(name)
    s = fv.GPUSolver2(m, p)
    s.set_state(z["U"])
    f = s.node_field()
    assert np.array_equal(f[:4], z["node_ruvp"].reshape(4, m.V))
    assert np.array_equal(f[4], z["node_Cp"]) and np.array_equal(f[5], z["node_Ma"])
    t = float(z["t"][0])
    vol, bnd = str(tmp_path / "v.dat"), str(tmp_path / "b.dat")
    s.write_tecplot_volume(vol, t, title="title", preset=2)
    s.write_tecplot_boundary(bnd, t, preset=1)
    assert open(vol, "rb").read() == gzip.decompress(z["volume_gz"].tobytes())
    assert open(bnd, "rb").read() == gzip.decompress(z["boundary_gz"].tobytes())
    _, _, cdw, clw = s.boundary_forces(m.NB)
    assert ("%e" % clw, "%e" % cdw) == ref_forces(z)
