"""The edge-coloured scatter ([gpu] edge_colour = 1): the residual summed colour by
colour (each colour's edges add their fluxes into the cells' sums; no two edges of a
colour write the same cell) in place of the per-cell gather in the reference's slot
order.  The colouring read back from the device and mapped to the reference's edge
numbering is a proper colouring of the cells each edge writes; the residual and the
steps match the reference's own results (the golden fixtures) at the tolerances the
gather meets; the two forms agree step for step up to the order of the sums; and the
batched form and the adjoint refuse the option."""
import numpy as np
import pytest

import cfd_solver_2d_gpu_gb300 as fv
from cfd_solver_2d_gpu_gb300 import cases
from golden import make_golden

pytestmark = pytest.mark.gpu
NAMES = make_golden.names()


def rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def make(tp, sp, colour=1):
    p = fv.Params.from_toml(tp)
    p.edge_colour = colour
    m = fv.Mesh.read_su2(sp, p)
    return fv.GPUSolver2(m, p), p, m


def check_colouring(s, m):
    colour, nc = s.edge_colours()
    E, N = m.E, m.N
    assert 1 <= nc <= 5 and colour.min() == 0 and colour.max() == nc - 1
    eL, eR = m.array("edge_L"), m.array("edge_R")
    ee = m.array("elem_edges")[:3]
    in_r = np.zeros(E, dtype=bool)  # the edge is one of its R cell's edges
    for j in range(3):
        cells = np.arange(N)
        e = ee[j]
        in_r[e[eR[e] == cells]] = True
    for k in range(nc):
        mine = np.nonzero(colour == k)[0]
        writes = np.concatenate([eL[mine], eR[mine[in_r[mine]]]])
        assert len(np.unique(writes)) == len(writes), f"colour {k} writes a cell twice"
    return nc


@pytest.fixture(scope="module", params=NAMES)
def golden(request):
    return request.param, make_golden.load(request.param)


def test_colouring_is_proper_and_matches_the_reference(golden):
    name, (tp, sp, g) = golden
    s, p, m = make(tp, sp)
    check_colouring(s, m)
    assert rel(s.rhs(g["U0"]), g["rhs"]) <= 1e-12, name
    s.set_state(g["U0"])
    n = int(g["steps"][0])
    t = s.step(0.0, p.T_end, n)
    tol = 1e-9 if n >= 1000 else (1e-10 if p.reconstruct == 3002 else 1e-12)
    assert rel(s.get_state(), g["U"]) <= tol, (name, rel(s.get_state(), g["U"]))
    assert abs(t - g["t"][0]) <= 1e-11 * g["t"][0]


@pytest.mark.parametrize("flux", [2002, 2001])
def test_scatter_and_gather_agree(tmp_path, flux):
    """256 x 256 jittered vortex, LSQ + Barth, SSP-RK3: 50 steps scattered by colour and
    gathered in slot order agree to the order of the sums; both are deterministic."""
    tp, su2 = cases.vortex_large(str(tmp_path), n=256, flux=flux)
    a, p, m = make(tp, su2, colour=1)
    b, _, _ = make(tp, su2, colour=0)
    U0 = a.get_state()
    a.step(0.0, p.T_end, 50)
    b.step(0.0, p.T_end, 50)
    Ua, Ub = a.get_state(), b.get_state()
    assert rel(Ua, Ub) <= 1e-11, rel(Ua, Ub)
    a.set_state(U0)
    a.step(0.0, p.T_end, 50)
    assert np.array_equal(a.get_state(), Ua)
    assert check_colouring(a, m) <= 5


def test_batch_and_adjoint_refuse_the_option(tmp_path):
    tp, su2 = cases.vortex_small(str(tmp_path), n=16)
    s, p, m = make(tp, su2)
    with pytest.raises(fv.FvgbError) as e:
        fv.Batch([m], [p])
    assert e.value.code == -8
    with pytest.raises(fv.FvgbError) as e:
        fv.adjoint_forward(s, s.get_state(), 3)
    assert e.value.code == -8
    off, _ = fv.GPUSolver2(m, fv.Params.from_toml(tp)).edge_colours()
    assert np.all(off == -1)
