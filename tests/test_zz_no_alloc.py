"""fvgb_rhs_noalloc: the residual for callers that own all device memory and
may not allocate more (an application handing this step a fixed part of its
own memory arena, or a path that cannot take the device-wide pause an
allocation can cause).  The test plays such a caller: it places the
reference-layout arrays on the GPU itself, calls the entry point through the
C ABI twice in a row on different states, and compares each result with the
ordinary residual entry point (fvgb_rhs) and with the oracle's residual (the
C restatement of the reference's calculateFunctionF) at the parity tolerance
(1e-12, relative L-infinity).  The file sorts last so a failure here comes after every
other test has run."""
import ctypes

import numpy as np
import pytest

import cfd_solver_2d_gpu_gb300 as fv
from cfd_solver_2d_gpu_gb300 import cases
from oracle.pyoracle import Oracle

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def device_mesh(mesh):
    """Copies the reference-layout arrays to the GPU (the caller's memory) and returns
    an fvgb_mesh_soa of device pointers plus the tensors that keep them alive."""
    import torch
    keep = {}
    soa = fv.MeshSoA()
    soa.num_node, soa.num_element, soa.num_edge, soa.num_boundary = mesh.V, mesh.N, mesh.E, mesh.NB
    for name in ("elem_edges", "elem_volume", "edge_L", "edge_R", "edge_setID", "edge_length", "edge_normal",
                 "boundary_type", "elem_neighbors", "elem_nodes", "node_xy", "elem_xy", "edge_nodes",
                 "edge_periodicPair", "edge_distance", "edge_xy"):
        t = torch.from_numpy(np.ascontiguousarray(mesh.array(name))).cuda()
        keep[name] = t
        setattr(soa, name, t.data_ptr())
    return soa, keep


@pytest.mark.parametrize("kind", ["vortex_roe", "cylinder_llf", "dmr_roe", "mixed_channel_llf"])
def test_rhs_noalloc_matches_rhs(tmp_path, kind):
    import torch
    L = fv.lib()
    L.fvgb_rhs_noalloc.restype = ctypes.c_int
    L.fvgb_rhs_noalloc.argtypes = [ctypes.POINTER(fv.MeshSoA), ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                   ctypes.c_void_p]
    if kind == "vortex_roe":
        tp, su2 = cases.vortex_small(str(tmp_path), n=64)
    elif kind == "cylinder_llf":
        tp = str(tmp_path / "cyl.toml")
        with open(tp, "w") as f:
            f.write(cases.toml_text(equation=1, flux=2001, reconstruct=3001, gradient=1, limiter=1,
                                    time_advance=3103, CFL=0.5, ic_type=1, inf_mode=0, Ma=0.5))
        su2 = cases.cylinder_mesh(64, 32, directory=str(tmp_path))
    elif kind == "dmr_roe":  # double Mach reflection: "dsr" edges at p.dsr_time against the handle's clock
        tp = str(tmp_path / "dmr.toml")
        with open(tp, "w") as f:
            f.write(cases.toml_text(equation=1, flux=2002, reconstruct=3001, gradient=1, limiter=1,
                                    time_advance=3101, CFL=0.5, ic_type=4, dmr=(1.0 / 6.0, 0.0, 60.0),
                                    inlet=(8.0, 8.25, -30.0, 116.5, "angle"), outlet=(1.4, 0.0, 0.0, 1.0)))
        su2 = cases.dmr_mesh(48, jitter=0.2, directory=str(tmp_path))
    else:  # triangles and quads in one file, first order, LLF
        src = cases.channel_mesh(16, jitter=0.2, directory=str(tmp_path))
        su2 = cases.mixed_mesh(src, str(tmp_path / "mixed_channel.su2"))
        tp = str(tmp_path / "mixed.toml")
        with open(tp, "w") as f:
            f.write(cases.toml_text(flux=2001, reconstruct=3001, time_advance=3104, CFL=0.6, vortex=(2.5, 7.0, 3.0),
                                    inf=(1.0, 1.0, 0.3, 1.0), inlet=(1.0, 1.0, 0.3, 1.0),
                                    outlet=(1.0, 1.0, 0.0, 0.9)))
    p = fv.Params.from_toml(tp)
    mesh = fv.Mesh.read_su2(su2, p)
    solver = fv.GPUSolver2(mesh, p)
    U0 = solver.get_state()
    # the DMR run starts just before the shock reaches the tenth top edge's midpoint (t = 0.00413)
    t = solver.step(0.0041 if kind == "dmr_roe" else 0.0, p.T_end, 3)
    p.dsr_time = t  # the handle's clock after the steps
    U1 = solver.get_state()
    soa, keep = device_mesh(mesh)
    o = Oracle(tp, su2)
    o.params.dsr_time = t
    stream = torch.cuda.current_stream().cuda_stream
    for U in (U0, U1):  # two calls in a row share the library's edge-flux array
        Ud = torch.from_numpy(np.ascontiguousarray(U)).cuda()
        Rd = torch.full_like(Ud, float("nan"))
        rc = L.fvgb_rhs_noalloc(ctypes.byref(soa), ctypes.addressof(p), Ud.data_ptr(), Rd.data_ptr(), stream)
        assert rc == 0, L.fvgb_last_error().decode()
        torch.cuda.synchronize()
        ref = solver.rhs(U)
        got = Rd.cpu().numpy()
        assert rel(got, ref) <= 1e-12
        assert rel(got, o.rhs(U)[0]) <= 1e-12
    if kind == "dmr_roe":  # the time matters: at t = 0 the tenth top edge is still downstream (outlet state)
        p.dsr_time = 0.0
        rc = L.fvgb_rhs_noalloc(ctypes.byref(soa), ctypes.addressof(p), Ud.data_ptr(), Rd.data_ptr(), stream)
        assert rc == 0
        torch.cuda.synchronize()
        assert rel(Rd.cpu().numpy(), ref) > 1e-6


def test_rhs_noalloc_rejects_what_it_cannot_hold():
    L = fv.lib()
    L.fvgb_rhs_noalloc.restype = ctypes.c_int
    L.fvgb_rhs_noalloc.argtypes = [ctypes.POINTER(fv.MeshSoA), ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                   ctypes.c_void_p]
    p = fv.Params.default()
    p.reconstruct, p.limiter = 3001, 1
    soa = fv.MeshSoA()
    soa.num_element, soa.num_edge = 10, (1 << 20) + 1
    dummy = ctypes.c_double()
    assert L.fvgb_rhs_noalloc(ctypes.byref(soa), ctypes.addressof(p), ctypes.addressof(dummy),
                              ctypes.addressof(dummy), None) == -1
    assert "at most" in L.fvgb_last_error().decode()
    soa.num_edge = 10
    p.reconstruct = 3002
    assert L.fvgb_rhs_noalloc(ctypes.byref(soa), ctypes.addressof(p), ctypes.addressof(dummy),
                              ctypes.addressof(dummy), None) == -8
