"""ctypes bindings for the C restatement of the reference step (oracle/fvm_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, and only as the checker.

`params_from_toml` restates how the reference turns input.toml into its
globals (FVMR/src/input/TomlFileManager.cpp:110-170 and 200-265, defaults
from FVMR/src/global/GlobalPara.cpp:4-90, mu0 from Re at
TomlFileManager.cpp:79-104), plus the keys of the [gpu] table that select the
reference-compatible or corrected behaviour of three quirks.
"""
import ctypes
import math
import os
import subprocess
import tomllib

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libfvm_oracle.so")


class OmMesh(ctypes.Structure):
    _fields_ = [("N", ctypes.c_int), ("E", ctypes.c_int), ("V", ctypes.c_int), ("NB", ctypes.c_int)] + [
        (name, ctypes.c_void_p)
        for name in ("node_xy", "elem_nodes", "elem_edges", "elem_nbrs", "elem_xy", "elem_vol", "edge_nodes",
                     "edge_L", "edge_R", "edge_set", "edge_pair", "edge_len", "edge_dist", "edge_xy",
                     "edge_normal", "bc_type")
    ]


class OmParams(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int) for n in ("equation", "flux_scheme", "reconstruct", "gradient", "limiter",
                                           "time_advance", "lsq_det_ref", "wall_bc_ref", "restrict_ref", "pad_")] + [
        (n, ctypes.c_double) for n in ("gamma", "R", "Pr", "mu0", "T0", "CFL", "T_end")] + [
        ("inf", ctypes.c_double * 4), ("inlet", ctypes.c_double * 4), ("outlet", ctypes.c_double * 4),
        ("shock", ctypes.c_double * 4), ("dsr", ctypes.c_double * 3), ("dsr_time", ctypes.c_double),
        ("steady", ctypes.c_int), ("pad2_", ctypes.c_int)]


def build():
    subprocess.run(["make", "-s", "-C", HERE], check=True)


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        dp = ctypes.POINTER(ctypes.c_double)
        L.om_mesh_read_su2.restype = ctypes.POINTER(OmMesh)
        L.om_mesh_read_su2.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.c_double, ctypes.c_char_p, ctypes.c_int]
        L.om_mesh_free.argtypes = [ctypes.POINTER(OmMesh)]
        L.om_init_field.argtypes = [ctypes.POINTER(OmMesh), ctypes.POINTER(OmParams), ctypes.c_int, dp, dp]
        L.om_rhs.argtypes = [ctypes.POINTER(OmMesh), ctypes.POINTER(OmParams), dp, dp, dp, dp]
        L.om_dt.argtypes = [ctypes.POINTER(OmMesh), ctypes.POINTER(OmParams), dp, dp, dp]
        L.om_restrict.argtypes = [ctypes.POINTER(OmMesh), ctypes.POINTER(OmParams), dp]
        L.om_run.argtypes = [ctypes.POINTER(OmMesh), ctypes.POINTER(OmParams), dp, ctypes.c_int, dp, dp, dp]
        L.om_residual.argtypes = [ctypes.POINTER(OmMesh), dp, ctypes.c_int, dp]
        L.om_ruvp_from_mach.argtypes = [ctypes.c_double] * 6 + [dp]
        L.om_set_threads.argtypes = [ctypes.c_int]
        ip, fp = ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_float)
        L.om_node_field.argtypes = [ctypes.c_int, ctypes.c_int, ip, dp, ctypes.c_double, ctypes.c_double,
                                    ctypes.c_double, dp]
        L.om_node_field.restype = None
        L.om_boundary_forces.argtypes = [ctypes.c_int, ip, ip, ip, ctypes.c_int, ip, dp, dp, dp, ctypes.c_double,
                                         dp, dp, dp, dp]
        L.om_boundary_forces.restype = None
        L.om_colour_nodes.argtypes = [ctypes.c_int, ctypes.c_int, ip, dp, ctypes.c_float, ctypes.c_float, fp, fp]
        L.om_colour_nodes.restype = None
        L.om_set_threads.restype = ctypes.c_int
        L.om_set_threads(int(os.environ.get("FVM_ORACLE_THREADS", "1")))
        _lib = L
    return _lib


def set_threads(n):
    """Host threads of the oracle's loops (n <= 0 only reads them); returns the count in use."""
    return lib().om_set_threads(int(n))


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double)) if a is not None else None


def _ip(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))


def node_field(elem_nodes, U, V, gamma, inf):
    """om_node_field: (6, V) node values; elem_nodes (4, N) int32, U (4, N), inf = (rho, u, v, p)."""
    elem_nodes = np.ascontiguousarray(elem_nodes, dtype=np.int32)
    U = np.ascontiguousarray(U, dtype=np.float64)
    N = U.shape[1]
    p_inf = float(inf[3])
    pdyn = 0.5 * float(inf[0]) * (float(inf[1]) * float(inf[1]) + float(inf[2]) * float(inf[2]))
    out = np.empty((6, V))
    lib().om_node_field(N, V, _ip(elem_nodes), _dp(U), float(gamma), p_inf, pdyn, _dp(out))
    return out


def boundary_forces(set_off, set_list, bc_type, edge_nodes, edge_normal, edge_len, Cp, ref_area):
    """om_boundary_forces: (CD[NB], CL[NB], CD_wall, CL_wall)."""
    set_off = np.ascontiguousarray(set_off, dtype=np.int32)
    set_list = np.ascontiguousarray(set_list, dtype=np.int32)
    bc_type = np.ascontiguousarray(bc_type, dtype=np.int32)
    edge_nodes = np.ascontiguousarray(edge_nodes, dtype=np.int32)
    E = edge_nodes.shape[1]
    NB = len(bc_type)
    cd, cl = np.empty(NB), np.empty(NB)
    dw, lw = ctypes.c_double(), ctypes.c_double()
    lib().om_boundary_forces(NB, _ip(set_off), _ip(set_list), _ip(bc_type), E, _ip(edge_nodes),
                             _dp(np.ascontiguousarray(edge_normal, dtype=np.float64)),
                             _dp(np.ascontiguousarray(edge_len, dtype=np.float64)),
                             _dp(np.ascontiguousarray(Cp, dtype=np.float64)), float(ref_area), _dp(cd), _dp(cl),
                             ctypes.byref(dw), ctypes.byref(lw))
    return cd, cl, dw.value, lw.value


def colour_nodes(elem_nodes, U, V, lo, hi):
    """om_colour_nodes: (rgb (V, 3) float32, node values (V,) float32)."""
    elem_nodes = np.ascontiguousarray(elem_nodes, dtype=np.int32)
    U = np.ascontiguousarray(U, dtype=np.float64)
    rgb = np.empty((V, 3), dtype=np.float32)
    val = np.empty(V, dtype=np.float32)
    fp = ctypes.POINTER(ctypes.c_float)
    lib().om_colour_nodes(U.shape[1], V, _ip(elem_nodes), _dp(U), float(lo), float(hi), rgb.ctypes.data_as(fp),
                          val.ctypes.data_as(fp))
    return rgb, val


def ruvp_from_mach(Ma, aoa, T0, p0, gamma, R):
    out = np.zeros(4)
    lib().om_ruvp_from_mach(Ma, aoa, T0, p0, gamma, R, _dp(out))
    return out


# ---- input.toml -> parameters ------------------------------------------------

_QUIRK_KEYS = {"lsq_det": "lsq_det_ref", "wall_bc": "wall_bc_ref", "restrict": "restrict_ref"}


def read_config(toml_path_or_dict):
    if isinstance(toml_path_or_dict, dict):
        return toml_path_or_dict
    with open(toml_path_or_dict, "rb") as f:
        return tomllib.load(f)


def params_from_toml(cfg):
    """Returns (OmParams, info) for a parsed input.toml."""
    cfg = read_config(cfg)
    g = lambda path, default=None: _get(cfg, path, default)
    p = OmParams()
    gamma = float(g("constant.gamma", 1.4))
    T0 = float(g("constant.T0", 288.16))
    p0 = float(g("constant.p0", 101325.0))
    R = 287.06
    p.gamma, p.R, p.T0 = gamma, R, T0
    p.Pr = float(g("constant.Pr", 0.73))
    ref_area = float(g("constant.referenceArea", 1.0)) * float(g("constant.mesh_scale_factor", 1.0))
    bcs = {}
    for name in ("inf", "inlet", "outlet"):
        bcs[name] = _bc_ruvp(cfg, f"boundaryCondition.2D.{name}", gamma, T0, p0, R)
    for name in ("inf", "inlet", "outlet"):
        getattr(p, name)[:] = bcs[name]
    ic_type = int(g("initialCondition.type", 1))
    # reference flow for Re <-> mu0 (TomlFileManager.cpp:47-104)
    if ic_type in (3, 4):
        ui, uo = math.hypot(bcs["inlet"][1], bcs["inlet"][2]), math.hypot(bcs["outlet"][1], bcs["outlet"][2])
        rho_ref, U_ref = (bcs["inlet"][0], ui) if ui > uo else (bcs["outlet"][0], uo)
    else:
        rho_ref, U_ref = bcs["inf"][0], math.hypot(bcs["inf"][1], bcs["inf"][2])
    if bool(g("constant.calculate_mu0_by_Re", False)):
        Re = float(g("constant.Re", 1.0e8))
        p.mu0 = rho_ref * U_ref * ref_area / Re
    else:
        p.mu0 = float(g("constant.mu0", 17.9e-6))
    p.equation = int(g("physicsModel.equation", 1))
    p.CFL = float(g("time.CFL", 0.6))  # also in steady runs: time.CFL_steady is not used (TomlFileManager.cpp:159-160)
    p.steady = 1 if int(g("time.is_steady", 0)) else 0
    p.T_end = float(g("time.max_physical_time", 20))
    p.time_advance = int(g("time.time_advance", 3101))
    p.reconstruct = int(g("inviscid_flux_method.flag_reconstruct", 3001))
    p.gradient = int(g("inviscid_flux_method.flag_gradient", 1))
    p.flux_scheme = int(g("inviscid_flux_method.flux_conservation_scheme", 2002))
    p.limiter = int(g("inviscid_flux_method.flux_limiter", 2))
    for key, field in _QUIRK_KEYS.items():
        setattr(p, field, 1 if str(g(f"gpu.{key}", "ref")) == "ref" else 0)
    # FieldInitializer::initialize_using_config (FieldInitializer.cpp:74-110), defaults of
    # FieldInitializer.h:23-26 and CBoundaryDoubleShockReflect.h:12-14
    p.shock[:] = [float(g(f"initialCondition.shockTube.{k}", d)) for k, d in
                  (("shock_x", 0.0), ("shock_y", 0.0), ("shock_normal_x", 1.0), ("shock_normal_y", 0.0))]
    if ic_type == 4:
        p.dsr[:] = [float(g(f"initialCondition.doubleShockReflection.{k}")) for k in
                    ("shock_x", "shock_y", "shock_angle_degree")]
    else:
        p.dsr[:] = [0.0, 0.0, 60.0]
    info = {"ic_type": ic_type, "mesh_scale": float(g("constant.mesh_scale_factor", 1.0)),
            "vortex": [float(g("initialCondition.isentropicVortex.vortex_x", 0.0)),
                       float(g("initialCondition.isentropicVortex.vortex_y", 0.0)),
                       float(g("initialCondition.isentropicVortex.vortex_strength", 1.0))],
            "maxIteration": int(g("output.maxIteration", 5000))}
    return p, info


def _get(cfg, path, default=None):
    cur = cfg
    for k in path.split("."):
        if not isinstance(cur, dict) or k not in cur:
            return default
        cur = cur[k]
    return cur


def _bc_ruvp(cfg, parent, gamma, T0, p0, R):
    """TomlFileManager::getValue_boundaryCondition2D (TomlFileManager.cpp:200-265)."""
    sec = _get(cfg, parent)
    out = np.zeros(4)
    if not isinstance(sec, dict) or "input_mode" not in sec:
        return out
    mode = int(sec["input_mode"])
    if mode == 0:
        aoa = float(sec.get("AOA", sec.get("AoA", 0.0)))
        return ruvp_from_mach(float(sec["Ma"]), aoa, T0, p0, gamma, R)
    if mode == 1:
        return np.array([float(sec["rho"]), float(sec["u"]), float(sec["v"]), float(sec["p"])])
    if mode == 2:
        U = [float(sec["rho"]), float(sec["rhou"]), float(sec["rhov"]), float(sec["rhoE"])]
        r = U[0]
        u, v = U[1] / U[0], U[2] / U[0]
        return np.array([r, u, v, r * (gamma - 1) * (U[3] / U[0] - (u * u + v * v) * 0.5)])
    if mode == 3:
        ang = float(sec["angle_degree"]) * 3.1415926535897 / 180.0
        u = float(sec["u"])
        return np.array([float(sec["rho"]), u * math.cos(ang), u * math.sin(ang), float(sec["p"])])
    raise ValueError(f"invalid input_mode at {parent}")


# ---- mesh and solver ---------------------------------------------------------

class Oracle:
    """The oracle's mesh plus parameters for one case (input.toml + .su2)."""

    def __init__(self, toml, su2):
        self.params, self.info = params_from_toml(toml)
        err = ctypes.create_string_buffer(256)
        self._m = lib().om_mesh_read_su2(su2.encode(), self.params.equation, self.info["mesh_scale"], err, 256)
        if not self._m:
            raise RuntimeError(f"oracle mesh read failed: {err.value.decode()}")
        m = self._m.contents
        self.N, self.E, self.V, self.NB = m.N, m.E, m.V, m.NB

    def __del__(self):
        if getattr(self, "_m", None):
            lib().om_mesh_free(self._m)
            self._m = None

    def array(self, name):
        m = self._m.contents
        N, E, V, NB = self.N, self.E, self.V, self.NB
        spec = {"node_xy": ("d", (2, V)), "elem_nodes": ("i", (4, N)), "elem_edges": ("i", (4, N)),
                "elem_nbrs": ("i", (4, N)), "elem_xy": ("d", (2, N)), "elem_vol": ("d", (N,)),
                "edge_nodes": ("i", (2, E)), "edge_L": ("i", (E,)), "edge_R": ("i", (E,)), "edge_set": ("i", (E,)),
                "edge_pair": ("i", (E,)), "edge_len": ("d", (E,)), "edge_dist": ("d", (E,)),
                "edge_xy": ("d", (2, E)), "edge_normal": ("d", (2, E)), "bc_type": ("i", (NB,))}
        code, shape = spec[name]
        ct = ctypes.c_double if code == "d" else ctypes.c_int
        n = int(np.prod(shape))
        ptr = ctypes.cast(getattr(m, name), ctypes.POINTER(ct * n))
        return np.frombuffer(ptr.contents, dtype=np.float64 if code == "d" else np.int32).reshape(shape).copy()

    def init_field(self):
        U = np.zeros((4, self.N))
        vortex = np.array(self.info["vortex"], dtype=np.float64)
        rc = lib().om_init_field(self._m, ctypes.byref(self.params), self.info["ic_type"], _dp(vortex), _dp(U))
        if rc:
            raise RuntimeError(f"oracle init_field failed ({rc})")
        return U

    def rhs(self, U):
        U = np.ascontiguousarray(U, dtype=np.float64)
        R = np.zeros_like(U)
        gx, gy = np.zeros_like(U), np.zeros_like(U)
        rc = lib().om_rhs(self._m, ctypes.byref(self.params), _dp(U), _dp(R), _dp(gx), _dp(gy))
        if rc:
            raise RuntimeError(f"oracle rhs failed ({rc})")
        return R, gx, gy

    def dt(self, U):
        U = np.ascontiguousarray(U, dtype=np.float64)
        dt = np.zeros(1)
        alpha = np.zeros(self.N)
        rc = lib().om_dt(self._m, ctypes.byref(self.params), _dp(U), _dp(dt), _dp(alpha))
        if rc:
            raise RuntimeError(f"oracle dt failed ({rc})")
        return float(dt[0]), alpha

    def run(self, U, nsteps, t=0.0):
        U = np.array(U, dtype=np.float64, order="C")
        tt = np.array([t])
        dts = np.zeros(max(nsteps, 1))
        last = np.zeros_like(U)
        rc = lib().om_run(self._m, ctypes.byref(self.params), _dp(U), nsteps, _dp(tt), _dp(dts), _dp(last))
        if rc:
            raise RuntimeError(f"oracle run failed ({rc})")
        return U, float(tt[0]), dts[:nsteps], last

    def restrict(self, U):
        U = np.array(U, dtype=np.float64, order="C")
        n = lib().om_restrict(self._m, ctypes.byref(self.params), _dp(U))
        return U, n

    def residual(self, rhs, norm=0):
        out = np.zeros(4)
        lib().om_residual(self._m, _dp(np.ascontiguousarray(rhs, dtype=np.float64)), norm, _dp(out))
        return out
