"""GB300-native explicit finite-volume step for 2D unstructured meshes (FP64).

Python mirror of the reference's per-step interface over the C ABI of
include/fvgb.h (libfvgb.so, built in-tree by build.py):

    params = Params.from_toml("input.toml")          # TomlFileManager
    mesh = Mesh.read_su2("mesh.su2", params)          # SU2MeshReader + FVM_2D + OldDataConverter
    solver = GPUSolver2(mesh, params)                 # GPUSolver2::allocateMemory/initializeData
    t = solver.iteration_device(t, T)                 # CIteration::iteration_device
    res = solver.update_residual_vector()             # GPUSolver2::updateResidualVector

There is no CPU fallback: every compute call goes to the CUDA library, and
loading fails loudly when it is missing.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libfvgb.so")

__all__ = ["Params", "Mesh", "GPUSolver2", "FvgbError", "lib", "write_periodic_square", "write_cylinder",
           "initial_field"]


class FvgbError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"fvgb error {code}: {msg}")
        self.code = code


class Params(ctypes.Structure):
    """fvgb_params (include/fvgb.h)."""
    _fields_ = [(n, ctypes.c_int) for n in (
        "equation", "flux_scheme", "reconstruct", "gradient", "limiter", "time_advance", "lsq_det_ref",
        "wall_bc_ref", "restrict_ref", "ic_type", "renumber", "device")] + [
        (n, ctypes.c_double) for n in ("gamma", "R", "Pr", "mu0", "T0", "CFL", "T_end", "Re")] + [
        ("inf", ctypes.c_double * 4), ("inlet", ctypes.c_double * 4), ("outlet", ctypes.c_double * 4),
        ("vortex", ctypes.c_double * 3), ("shock", ctypes.c_double * 4), ("mesh_scale", ctypes.c_double),
        ("max_iteration", ctypes.c_int), ("edge_colour", ctypes.c_int), ("ref_area", ctypes.c_double),
        ("dsr", ctypes.c_double * 3), ("dsr_time", ctypes.c_double), ("steady", ctypes.c_int),
        ("pad2_", ctypes.c_int), ("CFL_steady", ctypes.c_double)]

    @classmethod
    def default(cls):
        p = cls()
        _check(lib().fvgb_params_default(ctypes.byref(p)))
        return p

    @classmethod
    def from_toml(cls, path):
        p = cls()
        name = ctypes.create_string_buffer(512)
        _check(lib().fvgb_params_read_toml(os.fsencode(path), ctypes.byref(p), name, 512))
        p.mesh_name = name.value.decode()
        return p


class MeshSoA(ctypes.Structure):
    _fields_ = [("num_node", ctypes.c_int), ("num_element", ctypes.c_int), ("num_edge", ctypes.c_int),
                ("num_boundary", ctypes.c_int)] + [
        (n, ctypes.c_void_p) for n in ("node_xy", "elem_nodes", "elem_edges", "elem_neighbors", "elem_xy",
                                       "elem_volume", "edge_nodes", "edge_L", "edge_R", "edge_setID",
                                       "edge_periodicPair", "edge_length", "edge_distance", "edge_xy",
                                       "edge_normal", "boundary_type", "set_edge_offsets", "set_edge_list",
                                       "set_names")]


_lib = None


def lib():
    """Loads libfvgb.so (building it first when it is missing or stale)."""
    global _lib
    if _lib is None:
        from . import build as _build
        try:
            _build.build()
        except Exception as exc:  # no nvcc: use a prebuilt library if present
            if not os.path.exists(LIB_PATH):
                raise RuntimeError(f"libfvgb.so is missing and cannot be built: {exc}") from exc
        L = ctypes.CDLL(LIB_PATH)
        i, d, v, c = ctypes.c_int, ctypes.c_double, ctypes.c_void_p, ctypes.c_char_p
        dp, ip = ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int)
        sig = {
            "fvgb_params_default": (i, [v]),
            "fvgb_params_read_toml": (i, [c, v, c, i]),
            "fvgb_mesh_read_su2": (i, [c, i, d, ctypes.POINTER(v)]),
            "fvgb_mesh_view": (i, [v, ctypes.POINTER(MeshSoA)]),
            "fvgb_mesh_free": (None, [v]),
            "fvgb_write_su2_periodic_square": (i, [c, i, d, d, ctypes.c_ulonglong]),
            "fvgb_write_su2_cylinder": (i, [c, i, i, d, d, d]),
            "fvgb_initial_field": (i, [ctypes.POINTER(MeshSoA), v, dp]),
            "fvgb_read_continue": (i, [c, i, ctypes.POINTER(v), dp, ip, dp]),
            "fvgb_continue_state": (i, [v, dp]),
            "fvgb_write_continue": (i, [v, c, d, i, d, dp]),
            "fvgb_find_continue_file": (i, [c, c, c, i]),
            "fvgb_run_config_read_toml": (i, [c, v]),
            "fvgb_create": (i, [ctypes.POINTER(MeshSoA), v, ctypes.POINTER(v)]),
            "fvgb_destroy": (None, [v]),
            "fvgb_set_state": (i, [v, dp]),
            "fvgb_get_state": (i, [v, dp]),
            "fvgb_step": (i, [v, dp, d, i]),
            "fvgb_step_async": (i, [v, d, i]),
            "fvgb_set_time": (i, [v, d]),
            "fvgb_set_cfl": (i, [v, d]),
            "fvgb_time": (i, [v, dp, dp]),
            "fvgb_synchronize": (i, [v]),
            "fvgb_rhs": (i, [v, dp, dp, dp, dp]),
            "fvgb_rhs_vjp": (i, [v, dp, dp, dp]),
            "fvgb_dt": (i, [v, dp]),
            "fvgb_residual": (i, [v, i, dp]),
            "fvgb_device_status": (i, [v, ctypes.POINTER(ctypes.c_longlong)]),
            "fvgb_device_state": (i, [v, ctypes.POINTER(v), ip]),
            "fvgb_cell_permutation": (i, [v, ip]),
            "fvgb_edge_permutation": (i, [v, ip]),
            "fvgb_layout_connectivity": (i, [v, ip, ip, ip, ip]),
            "fvgb_edge_colours": (i, [v, ip, ip]),
            "fvgb_kernel_launches": (ctypes.c_longlong, [v]),
            "fvgb_profile_steps": (i, [v, d, i, dp, ip]),
            "fvgb_step_timed": (i, [v, d, i, dp]),
            "fvgb_batch_create": (i, [i, ctypes.POINTER(ctypes.POINTER(MeshSoA)), v, ctypes.POINTER(v)]),
            "fvgb_batch_destroy": (None, [v]),
            "fvgb_batch_set_state": (i, [v, i, dp]),
            "fvgb_batch_get_state": (i, [v, i, dp]),
            "fvgb_batch_step": (i, [v, dp, dp, i]),
            "fvgb_batch_step_timed": (i, [v, i, dp]),
            "fvgb_batch_tune": (i, [v, i, c, i]),
            "fvgb_batch_info": (i, [v, ctypes.POINTER(ctypes.c_longlong)]),
            "fvgb_fp64_peak": (i, [i, dp]),
            "fvgb_barrier_selftest": (i, [i, i, i, ctypes.c_longlong, ip, ip]),
            "fvgb_node_field": (i, [v, dp]),
            "fvgb_boundary_forces": (i, [v, dp, dp, dp, dp]),
            "fvgb_write_tecplot_volume": (i, [v, c, c, d, i]),
            "fvgb_write_tecplot_boundary": (i, [v, c, d, i]),
            "fvgb_colour_nodes": (i, [v, d, d, ctypes.POINTER(ctypes.POINTER(ctypes.c_float)),
                                      ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float)]),
            "fvgb_num_nodes": (i, [v, ip]),
            "fvgb_output_timed": (i, [v, i, dp, dp]),
            "fvgb_last_error": (c, []),
            "fvgb_version": (c, []),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _check(rc):
    if rc != 0:
        raise FvgbError(rc, lib().fvgb_last_error().decode())
    return rc


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double)) if a is not None else None


def _ip(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int)) if a is not None else None


class Mesh:
    """Host mesh in the reference's numbering (fvgb_mesh)."""

    def __init__(self, ptr):
        self._ptr = ptr
        self.soa = MeshSoA()
        _check(lib().fvgb_mesh_view(self._ptr, ctypes.byref(self.soa)))
        s = self.soa
        self.V, self.N, self.E, self.NB = s.num_node, s.num_element, s.num_edge, s.num_boundary

    @classmethod
    def read_su2(cls, path, params=None, equation=None, scale=None):
        eq = equation if equation is not None else (params.equation if params is not None else 1)
        sc = scale if scale is not None else (params.mesh_scale if params is not None else 1.0)
        ptr = ctypes.c_void_p()
        _check(lib().fvgb_mesh_read_su2(os.fsencode(path), int(eq), float(sc), ctypes.byref(ptr)))
        return cls(ptr)

    @classmethod
    def read_continue(cls, path, params=None, equation=None):
        """A continue (pause_*.dat) file: returns (mesh, U[4][N], t, istep, CFL or None)."""
        eq = equation if equation is not None else (params.equation if params is not None else 1)
        ptr = ctypes.c_void_p()
        t, istep, cfl = ctypes.c_double(), ctypes.c_int(), ctypes.c_double()
        _check(lib().fvgb_read_continue(os.fsencode(path), int(eq), ctypes.byref(ptr), ctypes.byref(t),
                                        ctypes.byref(istep), ctypes.byref(cfl)))
        mesh = cls(ptr)
        U = np.empty((4, mesh.N))
        _check(lib().fvgb_continue_state(mesh._ptr, _dp(U)))
        return mesh, U, t.value, istep.value, (cfl.value if cfl.value >= 0 else None)

    def write_continue(self, path, U, t, istep, cfl):
        """FieldWriter::writeContinueFile_1's format, 17 significant digits."""
        U = np.ascontiguousarray(U, dtype=np.float64)
        if U.shape != (4, self.N):
            raise ValueError(f"U must be (4, {self.N})")
        _check(lib().fvgb_write_continue(self._ptr, os.fsencode(path), float(t), int(istep), float(cfl), _dp(U)))

    def __del__(self):
        if getattr(self, "_ptr", None):
            lib().fvgb_mesh_free(self._ptr)
            self._ptr = None

    def array(self, name):
        N, E, V, NB = self.N, self.E, self.V, self.NB
        spec = {"node_xy": ("d", (2, V)), "elem_nodes": ("i", (4, N)), "elem_edges": ("i", (4, N)),
                "elem_neighbors": ("i", (4, N)), "elem_xy": ("d", (2, N)), "elem_volume": ("d", (N,)),
                "edge_nodes": ("i", (2, E)), "edge_L": ("i", (E,)), "edge_R": ("i", (E,)),
                "edge_setID": ("i", (E,)), "edge_periodicPair": ("i", (E,)), "edge_length": ("d", (E,)),
                "edge_distance": ("d", (E,)), "edge_xy": ("d", (2, E)), "edge_normal": ("d", (2, E)),
                "boundary_type": ("i", (NB,)), "set_edge_offsets": ("i", (NB + 1,))}
        if name == "set_edge_list":
            spec[name] = ("i", (int(self.array("set_edge_offsets")[-1]),))
        code, shape = spec[name]
        ct = ctypes.c_double if code == "d" else ctypes.c_int
        n = int(np.prod(shape))
        ptr = ctypes.cast(getattr(self.soa, name), ctypes.POINTER(ct * n))
        return np.frombuffer(ptr.contents, dtype=np.float64 if code == "d" else np.int32).reshape(shape).copy()


class RunConfig(ctypes.Structure):
    """fvgb_run_config (include/fvgb.h): the driver loop's keys of input.toml."""
    _fields_ = [("continue_run", ctypes.c_int), ("step_per_print", ctypes.c_int),
                ("step_per_output_field", ctypes.c_int), ("step_per_output_hist", ctypes.c_int),
                ("start_output_field", ctypes.c_int), ("max_iteration", ctypes.c_int),
                ("tolerance_residual", ctypes.c_double), ("filename", ctypes.c_char * 256),
                ("mesh_file_type", ctypes.c_char * 16), ("volume_preset", ctypes.c_int),
                ("boundary_preset", ctypes.c_int), ("time_strategy", ctypes.c_int)]


def run_config(path):
    """The driver's keys of input.toml (fvgb_run_config_read_toml) as a dict."""
    c = RunConfig()
    _check(lib().fvgb_run_config_read_toml(os.fsencode(path), ctypes.byref(c)))
    out = {name: getattr(c, name) for name, _ in RunConfig._fields_}
    out["filename"] = c.filename.decode()
    out["mesh_file_type"] = c.mesh_file_type.decode()
    return out


def find_continue_file(directory, name):
    """The newest pause_<name>[n].dat in directory (largest n > 0), or None."""
    buf = ctypes.create_string_buffer(4096)
    rc = lib().fvgb_find_continue_file(os.fsencode(directory), os.fsencode(name), buf, 4096)
    if rc == -2:  # FVGB_ERR_IO: none there
        return None
    _check(rc)
    return os.fsdecode(buf.value)


def barrier_selftest(blocks=8, absent_block=-1, spin_limit=200000, device=0):
    """fvgb_barrier_selftest: (timed_out, blocks whose wait succeeded)."""
    t, passed = ctypes.c_int(), ctypes.c_int()
    _check(lib().fvgb_barrier_selftest(int(device), int(blocks), int(absent_block), int(spin_limit),
                                       ctypes.byref(t), ctypes.byref(passed)))
    return bool(t.value), passed.value


def fp64_peak(device=0):
    """The device's FP64 rate in GFLOP/s (FMA = 2 flops), measured now (fvgb_fp64_peak)."""
    g = ctypes.c_double()
    _check(lib().fvgb_fp64_peak(int(device), ctypes.byref(g)))
    return g.value


def initial_field(mesh, params):
    U = np.zeros((4, mesh.N))
    _check(lib().fvgb_initial_field(ctypes.byref(mesh.soa), ctypes.byref(params), _dp(U)))
    return U


def write_periodic_square(path, n, L=10.0, jitter=0.0, seed=20261203):
    _check(lib().fvgb_write_su2_periodic_square(os.fsencode(path), int(n), float(L), float(jitter), int(seed)))


def write_cylinder(path, n_theta, n_r, r0=0.5, r1=20.0, first_dr=1e-3):
    _check(lib().fvgb_write_su2_cylinder(os.fsencode(path), int(n_theta), int(n_r), float(r0), float(r1),
                                          float(first_dr)))


class GPUSolver2:
    """One solver on one GPU (fvgb_handle); names follow GPU::GPUSolver2 and CIteration."""

    def __init__(self, mesh, params):
        self.mesh, self.params = mesh, params
        self._h = ctypes.c_void_p()
        _check(lib().fvgb_create(ctypes.byref(mesh.soa), ctypes.byref(params), ctypes.byref(self._h)))
        self.N, self.E = mesh.N, mesh.E

    def close(self):
        if getattr(self, "_h", None):
            lib().fvgb_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    # state ---------------------------------------------------------------
    def set_state(self, U):
        U = np.ascontiguousarray(U, dtype=np.float64)
        if U.shape != (4, self.N):
            raise ValueError(f"state must have shape (4, {self.N})")
        _check(lib().fvgb_set_state(self._h, _dp(U)))

    def get_state(self, out=None):
        U = out if out is not None else np.empty((4, self.N))
        _check(lib().fvgb_get_state(self._h, _dp(U)))
        return U

    def set_state_ptr(self, host_ptr):
        _check(lib().fvgb_set_state(self._h, ctypes.cast(host_ptr, ctypes.POINTER(ctypes.c_double))))

    def get_state_ptr(self, host_ptr):
        _check(lib().fvgb_get_state(self._h, ctypes.cast(host_ptr, ctypes.POINTER(ctypes.c_double))))

    # stepping --------------------------------------------------------------
    def iteration_device(self, t, T):
        """One step of CIteration::iteration_device; returns the new time."""
        return self.step(t, T, 1)

    def step(self, t, T, nsteps):
        tt = ctypes.c_double(t)
        _check(lib().fvgb_step(self._h, ctypes.byref(tt), float(T), int(nsteps)))
        return tt.value

    def step_async(self, T, nsteps):
        _check(lib().fvgb_step_async(self._h, float(T), int(nsteps)))

    def set_time(self, t):
        _check(lib().fvgb_set_time(self._h, float(t)))

    def set_cfl(self, CFL):
        _check(lib().fvgb_set_cfl(self._h, float(CFL)))

    def time(self):
        t, dt = ctypes.c_double(), ctypes.c_double()
        _check(lib().fvgb_time(self._h, ctypes.byref(t), ctypes.byref(dt)))
        return t.value, dt.value

    def synchronize(self):
        _check(lib().fvgb_synchronize(self._h))

    # parity hooks --------------------------------------------------------------
    def rhs(self, U, gradients=False):
        U = np.ascontiguousarray(U, dtype=np.float64)
        R = np.empty_like(U)
        gx = np.empty_like(U) if gradients else None
        gy = np.empty_like(U) if gradients else None
        _check(lib().fvgb_rhs(self._h, _dp(U), _dp(R), _dp(gx), _dp(gy)))
        return (R, gx, gy) if gradients else R

    def rhs_vjp(self, U, seed):
        """(dR/dU)^T seed at U, R = rhs(U) (fvgb_rhs_vjp); arrays [4][N], reference numbering."""
        U = np.ascontiguousarray(U, dtype=np.float64)
        seed = np.ascontiguousarray(seed, dtype=np.float64)
        g = np.empty_like(U)
        _check(lib().fvgb_rhs_vjp(self._h, _dp(U), _dp(seed), _dp(g)))
        return g

    def dt(self):
        out = ctypes.c_double()
        _check(lib().fvgb_dt(self._h, ctypes.byref(out)))
        return out.value

    # field output --------------------------------------------------------------
    def node_field(self):
        """FieldWriter::update_nodeField on the device: (6, V) = rho, u, v, p, Cp, Ma per node."""
        out = np.empty((6, self.num_nodes()))
        _check(lib().fvgb_node_field(self._h, _dp(out)))
        return out

    def num_nodes(self):
        v = ctypes.c_int()
        _check(lib().fvgb_num_nodes(self._h, ctypes.byref(v)))
        return v.value

    def boundary_forces(self, n_sets):
        """calculate_edgeSet_force: (CD[NB], CL[NB], CD_wall, CL_wall)."""
        cd, cl = np.empty(n_sets), np.empty(n_sets)
        dw, lw = ctypes.c_double(), ctypes.c_double()
        _check(lib().fvgb_boundary_forces(self._h, _dp(cd), _dp(cl), ctypes.byref(dw), ctypes.byref(lw)))
        return cd, cl, dw.value, lw.value

    def write_tecplot_volume(self, path, t, title="title", preset=2):
        _check(lib().fvgb_write_tecplot_volume(self._h, os.fsencode(path), title.encode(), float(t), int(preset)))

    def write_tecplot_boundary(self, path, t, preset=1):
        _check(lib().fvgb_write_tecplot_boundary(self._h, os.fsencode(path), float(t), int(preset)))

    def colour_nodes(self, range_lo=0.0, range_hi=1.0):
        """The GUI's field colouring into a device buffer; returns (rgb (V, 3) float32, node values (V,),
        device pointer of the [V][3] buffer)."""
        V = self.num_nodes()
        rgb = np.empty((V, 3), dtype=np.float32)
        val = np.empty(V, dtype=np.float32)
        dev = ctypes.POINTER(ctypes.c_float)()
        fp = ctypes.POINTER(ctypes.c_float)
        _check(lib().fvgb_colour_nodes(self._h, float(range_lo), float(range_hi), ctypes.byref(dev),
                                       rgb.ctypes.data_as(fp), val.ctypes.data_as(fp)))
        return rgb, val, ctypes.cast(dev, ctypes.c_void_p).value

    def output_timed(self, reps):
        """Device ms of reps node-value launches and of reps colouring launches."""
        a, b = ctypes.c_double(), ctypes.c_double()
        _check(lib().fvgb_output_timed(self._h, int(reps), ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value

    def update_residual_vector(self, norm=0):
        out = np.zeros(4)
        _check(lib().fvgb_residual(self._h, int(norm), _dp(out)))
        return out

    def device_status(self):
        out = (ctypes.c_longlong * 4)()
        _check(lib().fvgb_device_status(self._h, out))
        return list(out)

    def device_state(self):
        p, n = ctypes.c_void_p(), ctypes.c_int()
        _check(lib().fvgb_device_state(self._h, ctypes.byref(p), ctypes.byref(n)))
        return p.value, n.value

    def cell_permutation(self):
        out = np.empty(self.N, dtype=np.int32)
        _check(lib().fvgb_cell_permutation(self._h, _ip(out)))
        return out

    def edge_permutation(self):
        out = np.empty(self.E, dtype=np.int32)
        _check(lib().fvgb_edge_permutation(self._h, _ip(out)))
        return out

    def edge_colours(self):
        """(colour of each reference edge, number of colours) of [gpu] edge_colour = 1."""
        out = np.empty(self.E, dtype=np.int32)
        n = ctypes.c_int()
        _check(lib().fvgb_edge_colours(self._h, _ip(out), ctypes.byref(n)))
        return out, n.value

    def layout_connectivity(self):
        ee = np.empty((3, self.N), dtype=np.int32)
        nb = np.empty((3, self.N), dtype=np.int32)
        eL = np.empty(self.E, dtype=np.int32)
        eR = np.empty(self.E, dtype=np.int32)
        _check(lib().fvgb_layout_connectivity(self._h, _ip(ee), _ip(nb), _ip(eL), _ip(eR)))
        return ee, nb, eL, eR

    def kernel_launches(self):
        return int(lib().fvgb_kernel_launches(self._h))

    def step_timed(self, T, nsteps):
        """nsteps bracketed by CUDA events on the solver's stream; returns device milliseconds."""
        ms = ctypes.c_double()
        _check(lib().fvgb_step_timed(self._h, float(T), int(nsteps), ctypes.byref(ms)))
        return ms.value

    PROFILE_GROUPS = ("dt", "gradient", "flux", "update", "restrict")

    def profile_steps(self, T, nsteps):
        """Per kernel group: (total ms, number of timed launches) over nsteps run without the graph."""
        ms = np.zeros(5)
        cnt = np.zeros(5, dtype=np.int32)
        _check(lib().fvgb_profile_steps(self._h, float(T), int(nsteps), _dp(ms), _ip(cnt)))
        return {k: (float(ms[i]), int(cnt[i])) for i, k in enumerate(self.PROFILE_GROUPS)}


class Batch:
    """Many Euler instances (fvgb_batch): one persistent launch per Runge-Kutta stage."""

    def __init__(self, meshes, params_list):
        if len(meshes) != len(params_list) or not meshes:
            raise ValueError("one parameter set per mesh")
        self.meshes, self.params = list(meshes), list(params_list)
        self.n = len(meshes)
        arr_m = (ctypes.POINTER(MeshSoA) * self.n)(*[ctypes.pointer(m.soa) for m in self.meshes])
        arr_p = (Params * self.n)(*self.params)
        self._h = ctypes.c_void_p()
        _check(lib().fvgb_batch_create(self.n, arr_m, ctypes.cast(arr_p, ctypes.c_void_p), ctypes.byref(self._h)))
        self.t = np.zeros(self.n)

    def close(self):
        if getattr(self, "_h", None):
            lib().fvgb_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def set_state(self, i, U):
        U = np.ascontiguousarray(U, dtype=np.float64)
        _check(lib().fvgb_batch_set_state(self._h, int(i), _dp(U)))

    def get_state(self, i):
        U = np.empty((4, self.meshes[i].N))
        _check(lib().fvgb_batch_get_state(self._h, int(i), _dp(U)))
        return U

    def step(self, nsteps, T=None):
        t = np.ascontiguousarray(self.t, dtype=np.float64)
        TT = None if T is None else np.ascontiguousarray(T, dtype=np.float64)
        _check(lib().fvgb_batch_step(self._h, _dp(t), _dp(TT), int(nsteps)))
        self.t = t
        return t

    def step_timed(self, nsteps):
        ms = ctypes.c_double()
        _check(lib().fvgb_batch_step_timed(self._h, int(nsteps), ctypes.byref(ms)))
        return ms.value

    def tune(self, trial_steps=2):
        buf = ctypes.create_string_buffer(8192)
        _check(lib().fvgb_batch_tune(self._h, int(trial_steps), buf, 8192))
        return buf.value.decode()

    def info(self):
        out = (ctypes.c_longlong * 8)()
        _check(lib().fvgb_batch_info(self._h, out))
        keys = ("instances", "cells", "edges", "grid", "block", "launches", "tile", "graph")
        return dict(zip(keys, list(out)))


def _bind_adjoint():
    L = lib()
    dp = ctypes.POINTER(ctypes.c_double)
    L.fvgb_adjoint_forward.restype = ctypes.c_int
    L.fvgb_adjoint_forward.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, dp, ctypes.c_double, dp, dp]
    L.fvgb_adjoint_backward.restype = ctypes.c_int
    L.fvgb_adjoint_backward.argtypes = [ctypes.c_void_p, dp, dp, dp]
    L.fvgb_adjoint_release.restype = None
    L.fvgb_adjoint_release.argtypes = [ctypes.c_void_p]
    L.fvgb_adjoint_overlap.restype = ctypes.c_int
    L.fvgb_adjoint_overlap.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_int)]
    return L


def adjoint_overlap(solver, mode=None):
    """Sets (mode 1 or 0, from the next adjoint_forward) whether the backward sweep recomputes
    each segment beside the reverse of the next on a second stream; returns whether the
    current adjoint workspace does (False before the first adjoint_forward)."""
    L = _bind_adjoint()
    if mode is not None:
        solver._adj_overlap = 1 if mode else 0
    cur = ctypes.c_int()
    _check(L.fvgb_adjoint_overlap(solver._h, getattr(solver, "_adj_overlap", 1), ctypes.byref(cur)))
    return bool(cur.value)


def adjoint_forward(solver, U0, nsteps, n_checkpoints=None, t0=0.0):
    """K steps from U0 keeping checkpoints; returns (U_K, forward milliseconds)."""
    L = _bind_adjoint()
    U0 = np.ascontiguousarray(U0, dtype=np.float64)
    UK = np.empty_like(U0)
    ms = ctypes.c_double()
    nck = n_checkpoints if n_checkpoints is not None else max(1, int(round(np.sqrt(nsteps))))
    _check(L.fvgb_adjoint_forward(solver._h, int(nsteps), int(nck), _dp(U0), float(t0), _dp(UK), ctypes.byref(ms)))
    return UK, ms.value


def adjoint_backward(solver, seed):
    """dL/dU_0 for the seed dL/dU_K of the last adjoint_forward; returns (grad, backward milliseconds)."""
    L = _bind_adjoint()
    seed = np.ascontiguousarray(seed, dtype=np.float64)
    g = np.empty_like(seed)
    ms = ctypes.c_double()
    _check(L.fvgb_adjoint_backward(solver._h, _dp(seed), _dp(g), ctypes.byref(ms)))
    return g, ms.value
