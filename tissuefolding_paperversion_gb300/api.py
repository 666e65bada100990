"""ctypes binding of libtfgpu.so (include/tf_gpu.h).

Python is plumbing here: tests and the benchmark drive the C ABI through this
module exactly as a C or C++ host would.  Loading fails loudly when the
library is missing -- there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

TF_OK = 0
TF_NOT_CONVERGED = 1
TF_KRYLOV_NOT_CONVERGED = 2
TF_KRYLOV_BREAKDOWN = 3
TF_NAN_DETECTED = 4
TF_BAD_INPUT = 5
TF_CUDA_ERROR = 6
TF_NO_DEVICE = 7
TF_OUT_OF_MEMORY = 8

EXPORTED = [
    "tf_status_string", "tf_last_error", "tf_create", "tf_destroy", "tf_set_positions", "tf_get_positions",
    "tf_set_Fg", "tf_get_Fg", "tf_set_growth_rates", "tf_begin_step", "tf_assemble", "tf_add_external_forces",
    "tf_solve", "tf_update", "tf_end_step", "tf_newton_step", "tf_get_residual", "tf_get_delta_u",
    "tf_get_viscosity_surfaces", "tf_set_viscosity_surfaces", "tf_set_state", "tf_export_csr",
    "tf_element_eval", "tf_get_sizes", "tf_get_stream", "tf_launch_count", "tf_time_assembly",
    "tf_solve_bsr_static", "tf_batch_create", "tf_batch_step", "tf_get_instances", "tf_elements_per_cta",
    "tf_solve_variants",
    "tf_adj_forward", "tf_adj_backward", "tf_adj_free", "tf_multigrid_info", "tf_multigrid_blocks", "tf_read_mesh_file",
    "tf_write_frame", "tf_add_K_triplets", "tf_set_dof_bindings", "tf_set_packing", "tf_get_packing",
    "tf_packing_masses", "tf_add_uniform_growth", "tf_add_ring_growth", "tf_add_grid_growth",
    "tf_clear_growth_functions", "tf_set_grid_growth_mode",
    "tf_repin_grid_growth", "tf_grid_growth_positions", "tf_set_time", "tf_get_time", "tf_measure_bandwidth",
]


def measure_bandwidth(device: int = 0, nbytes: int = 2 << 30, reps: int = 10) -> dict:
    """HBM bandwidth of a 16-byte-load read stream, a bulk-copy (TMA) read
    stream and a copy on `device`, in GB/s (tf_measure_bandwidth)."""
    L = load()
    r, b, c = C.c_double(), C.c_double(), C.c_double()
    st = L.tf_measure_bandwidth(device, nbytes, reps, C.byref(r), C.byref(b), C.byref(c))
    if st != 0:
        raise TfError(f"tf_measure_bandwidth: {L.tf_status_string(st).decode()}: {L.tf_last_error().decode()}")
    return {"read_gbs": r.value, "bulk_read_gbs": b.value, "copy_gbs": c.value, "bytes": nbytes}


class TfError(RuntimeError):
    def __init__(self, status: int, where: str, msg: str):
        super().__init__(f"{where}: status {status} ({msg})")
        self.status = status


class tf_mesh(C.Structure):
    _fields_ = [("n_nodes", C.c_int32), ("n_elems", C.c_int32), ("node_pos", C.c_void_p), ("conn", C.c_void_p),
                ("fixed", C.c_void_p), ("ext_visc", C.c_void_p), ("node_placement", C.c_void_p),
                ("ref_pos", C.c_void_p)]


class tf_material(C.Structure):
    _fields_ = [("E", C.c_void_p), ("nu", C.c_void_p), ("eta", C.c_void_p)]


class tf_options(C.Structure):
    _fields_ = [("newton_tol", C.c_double), ("newton_max_iter", C.c_int32), ("krylov_rtol", C.c_double),
                ("krylov_max_iter", C.c_int32), ("krylov_method", C.c_int32), ("deterministic", C.c_int32),
                ("device", C.c_int32), ("autotune_off", C.c_int32), ("precond", C.c_int32),
                ("update_atol", C.c_double), ("host_loops", C.c_int32), ("multigrid_reuse_steps", C.c_int32)]


class tf_step_stats(C.Structure):
    _fields_ = [("newton_iters", C.c_int32), ("krylov_iters_total", C.c_int32), ("krylov_iters_max", C.c_int32),
                ("converged", C.c_int32), ("dunorm", C.c_double * 32), ("final_relres", C.c_double),
                ("ms_assemble", C.c_float), ("ms_solve", C.c_float), ("ms_total", C.c_float),
                ("device_iters", C.c_int32), ("device_handback", C.c_int32)]


_lib = None


def checked() -> bool:
    """TF_CHECKED=1 in the environment selects the checked build."""
    return os.environ.get("TF_CHECKED") == "1"


def library_path() -> str:
    return _build.LIB_CHECKED if checked() else _build.LIB


def load(build_if_missing: bool = True):
    """Loads libtfgpu.so (building it first when it is missing)."""
    global _lib
    if _lib is not None:
        return _lib
    path = library_path()
    if not os.path.exists(path):
        if not build_if_missing:
            raise RuntimeError(f"{path} is missing; run tissuefolding_paperversion_gb300.build.build()")
        _build.build(checked=checked())
    L = C.CDLL(path)
    vp, dp, ip, i32, i64 = C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_int32), C.c_int32, C.c_int64
    L.tf_status_string.restype = C.c_char_p
    L.tf_status_string.argtypes = [C.c_int]
    L.tf_last_error.restype = C.c_char_p
    L.tf_create.argtypes = [C.POINTER(tf_mesh), C.POINTER(tf_material), C.POINTER(tf_options), C.POINTER(vp)]
    for name in ["tf_destroy", "tf_begin_step", "tf_assemble", "tf_end_step"]:
        getattr(L, name).argtypes = [vp] if name != "tf_begin_step" else [vp, C.c_double]
    for name in ["tf_set_positions", "tf_get_positions", "tf_set_Fg", "tf_set_growth_rates",
                 "tf_add_external_forces", "tf_get_residual", "tf_get_delta_u", "tf_get_viscosity_surfaces",
                 "tf_set_viscosity_surfaces"]:
        getattr(L, name).argtypes = [vp, vp]
    L.tf_get_Fg.argtypes = [vp, vp, vp]
    L.tf_solve.argtypes = [vp, ip, dp]
    L.tf_update.argtypes = [vp, ip, dp]
    L.tf_newton_step.argtypes = [vp, C.c_double, C.POINTER(tf_step_stats)]
    L.tf_set_state.argtypes = [vp, vp, vp, C.c_double]
    L.tf_export_csr.argtypes = [vp, C.c_double, vp, vp, vp, C.POINTER(i64)]
    L.tf_element_eval.argtypes = [vp, i32, i32, vp, vp, vp, vp]
    L.tf_get_sizes.argtypes = [vp, C.POINTER(i64), C.POINTER(i64), C.POINTER(i64)]
    L.tf_get_stream.restype = vp
    L.tf_get_stream.argtypes = [vp]
    L.tf_launch_count.restype = i64
    L.tf_launch_count.argtypes = [vp]
    L.tf_time_assembly.argtypes = [vp, i32, C.POINTER(C.c_float), C.POINTER(C.c_float)]
    L.tf_batch_create.restype = C.c_int
    L.tf_batch_create.argtypes = [C.POINTER(tf_mesh), C.POINTER(tf_material), i32, C.POINTER(tf_options), C.POINTER(vp)]
    L.tf_batch_step.restype = C.c_int
    L.tf_batch_step.argtypes = [vp, C.c_double, vp, vp, C.POINTER(tf_step_stats)]
    L.tf_get_instances.restype = C.c_int
    L.tf_get_instances.argtypes = [vp, ip, vp, vp]
    L.tf_elements_per_cta.restype = i32
    L.tf_elements_per_cta.argtypes = [vp]
    L.tf_solve_variants.argtypes = [vp, ip, ip]
    L.tf_solve_bsr_static.restype = C.c_int
    L.tf_solve_bsr_static.argtypes = [i32, vp, vp, vp, vp, vp, C.c_double, i32, vp, ip, dp]
    L.tf_adj_forward.restype = C.c_int
    L.tf_adj_forward.argtypes = [vp, vp, vp, i32, C.c_double, i32, vp, dp, C.POINTER(vp)]
    L.tf_adj_backward.restype = C.c_int
    L.tf_adj_backward.argtypes = [vp, vp, C.c_double, vp, vp]
    L.tf_adj_free.restype = C.c_int
    L.tf_adj_free.argtypes = [vp]
    L.tf_multigrid_info.restype = C.c_int
    L.tf_multigrid_info.argtypes = [vp, ip, vp, vp]
    L.tf_multigrid_blocks.argtypes = [vp, vp, vp]
    L.tf_set_dof_bindings.restype = C.c_int
    L.tf_set_dof_bindings.argtypes = [vp, i32, vp, vp]
    L.tf_add_K_triplets.restype = C.c_int
    L.tf_add_K_triplets.argtypes = [vp, i64, vp, vp, vp]
    L.tf_set_packing.restype = C.c_int
    L.tf_set_packing.argtypes = [vp, i32, i32]
    L.tf_get_packing.restype = C.c_int
    L.tf_get_packing.argtypes = [vp, C.POINTER(C.c_int64), vp, vp, vp, C.POINTER(C.c_double),
                                 C.POINTER(C.c_double)]
    L.tf_packing_masses.restype = C.c_int
    L.tf_packing_masses.argtypes = [vp, vp]
    L.tf_add_grid_growth.restype = C.c_int
    L.tf_add_grid_growth.argtypes = [vp, i32, i32, vp, vp, C.c_double, C.c_double, C.c_double, C.c_double]
    L.tf_add_uniform_growth.restype = C.c_int
    L.tf_add_uniform_growth.argtypes = [vp, vp, C.c_double, C.c_double, C.c_double, C.c_double, C.c_double]
    L.tf_add_ring_growth.restype = C.c_int
    L.tf_add_ring_growth.argtypes = [vp, C.c_double, C.c_double, C.c_double, C.c_double, vp, C.c_double,
                                     C.c_double, C.c_double, C.c_double, C.c_double]
    L.tf_clear_growth_functions.restype = C.c_int
    L.tf_clear_growth_functions.argtypes = [vp]
    L.tf_set_grid_growth_mode.restype = C.c_int
    L.tf_set_grid_growth_mode.argtypes = [vp, i32, i32]
    L.tf_repin_grid_growth.restype = C.c_int
    L.tf_repin_grid_growth.argtypes = [vp]
    L.tf_grid_growth_positions.restype = C.c_int
    L.tf_grid_growth_positions.argtypes = [vp, vp, vp, vp]
    L.tf_measure_bandwidth.restype = C.c_int
    L.tf_measure_bandwidth.argtypes = [i32, i64, i32, dp, dp, dp]
    L.tf_set_time.restype = C.c_int
    L.tf_set_time.argtypes = [vp, C.c_double]
    L.tf_get_time.restype = C.c_int
    L.tf_get_time.argtypes = [vp, C.POINTER(C.c_double)]
    L.tf_read_mesh_file.restype = C.c_int
    L.tf_read_mesh_file.argtypes = [C.c_char_p, ip, ip, vp, vp, vp, vp, vp, vp]
    L.tf_write_frame.restype = C.c_int
    L.tf_write_frame.argtypes = [C.c_char_p, i32, C.c_double, i32, vp, vp, vp, vp, i32, vp, vp]
    for name in ["tf_create", "tf_destroy", "tf_set_positions", "tf_get_positions", "tf_set_Fg", "tf_get_Fg",
                 "tf_set_growth_rates", "tf_begin_step", "tf_assemble", "tf_add_external_forces", "tf_solve",
                 "tf_update", "tf_end_step", "tf_newton_step", "tf_get_residual", "tf_get_delta_u",
                 "tf_get_viscosity_surfaces", "tf_set_viscosity_surfaces", "tf_set_state", "tf_export_csr",
                 "tf_element_eval", "tf_get_sizes", "tf_time_assembly"]:
        getattr(L, name).restype = C.c_int
    _lib = L
    return L


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


def _mesh_structs(t):
    a = dict(
        pos=np.ascontiguousarray(t.pos, dtype=np.float64),
        conn=np.ascontiguousarray(t.conn, dtype=np.int32),
        fixed=np.ascontiguousarray(t.fixed, dtype=np.uint8),
        ext_visc=np.ascontiguousarray(t.ext_visc, dtype=np.float64),
        placement=np.ascontiguousarray(t.node_placement, dtype=np.int32),
        E=np.ascontiguousarray(t.E, dtype=np.float64),
        nu=np.ascontiguousarray(t.nu, dtype=np.float64),
        eta=np.ascontiguousarray(t.eta, dtype=np.float64),
    )
    ref = getattr(t, "ref_pos", None)
    a["ref"] = None if ref is None else np.ascontiguousarray(ref, dtype=np.float64)
    m = tf_mesh(t.n_nodes, t.n_elems, _ptr(a["pos"]), _ptr(a["conn"]), _ptr(a["fixed"]), _ptr(a["ext_visc"]),
                _ptr(a["placement"]), _ptr(a["ref"]))
    mat = tf_material(_ptr(a["E"]), _ptr(a["nu"]), _ptr(a["eta"]))
    return a, m, mat


class Solver:
    """One GPU Newton solver over one tissue (a ``tf_handle``).  The keyword
    arguments are the fields of ``tf_options``.  ``precond``: 0 auto
    (smoothed-aggregation multigrid from 20,000 nodes on, else block-Jacobi),
    1 block-Jacobi, 2 smoothed-aggregation multigrid, 3 plain-aggregation
    multigrid.  ``update_atol``: the absolute accuracy a Newton update needs
    (0: newton_tol x 1e-4, negative: every solve to krylov_rtol).
    ``host_loops``: host-driven Newton iterations and host-checked Krylov
    chunks instead of the device-side loops (same results).
    ``multigrid_reuse_steps``: time steps the multigrid's coarse levels are
    kept for (0: the default, 4; negative: rebuilt at every step)."""

    def __init__(self, tissue, newton_tol=1e-8, newton_max_iter=20, krylov_rtol=1e-8, krylov_max_iter=20000,
                 krylov_method=0, deterministic=False, device=0, autotune=True, precond=0, update_atol=0.0,
                 host_loops=False, multigrid_reuse_steps=0):
        self.L = load()
        t = tissue
        self.t = t
        self.nn, self.ne = t.n_nodes, t.n_elems
        self._arrays, m, mat = _mesh_structs(t)
        opt = tf_options(newton_tol, newton_max_iter, krylov_rtol, krylov_max_iter, krylov_method,
                         1 if deterministic else 0, device, 0 if autotune else 1, precond, update_atol,
                         1 if host_loops else 0, multigrid_reuse_steps)
        h = C.c_void_p()
        self._check(self.L.tf_create(C.byref(m), C.byref(mat), C.byref(opt), C.byref(h)), "tf_create")
        self.h = h

    # -- plumbing -----------------------------------------------------------
    def _check(self, s, where, allow=()):
        if s != TF_OK and s not in allow:
            msg = self.L.tf_last_error().decode()
            raise TfError(s, where, msg)
        return s

    def close(self):
        if getattr(self, "h", None):
            self.L.tf_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- state --------------------------------------------------------------
    def set_positions(self, pos):
        p = np.ascontiguousarray(pos, dtype=np.float64)
        self._check(self.L.tf_set_positions(self.h, _ptr(p)), "tf_set_positions")

    def positions(self):
        p = np.zeros(3 * self.nn)
        self._check(self.L.tf_get_positions(self.h, _ptr(p)), "tf_get_positions")
        return p

    def set_Fg(self, Fg):
        f = np.ascontiguousarray(Fg, dtype=np.float64)
        self._check(self.L.tf_set_Fg(self.h, _ptr(f)), "tf_set_Fg")

    def get_Fg(self):
        f = np.zeros(9 * self.ne)
        i = np.zeros(9 * self.ne)
        self._check(self.L.tf_get_Fg(self.h, _ptr(f), _ptr(i)), "tf_get_Fg")
        return f, i

    def set_growth_rates(self, rates):
        r = None if rates is None else np.ascontiguousarray(rates, dtype=np.float64)
        self._check(self.L.tf_set_growth_rates(self.h, _ptr(r)), "tf_set_growth_rates")

    def set_state(self, uk, un, dt):
        a = np.ascontiguousarray(uk, dtype=np.float64)
        b = np.ascontiguousarray(un, dtype=np.float64)
        self._check(self.L.tf_set_state(self.h, _ptr(a), _ptr(b), dt), "tf_set_state")

    def set_viscosity_surfaces(self, area):
        a = np.ascontiguousarray(area, dtype=np.float64)
        self._check(self.L.tf_set_viscosity_surfaces(self.h, _ptr(a)), "tf_set_viscosity_surfaces")

    def viscosity_surfaces(self):
        a = np.zeros(self.nn)
        self._check(self.L.tf_get_viscosity_surfaces(self.h, _ptr(a)), "tf_get_viscosity_surfaces")
        return a

    # -- the NewtonRaphsonSolver call sequence --------------------------------
    def begin_step(self, dt):
        self._check(self.L.tf_begin_step(self.h, dt), "tf_begin_step")

    def assemble(self):
        self._check(self.L.tf_assemble(self.h), "tf_assemble")

    def add_external_forces(self, gext):
        g = np.ascontiguousarray(gext, dtype=np.float64)
        self._check(self.L.tf_add_external_forces(self.h, _ptr(g)), "tf_add_external_forces")

    def set_dof_bindings(self, slave_dofs, master_dofs):
        """Bound DOF couples (slave follows master), applied at every solve."""
        s = np.ascontiguousarray(slave_dofs, dtype=np.int32)
        m = np.ascontiguousarray(master_dofs, dtype=np.int32)
        self._bind = (s, m)
        self._check(self.L.tf_set_dof_bindings(self.h, s.size, _ptr(s), _ptr(m)), "tf_set_dof_bindings")

    def set_packing(self, enable=True, reference_merge=True):
        """Implicit packing between tissue surfaces: couples detected at every
        begin_step, their forces and Jacobian added at every assemble.
        reference_merge keeps the reference's merge, which leaves out the
        couples found from the last of its 16 node segments."""
        self._check(self.L.tf_set_packing(self.h, 1 if enable else 0, 1 if reference_merge else 0),
                    "tf_set_packing")

    def packing(self):
        """Couples of the last detection: dict with nodes (n, 2), w (n, 3),
        mbar (n,), threshold, detect."""
        n = C.c_int64(0)
        thr = C.c_double(0.0)
        det = C.c_double(0.0)
        self._check(self.L.tf_get_packing(self.h, C.byref(n), None, None, None, C.byref(thr), C.byref(det)),
                    "tf_get_packing")
        nodes = np.zeros((n.value, 2), dtype=np.int32)
        w = np.zeros((n.value, 3))
        mbar = np.zeros(n.value)
        self._check(self.L.tf_get_packing(self.h, C.byref(n), _ptr(nodes), _ptr(w), _ptr(mbar), C.byref(thr),
                                          C.byref(det)), "tf_get_packing")
        return {"nodes": nodes, "w": w, "mbar": mbar, "threshold": thr.value, "detect": det.value}

    def packing_masses(self):
        m = np.zeros(self.nn)
        self._check(self.L.tf_packing_masses(self.h, _ptr(m)), "tf_packing_masses")
        return m

    def add_uniform_growth(self, rates, angle_rad=0.0, init_time=-1e30, end_time=1e30, zmin=0.0, zmax=1.0):
        """Uniform growth function (type 1): rates (3,) in 1/s oriented by
        angle_rad in the xy plane."""
        r = np.ascontiguousarray(rates, dtype=np.float64).reshape(3)
        self._check(self.L.tf_add_uniform_growth(self.h, _ptr(r), angle_rad, init_time, end_time, zmin, zmax),
                    "tf_add_uniform_growth")

    def add_ring_growth(self, centre, inner_radius, outer_radius, rates, angle_rad=0.0, init_time=-1e30,
                        end_time=1e30, zmin=0.0, zmax=1.0):
        """Ring growth function (type 2): rates (3,) at the inner radius,
        falling linearly to 0 at the outer radius."""
        r = np.ascontiguousarray(rates, dtype=np.float64).reshape(3)
        self._check(self.L.tf_add_ring_growth(self.h, float(centre[0]), float(centre[1]), inner_radius,
                                              outer_radius, _ptr(r), angle_rad, init_time, end_time, zmin, zmax),
                    "tf_add_ring_growth")

    def add_grid_growth(self, rates, angles_deg=None, init_time=-1e30, end_time=1e30, zmin=0.0, zmax=1.0):
        """Grid-based growth function (growth type 3): rates (nx, ny, 3) in
        1/s at the grid points over the tissue's bounding box, angles_deg
        (nx, ny) their xy orientation; active for init_time <= t < end_time
        on prisms whose initial relative z is within [zmin, zmax]."""
        r = np.ascontiguousarray(rates, dtype=np.float64)
        if r.ndim != 3 or r.shape[2] != 3:
            raise ValueError("rates must have shape (nx, ny, 3)")
        a = None if angles_deg is None else np.ascontiguousarray(angles_deg, dtype=np.float64)
        if a is not None and a.shape != r.shape[:2]:
            raise ValueError("angles_deg must have shape (nx, ny)")
        self._check(self.L.tf_add_grid_growth(self.h, r.shape[0], r.shape[1], _ptr(r), _ptr(a) if a is not None
                                              else None, init_time, end_time, zmin, zmax), "tf_add_grid_growth")

    def clear_growth_functions(self):
        self._check(self.L.tf_clear_growth_functions(self.h), "tf_clear_growth_functions")

    def set_grid_growth_mode(self, interpolation=1, pinned_on_initial_mesh=False):
        """interpolation 0: nearest grid point, 1: bilinear (the default);
        pinned: positions of the initial mesh instead of each step's start."""
        self._check(self.L.tf_set_grid_growth_mode(self.h, int(interpolation), 1 if pinned_on_initial_mesh else 0),
                    "tf_set_grid_growth_mode")

    def repin_grid_growth(self):
        self._check(self.L.tf_repin_grid_growth(self.h), "tf_repin_grid_growth")

    def grid_growth_positions(self):
        """(relz (ne,), pinned (ne, 2), current (ne, 2)) bounding-box positions."""
        z = np.zeros(self.ne)
        p0 = np.zeros(2 * self.ne)
        p = np.zeros(2 * self.ne)
        self._check(self.L.tf_grid_growth_positions(self.h, _ptr(z), _ptr(p0), _ptr(p)), "tf_grid_growth_positions")
        return z, p0.reshape(2, -1).T.copy(), p.reshape(2, -1).T.copy()

    @property
    def time(self):
        t = C.c_double(0.0)
        self._check(self.L.tf_get_time(self.h, C.byref(t)), "tf_get_time")
        return t.value

    @time.setter
    def time(self, value):
        self._check(self.L.tf_set_time(self.h, float(value)), "tf_set_time")

    def add_K_triplets(self, rows, cols, vals):
        """K(rows[k], cols[k]) += vals[k] after assemble() (packing/myosin-type writers)."""
        r = np.ascontiguousarray(rows, dtype=np.int32)
        c = np.ascontiguousarray(cols, dtype=np.int32)
        v = np.ascontiguousarray(vals, dtype=np.float64)
        self._check(self.L.tf_add_K_triplets(self.h, r.size, _ptr(r), _ptr(c), _ptr(v)), "tf_add_K_triplets")

    def solve(self, allow_not_converged=False):
        it = C.c_int32(0)
        rr = C.c_double(0.0)
        allow = (TF_KRYLOV_NOT_CONVERGED,) if allow_not_converged else ()
        s = self._check(self.L.tf_solve(self.h, C.byref(it), C.byref(rr)), "tf_solve", allow)
        return {"status": s, "iters": it.value, "relres": rr.value}

    def update(self):
        conv = C.c_int32(0)
        dn = C.c_double(0.0)
        self._check(self.L.tf_update(self.h, C.byref(conv), C.byref(dn)), "tf_update")
        return bool(conv.value), dn.value

    def end_step(self):
        self._check(self.L.tf_end_step(self.h), "tf_end_step")

    def newton_step(self, dt, allow_not_converged=True):
        st = tf_step_stats()
        allow = (TF_NOT_CONVERGED,) if allow_not_converged else ()
        s = self._check(self.L.tf_newton_step(self.h, dt, C.byref(st)), "tf_newton_step", allow)
        n = st.newton_iters
        return {"status": s, "iters": n, "dunorm": np.array(st.dunorm[: min(n, 32)]),
                "krylov_total": st.krylov_iters_total, "krylov_max": st.krylov_iters_max,
                "converged": bool(st.converged), "relres": st.final_relres, "ms_assemble": st.ms_assemble,
                "ms_solve": st.ms_solve, "ms_total": st.ms_total, "device_iters": st.device_iters,
                "device_handback": st.device_handback}

    # -- inspection ---------------------------------------------------------
    def residual(self):
        g = np.zeros(3 * self.nn)
        self._check(self.L.tf_get_residual(self.h, _ptr(g)), "tf_get_residual")
        return g

    def delta_u(self):
        d = np.zeros(3 * self.nn)
        self._check(self.L.tf_get_delta_u(self.h, _ptr(d)), "tf_get_delta_u")
        return d

    def export_csr(self, drop=1e-13):
        n = C.c_int64(0)
        self._check(self.L.tf_export_csr(self.h, drop, None, None, None, C.byref(n)), "tf_export_csr")
        ia = np.zeros(3 * self.nn + 1, dtype=np.int32)
        ja = np.zeros(n.value, dtype=np.int32)
        a = np.zeros(n.value)
        self._check(self.L.tf_export_csr(self.h, drop, _ptr(ia), _ptr(ja), _ptr(a), C.byref(n)), "tf_export_csr")
        return ia, ja, a

    def element_eval(self, e0=0, count=None, want_k=True):
        count = self.ne - e0 if count is None else count
        Ke = np.zeros(324 * count) if want_k else None
        Kv = np.zeros(324 * count) if want_k else None
        fe = np.zeros(18 * count)
        fv = np.zeros(18 * count)
        self._check(self.L.tf_element_eval(self.h, e0, count, _ptr(Ke), _ptr(Kv), _ptr(fe), _ptr(fv)),
                    "tf_element_eval")
        r = {"fe": fe.reshape(count, 6, 3), "fv": fv.reshape(count, 6, 3)}
        if want_k:
            r["Ke"] = Ke.reshape(count, 18, 18)
            r["Kv"] = Kv.reshape(count, 18, 18)
        return r

    def sizes(self):
        a, b, c = C.c_int64(0), C.c_int64(0), C.c_int64(0)
        self._check(self.L.tf_get_sizes(self.h, C.byref(a), C.byref(b), C.byref(c)), "tf_get_sizes")
        return a.value, b.value, c.value

    def stream(self):
        return self.L.tf_get_stream(self.h)

    def launch_count(self):
        return int(self.L.tf_launch_count(self.h))

    def time_assembly(self, iters):
        a, b = C.c_float(0), C.c_float(0)
        self._check(self.L.tf_time_assembly(self.h, iters, C.byref(a), C.byref(b)), "tf_time_assembly")
        return a.value, b.value

    def multigrid_info(self):
        """(nodes per level, smoother weights) of the multigrid hierarchy; empty
        lists when block-Jacobi is used."""
        lv = C.c_int32(0)
        nodes = np.zeros(10, dtype=np.int32)
        w = np.zeros(10)
        self._check(self.L.tf_multigrid_info(self.h, C.byref(lv), _ptr(nodes), _ptr(w)), "tf_multigrid_info")
        return nodes[: lv.value].tolist(), w[: lv.value].tolist()

    def tiles(self):
        """The autotuner's choices: prisms per CTA of the element kernel and
        the slots in flight per lane of the FP64 SpMV and of the level-0
        smoother (chosen at the first solve)."""
        su, mu = C.c_int32(0), C.c_int32(0)
        self._check(self.L.tf_solve_variants(self.h, C.byref(su), C.byref(mu)), "tf_solve_variants")
        return {"elements_per_cta": int(self.L.tf_elements_per_cta(self.h)), "spmv_unroll": su.value,
                "smoother_unroll": mu.value}

    def multigrid_blocks(self):
        """(matrix blocks, prolongator blocks) per level of the hierarchy."""
        nodes, _ = self.multigrid_info()
        b = np.zeros(10, dtype=np.int64)
        p = np.zeros(10, dtype=np.int64)
        self._check(self.L.tf_multigrid_blocks(self.h, _ptr(b), _ptr(p)), "tf_multigrid_blocks")
        return b[: len(nodes)].tolist(), p[: len(nodes)].tolist()

    # -- adjoint --------------------------------------------------------------
    def adjoint_forward(self, rate, logE, n_steps, dt, every, loss_params):
        """Run ``n_steps`` steps from the current positions with Fg = I, growth
        rates (r_e, r_e, 0) and E_e = exp(logE_e); returns (loss, saved)."""
        r = np.ascontiguousarray(rate, dtype=np.float64)
        e = np.ascontiguousarray(logE, dtype=np.float64)
        lp = np.ascontiguousarray(loss_params, dtype=np.float64)
        if r.shape != (self.ne,) or e.shape != (self.ne,) or lp.shape != (4,):
            raise ValueError("rate and logE need one value per element, loss_params four values")
        loss = C.c_double(0.0)
        saved = C.c_void_p()
        self._check(self.L.tf_adj_forward(self.h, _ptr(r), _ptr(e), n_steps, dt, every, _ptr(lp), C.byref(loss),
                                          C.byref(saved)), "tf_adj_forward", (TF_NOT_CONVERGED,))
        return loss.value, AdjointState(self.L, saved)

    def adjoint_backward(self, saved, dloss=1.0):
        """Gradients (dL/d rate, dL/d logE) for the run held by ``saved``."""
        gr = np.zeros(self.ne)
        ge = np.zeros(self.ne)
        self._check(self.L.tf_adj_backward(self.h, saved.p, dloss, _ptr(gr), _ptr(ge)), "tf_adj_backward")
        return gr, ge


class AdjointState:
    """Saved states of one adjoint forward run (``tf_adjoint``)."""

    def __init__(self, L, p):
        self.L = L
        self.p = p

    def free(self):
        if self.p:
            self.L.tf_adj_free(self.p)
            self.p = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class Batch(Solver):
    """Many independent tissues in one handle (tf_batch_create)."""

    def __init__(self, tissues, newton_tol=1e-8, newton_max_iter=20, krylov_rtol=1e-8, krylov_max_iter=20000,
                 krylov_method=0, deterministic=False, device=0, autotune=True, precond=0, update_atol=0.0,
                 host_loops=False, multigrid_reuse_steps=0):
        self.L = load()
        self.tissues = list(tissues)
        n = len(self.tissues)
        keep, meshes, mats = [], (tf_mesh * n)(), (tf_material * n)()
        for i, t in enumerate(self.tissues):
            a, m, mat = _mesh_structs(t)
            keep.append(a)
            meshes[i] = m
            mats[i] = mat
        self._arrays = keep
        opt = tf_options(newton_tol, newton_max_iter, krylov_rtol, krylov_max_iter, krylov_method,
                         1 if deterministic else 0, device, 0 if autotune else 1, precond, update_atol,
                         1 if host_loops else 0, multigrid_reuse_steps)
        h = C.c_void_p()
        self._check(self.L.tf_batch_create(meshes, mats, n, C.byref(opt), C.byref(h)), "tf_batch_create")
        self.h = h
        cnt = C.c_int32(0)
        self.node_off = np.zeros(n + 1, dtype=np.int32)
        self.elem_off = np.zeros(n + 1, dtype=np.int32)
        self._check(self.L.tf_get_instances(self.h, C.byref(cnt), _ptr(self.node_off), _ptr(self.elem_off)),
                    "tf_get_instances")
        self.n_instances = cnt.value
        self.nn, self.ne = int(self.node_off[-1]), int(self.elem_off[-1])

    def set_growth_rates(self, rates=None):
        if rates is None:
            rates = np.concatenate([t.rates for t in self.tissues])
        super().set_growth_rates(rates)

    def step(self, dt, allow_not_converged=True):
        n = self.n_instances
        iters = np.zeros(n, dtype=np.int32)
        conv = np.zeros(n, dtype=np.int32)
        st = tf_step_stats()
        allow = (TF_NOT_CONVERGED,) if allow_not_converged else ()
        s = self._check(self.L.tf_batch_step(self.h, dt, _ptr(iters), _ptr(conv), C.byref(st)), "tf_batch_step", allow)
        return {"status": s, "iters": iters, "converged": conv.astype(bool), "krylov_total": st.krylov_iters_total,
                "ms_total": st.ms_total, "ms_assemble": st.ms_assemble, "newton_rounds": st.newton_iters,
                "device_iters": st.device_iters, "device_handback": st.device_handback}

    def instance_positions(self, i):
        p = self.positions()
        return p[3 * self.node_off[i]:3 * self.node_off[i + 1]]

    def elements_per_cta(self):
        return int(self.L.tf_elements_per_cta(self.h))


def _raise(L, s, where):
    if s != TF_OK:
        raise TfError(s, where, L.tf_last_error().decode())


def read_mesh_file(path):
    """The reference's .mesh input file: dict with pos (3N), conn (6E, after the
    reference's orientation check), placement, tissue_type, at_circumference
    (N) and ref_pos (18E)."""
    L = load()
    nn, ne = C.c_int32(0), C.c_int32(0)
    b = os.fsencode(path)
    _raise(L, L.tf_read_mesh_file(b, C.byref(nn), C.byref(ne), None, None, None, None, None, None),
           "tf_read_mesh_file")
    n, e = nn.value, ne.value
    out = {"pos": np.zeros(3 * n), "conn": np.zeros(6 * e, dtype=np.int32), "placement": np.zeros(n, dtype=np.int32),
           "tissue_type": np.zeros(n, dtype=np.int32), "at_circumference": np.zeros(n, dtype=np.int32),
           "ref_pos": np.zeros(18 * e)}
    _raise(L, L.tf_read_mesh_file(b, C.byref(nn), C.byref(ne), _ptr(out["pos"]), _ptr(out["conn"]),
                                  _ptr(out["placement"]), _ptr(out["tissue_type"]), _ptr(out["at_circumference"]),
                                  _ptr(out["ref_pos"])), "tf_read_mesh_file")
    return out


def write_frame(path, time_sec, pos, conn, placement, tissue_type=None, at_circumference=None, ref_pos=None,
                append=True):
    """Append one save frame in the reference's format (its viewer's input)."""
    L = load()
    p = np.ascontiguousarray(pos, dtype=np.float64)
    c = np.ascontiguousarray(conn, dtype=np.int32)
    n, e = p.size // 3, c.size // 6
    pl = np.ascontiguousarray(placement, dtype=np.int32)
    ty = np.zeros(n, dtype=np.int32) if tissue_type is None else np.ascontiguousarray(tissue_type, dtype=np.int32)
    ci = np.zeros(n, dtype=np.int32) if at_circumference is None else np.ascontiguousarray(at_circumference,
                                                                                         dtype=np.int32)
    rp = (p.reshape(-1, 3)[c.reshape(-1, 6)].reshape(-1) if ref_pos is None
          else np.ascontiguousarray(ref_pos, dtype=np.float64))
    _raise(L, L.tf_write_frame(os.fsencode(path), 1 if append else 0, float(time_sec), n, _ptr(p), _ptr(pl),
                               _ptr(ty), _ptr(ci), e, _ptr(c), _ptr(rp)), "tf_write_frame")

