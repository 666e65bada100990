"""ctypes bindings for the CPU oracle.  TEST INFRASTRUCTURE ONLY.

Two oracles live here:

* ``Port`` wraps ``_build/libtforacle.so``: the plain-C restatement of the
  reference's implicit prism step (``tf_oracle.c``).  It builds on any host
  with gcc and is what the GPU parity tests, ``smoke()`` and the CPU baseline
  of ``bench.py`` use.
* ``Ref`` wraps ``_ref/libtfref.so``: the reference's own sources compiled with
  project-written GSL / uBLAS / Pardiso stand-ins (``ref/Makefile``).  It only
  builds where the reference checkout is present and pins ``Port`` (and the
  golden fixtures under ``tests/golden``).

Only tests, ``__graft_entry__.smoke`` and the CPU-baseline leg of ``bench.py``
may import this module.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_LIB = os.path.join(HERE, "_build", "libtforacle.so")
REF_LIB = os.path.join(HERE, "_ref", "libtfref.so")
# root of the reference checkout (read only); TF_REFERENCE_DIR overrides it
REF_ROOT = os.environ.get("TF_REFERENCE_DIR", "/root/reference")
REF_SRC = os.path.join(REF_ROOT, "TissueFolding", "TissueFolding", "SourceCode")

LITERAL = 0
CLOSED = 1

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_u8 = np.ctypeslib.ndpointer(dtype=np.uint8, flags="C_CONTIGUOUS")


def build_port() -> str:
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return PORT_LIB


def build_ref() -> str | None:
    if not os.path.isdir(REF_SRC):
        return None
    subprocess.run(["make", "-s", "-j8", "-C", os.path.join(HERE, "ref"), f"REF={REF_SRC}"], check=True)
    return REF_LIB


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def _nullable(arr):
    return arr.ctypes.data_as(C.c_void_p) if arr is not None else None


class Port:
    """The C restatement (``tf_oracle.c``)."""

    _lib = None

    @classmethod
    def lib(cls):
        if cls._lib is None:
            if not os.path.exists(PORT_LIB):
                build_port()
            L = C.CDLL(PORT_LIB)
            L.tfo_create.restype = C.c_void_p
            L.tfo_create.argtypes = [C.c_int, C.c_int, _dp, _ip, _u8, _dp, _ip, _dp, _dp, _dp]
            L.tfo_destroy.argtypes = [C.c_void_p]
            L.tfo_set_threads.argtypes = [C.c_int]
            L.tfo_get_threads.restype = C.c_int
            L.tfo_set_Fg.argtypes = [C.c_void_p, _dp]
            L.tfo_get_Fg.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
            L.tfo_set_positions.argtypes = [C.c_void_p, _dp]
            L.tfo_get_positions.argtypes = [C.c_void_p, _dp]
            L.tfo_get_lame.argtypes = [C.c_void_p, _dp, _dp]
            L.tfo_get_placement.argtypes = [C.c_void_p, _ip]
            L.tfo_get_ref_geometry.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
            L.tfo_grow.argtypes = [C.c_void_p, C.c_double, _dp]
            L.tfo_update_viscosity_surfaces.argtypes = [C.c_void_p, C.c_void_p]
            L.tfo_set_viscosity_surfaces.argtypes = [C.c_void_p, _dp]
            L.tfo_element_eval.argtypes = [C.c_void_p, _dp, _dp, C.c_double, C.c_int, C.c_int, C.c_int,
                                           C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
            L.tfo_assemble.restype = C.c_long
            L.tfo_assemble.argtypes = [C.c_void_p, _dp, _dp, C.c_double, C.c_int]
            L.tfo_assemble_sample.restype = C.c_long
            L.tfo_assemble_sample.argtypes = [C.c_void_p, _dp, _dp, C.c_double, C.c_int, C.c_int]
            L.tfo_structure_nnz.restype = C.c_long
            L.tfo_structure_nnz.argtypes = [C.c_void_p]
            L.tfo_get_structure.argtypes = [C.c_void_p, _ip, _ip]
            L.tfo_get_values.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
            L.tfo_export_filtered.restype = C.c_long
            L.tfo_export_filtered.argtypes = [C.c_void_p, C.c_double, C.c_void_p, C.c_void_p, C.c_void_p]
            L.tfo_residual.argtypes = [C.c_void_p, _dp, _dp, C.c_double, _dp]
            L.tfo_solve.restype = C.c_int
            L.tfo_solve.argtypes = [C.c_void_p, _dp]
            L.tfo_step.restype = C.c_int
            L.tfo_step.argtypes = [C.c_void_p, C.c_double, C.c_void_p, C.c_int, C.POINTER(C.c_int), _dp, C.c_int]
            L.tfo_set_reference_shapes.restype = None
            L.tfo_set_reference_shapes.argtypes = [C.c_void_p, _dp]
            cls._lib = L
        return cls._lib

    def __init__(self, t):
        L = self.lib()
        self.t = t
        self.nn, self.ne = t.n_nodes, t.n_elems
        self._keep = [_f64(t.pos), _i32(t.conn), np.ascontiguousarray(t.fixed, dtype=np.uint8),
                      _f64(t.ext_visc), _i32(t.node_placement), _f64(t.E), _f64(t.nu), _f64(t.eta)]
        self.h = L.tfo_create(self.nn, self.ne, *self._keep)
        if getattr(t, "ref_pos", None) is not None:
            self._ref = _f64(t.ref_pos)
            L.tfo_set_reference_shapes(self.h, self._ref)

    def close(self):
        if self.h:
            self.lib().tfo_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @staticmethod
    def set_threads(n: int):
        Port.lib().tfo_set_threads(n)

    @staticmethod
    def threads() -> int:
        return Port.lib().tfo_get_threads()

    def set_Fg(self, Fg):
        self.lib().tfo_set_Fg(self.h, _f64(Fg))

    def get_Fg(self):
        Fg = np.zeros(9 * self.ne)
        inv = np.zeros(9 * self.ne)
        self.lib().tfo_get_Fg(self.h, Fg.ctypes.data_as(C.c_void_p), inv.ctypes.data_as(C.c_void_p))
        return Fg, inv

    def set_positions(self, pos):
        self.lib().tfo_set_positions(self.h, _f64(pos))

    def positions(self):
        p = np.zeros(3 * self.nn)
        self.lib().tfo_get_positions(self.h, p)
        return p

    def lame(self):
        lam, mu = np.zeros(self.ne), np.zeros(self.ne)
        self.lib().tfo_get_lame(self.h, lam, mu)
        return lam, mu

    def placement(self):
        p = np.zeros(self.ne, dtype=np.int32)
        self.lib().tfo_get_placement(self.h, p)
        return p

    def ref_geometry(self):
        det = np.zeros(6 * self.ne)
        inv = np.zeros(54 * self.ne)
        self.lib().tfo_get_ref_geometry(self.h, det.ctypes.data_as(C.c_void_p), inv.ctypes.data_as(C.c_void_p))
        return det, inv

    def grow(self, dt, rates):
        self.lib().tfo_grow(self.h, dt, _f64(rates))

    def update_viscosity_surfaces(self):
        a = np.zeros(self.nn)
        self.lib().tfo_update_viscosity_surfaces(self.h, a.ctypes.data_as(C.c_void_p))
        return a

    def set_viscosity_surfaces(self, area):
        self.lib().tfo_set_viscosity_surfaces(self.h, _f64(area))

    def element_eval(self, uk, un, dt, mode=LITERAL, e0=0, count=None, want_k=True):
        count = self.ne - e0 if count is None else count
        Ke = np.zeros(324 * count) if want_k else None
        Kv = np.zeros(324 * count) if want_k else None
        fe = np.zeros(18 * count)
        fv = np.zeros(18 * count)
        self.lib().tfo_element_eval(self.h, _f64(uk), _f64(un), dt, mode, e0, count,
                                    _nullable(Ke), _nullable(Kv), _nullable(fe), _nullable(fv))
        r = {"fe": fe.reshape(count, 6, 3), "fv": fv.reshape(count, 6, 3)}
        if want_k:
            r["Ke"] = Ke.reshape(count, 18, 18)
            r["Kv"] = Kv.reshape(count, 18, 18)
        return r

    def assemble(self, uk, un, dt, mode=CLOSED):
        return self.lib().tfo_assemble(self.h, _f64(uk), _f64(un), dt, mode)

    def assemble_sample(self, uk, un, dt, count, mode=LITERAL):
        return self.lib().tfo_assemble_sample(self.h, _f64(uk), _f64(un), dt, mode, int(count))

    def structure(self):
        nnz = self.lib().tfo_structure_nnz(self.h)
        ia = np.zeros(3 * self.nn + 1, dtype=np.int32)
        ja = np.zeros(nnz, dtype=np.int32)
        self.lib().tfo_get_structure(self.h, ia, ja)
        return ia, ja

    def values(self):
        nnz = self.lib().tfo_structure_nnz(self.h)
        a = np.zeros(nnz)
        g = np.zeros(3 * self.nn)
        self.lib().tfo_get_values(self.h, a.ctypes.data_as(C.c_void_p), g.ctypes.data_as(C.c_void_p))
        return a, g

    def rhs(self):
        """gSum of the last assembly with fixed DOFs zeroed (no matrix copy)."""
        g = np.zeros(3 * self.nn)
        self.lib().tfo_get_values(self.h, None, g.ctypes.data_as(C.c_void_p))
        return g

    def export_filtered(self, drop=1e-13):
        L = self.lib()
        n = L.tfo_export_filtered(self.h, drop, None, None, None)
        ia = np.zeros(3 * self.nn + 1, dtype=np.int32)
        ja = np.zeros(n, dtype=np.int32)
        a = np.zeros(n)
        L.tfo_export_filtered(self.h, drop, ia.ctypes.data_as(C.c_void_p), ja.ctypes.data_as(C.c_void_p),
                              a.ctypes.data_as(C.c_void_p))
        return ia, ja, a

    def residual(self, uk, un, dt):
        g = np.zeros(3 * self.nn)
        self.lib().tfo_residual(self.h, _f64(uk), _f64(un), dt, g)
        return g

    def solve(self):
        du = np.zeros(3 * self.nn)
        rc = self.lib().tfo_solve(self.h, du)
        if rc != 0:
            raise RuntimeError(f"oracle solve failed ({rc})")
        return du

    def step(self, dt, rates=None, mode=CLOSED):
        it = C.c_int(0)
        hist = np.zeros(64)
        r = _f64(rates) if rates is not None else None
        rc = self.lib().tfo_step(self.h, dt, _nullable(r), mode, C.byref(it), hist, 64)
        if rc < 0:
            raise RuntimeError("oracle step failed")
        return {"iters": it.value, "dunorm": hist[: min(it.value, 64)].copy(), "capped": bool(rc == 1)}


class Ref:
    """The reference's own sources (``oracle/_ref/libtfref.so``)."""

    _lib = None

    @classmethod
    def available(cls) -> bool:
        return os.path.exists(REF_LIB) or os.path.isdir(REF_SRC)

    @classmethod
    def lib(cls):
        if cls._lib is None:
            # the reference exits when OMP_NUM_THREADS is unset
            # (NewtonRaphsonSolver.cpp:502-507)
            os.environ.setdefault("OMP_NUM_THREADS", str(os.cpu_count() or 1))
            if not os.path.exists(REF_LIB):
                if build_ref() is None:
                    raise RuntimeError("the reference checkout is not present; oracle/_ref cannot be built")
            L = C.CDLL(REF_LIB)
            L.tfr_create.restype = C.c_void_p
            L.tfr_create.argtypes = [C.c_int, C.c_int, _dp, _ip, _u8, _dp, _ip, _dp, _dp, _dp]
            L.tfr_destroy.argtypes = [C.c_void_p]
            L.tfr_get_conn.argtypes = [C.c_void_p, _ip]
            L.tfr_get_lame.argtypes = [C.c_void_p, _dp, _dp]
            L.tfr_get_placement.argtypes = [C.c_void_p, _ip]
            L.tfr_set_Fg.argtypes = [C.c_void_p, _dp]
            L.tfr_get_Fg.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
            L.tfr_set_positions.argtypes = [C.c_void_p, _dp]
            L.tfr_get_positions.argtypes = [C.c_void_p, _dp]
            L.tfr_grow.argtypes = [C.c_void_p, C.c_double, _dp]
            L.tfr_update_viscosity_surfaces.argtypes = [C.c_void_p, C.c_void_p]
            L.tfr_element_eval.argtypes = [C.c_void_p, _dp, _dp, C.c_double, C.c_void_p, C.c_void_p,
                                           C.c_void_p, C.c_void_p]
            L.tfr_assemble.restype = C.c_long
            L.tfr_assemble.argtypes = [C.c_void_p, _dp, _dp, C.c_double]
            L.tfr_get_system.argtypes = [C.c_void_p, _ip, _ip, _dp, _dp]
            L.tfr_step.restype = C.c_int
            L.tfr_step.argtypes = [C.c_void_p, C.c_double, C.c_void_p, C.POINTER(C.c_int), _dp, C.c_int]
            L.tfr_set_bindings.restype = None
            L.tfr_set_bindings.argtypes = [C.c_void_p, C.c_int, _ip, _ip]
            L.tfr_set_packing.argtypes = [C.c_void_p, C.c_int, C.c_int]
            L.tfr_pack_detect.argtypes = [C.c_void_p]
            L.tfr_pack_count.restype = C.c_long
            L.tfr_pack_count.argtypes = [C.c_void_p]
            L.tfr_pack_get.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
            L.tfr_node_masses.argtypes = [C.c_void_p, _dp]
            L.tfr_pack_forces.argtypes = [C.c_void_p, _dp]
            L.tfr_add_grid_growth.argtypes = [C.c_void_p, C.c_int, C.c_int, _dp, C.c_void_p, C.c_double,
                                              C.c_double, C.c_double, C.c_double]
            L.tfr_add_uniform_growth.argtypes = [C.c_void_p, _dp, C.c_double, C.c_double, C.c_double, C.c_double,
                                                 C.c_double]
            L.tfr_add_ring_growth.argtypes = [C.c_void_p, C.c_double, C.c_double, C.c_double, C.c_double, _dp,
                                              C.c_double, C.c_double, C.c_double, C.c_double, C.c_double]
            L.tfr_clear_growth_functions.argtypes = [C.c_void_p]
            L.tfr_set_grid_mode.argtypes = [C.c_void_p, C.c_int, C.c_int]
            L.tfr_repin_grid_growth.argtypes = [C.c_void_p]
            L.tfr_set_time.argtypes = [C.c_void_p, C.c_double]
            L.tfr_get_time.restype = C.c_double
            L.tfr_get_time.argtypes = [C.c_void_p]
            L.tfr_grid_positions.argtypes = [C.c_void_p, _dp, _dp, _dp]
            cls._lib = L
        return cls._lib

    def __init__(self, t):
        L = self.lib()
        self.t = t
        self.nn, self.ne = t.n_nodes, t.n_elems
        self._keep = [_f64(t.pos), _i32(t.conn), np.ascontiguousarray(t.fixed, dtype=np.uint8),
                      _f64(t.ext_visc), _i32(t.node_placement), _f64(t.E), _f64(t.nu), _f64(t.eta)]
        self.h = L.tfr_create(self.nn, self.ne, *self._keep)

    def close(self):
        if self.h:
            self.lib().tfr_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def conn(self):
        c = np.zeros(6 * self.ne, dtype=np.int32)
        self.lib().tfr_get_conn(self.h, c)
        return c

    def lame(self):
        lam, mu = np.zeros(self.ne), np.zeros(self.ne)
        self.lib().tfr_get_lame(self.h, lam, mu)
        return lam, mu

    def placement(self):
        p = np.zeros(self.ne, dtype=np.int32)
        self.lib().tfr_get_placement(self.h, p)
        return p

    def set_Fg(self, Fg):
        self.lib().tfr_set_Fg(self.h, _f64(Fg))

    def get_Fg(self):
        Fg = np.zeros(9 * self.ne)
        inv = np.zeros(9 * self.ne)
        self.lib().tfr_get_Fg(self.h, Fg.ctypes.data_as(C.c_void_p), inv.ctypes.data_as(C.c_void_p))
        return Fg, inv

    def set_positions(self, pos):
        self.lib().tfr_set_positions(self.h, _f64(pos))

    def positions(self):
        p = np.zeros(3 * self.nn)
        self.lib().tfr_get_positions(self.h, p)
        return p

    def grow(self, dt, rates):
        self.lib().tfr_grow(self.h, dt, _f64(rates))

    def update_viscosity_surfaces(self):
        a = np.zeros(self.nn)
        self.lib().tfr_update_viscosity_surfaces(self.h, a.ctypes.data_as(C.c_void_p))
        return a

    def element_eval(self, uk, un, dt):
        Ke = np.zeros(324 * self.ne)
        Kv = np.zeros(324 * self.ne)
        fe = np.zeros(18 * self.ne)
        fv = np.zeros(18 * self.ne)
        self.lib().tfr_element_eval(self.h, _f64(uk), _f64(un), dt, Ke.ctypes.data_as(C.c_void_p),
                                    Kv.ctypes.data_as(C.c_void_p), fe.ctypes.data_as(C.c_void_p),
                                    fv.ctypes.data_as(C.c_void_p))
        n = self.ne
        return {"Ke": Ke.reshape(n, 18, 18), "Kv": Kv.reshape(n, 18, 18),
                "fe": fe.reshape(n, 6, 3), "fv": fv.reshape(n, 6, 3)}

    def assemble(self, uk, un, dt):
        n = self.lib().tfr_assemble(self.h, _f64(uk), _f64(un), dt)
        ia = np.zeros(3 * self.nn + 1, dtype=np.int32)
        ja = np.zeros(n, dtype=np.int32)
        a = np.zeros(n)
        g = np.zeros(3 * self.nn)
        self.lib().tfr_get_system(self.h, ia, ja, a, g)
        return ia, ja, a, g

    def set_bindings(self, slave_dofs, master_dofs):
        s = _i32(slave_dofs)
        m = _i32(master_dofs)
        self._bind = (s, m)
        self.lib().tfr_set_bindings(self.h, int(s.size), s, m)

    def set_packing(self, on=True, drop_last_segment=True):
        """Implicit packing between tissue surfaces in every later step and
        assembly (Simulation::detectPacingNodes and the packing force and
        Jacobian writers)."""
        self.lib().tfr_set_packing(self.h, int(bool(on)), int(bool(drop_last_segment)))

    def pack_detect(self):
        """The start-of-step packing work at the current positions: bounding
        box, node masses, couple detection."""
        self.lib().tfr_pack_detect(self.h)

    def packing(self):
        """Couples of the last detection: dict with `nodes` (n, 2), `w`
        (n, 3), `mbar` (n,), `threshold`, `detect`."""
        L = self.lib()
        n = int(L.tfr_pack_count(self.h))
        nodes = np.zeros((n, 2), dtype=np.int32)
        w = np.zeros((n, 3))
        mbar = np.zeros(n)
        thr = C.c_double(0.0)
        det = C.c_double(0.0)
        L.tfr_pack_get(self.h, nodes.ctypes.data_as(C.c_void_p), w.ctypes.data_as(C.c_void_p),
                       mbar.ctypes.data_as(C.c_void_p), C.byref(thr), C.byref(det))
        return {"nodes": nodes, "w": w, "mbar": mbar, "threshold": thr.value, "detect": det.value}

    def node_masses(self):
        m = np.zeros(self.nn)
        self.lib().tfr_node_masses(self.h, m)
        return m

    def pack_forces(self):
        f = np.zeros(3 * self.nn)
        self.lib().tfr_pack_forces(self.h, f)
        return f

    def add_grid_growth(self, rates, angles_deg=None, init_time=-1e30, end_time=1e30, zmin=0.0, zmax=1.0):
        """The reference's GridBasedGrowthFunction: rates (nx, ny, 3) in 1/s,
        angles_deg (nx, ny)."""
        r = _f64(rates)
        a = None if angles_deg is None else _f64(angles_deg)
        self._grid_keep = getattr(self, "_grid_keep", []) + [r, a]
        self.lib().tfr_add_grid_growth(self.h, r.shape[0], r.shape[1], r.reshape(-1),
                                       None if a is None else a.ctypes.data_as(C.c_void_p),
                                       init_time, end_time, zmin, zmax)

    def add_uniform_growth(self, rates, angle_rad=0.0, init_time=-1e30, end_time=1e30, zmin=0.0, zmax=1.0):
        self.lib().tfr_add_uniform_growth(self.h, _f64(rates).reshape(3), angle_rad, init_time, end_time, zmin,
                                          zmax)

    def add_ring_growth(self, centre, inner_radius, outer_radius, rates, angle_rad=0.0, init_time=-1e30,
                        end_time=1e30, zmin=0.0, zmax=1.0):
        self.lib().tfr_add_ring_growth(self.h, float(centre[0]), float(centre[1]), inner_radius, outer_radius,
                                       _f64(rates).reshape(3), angle_rad, init_time, end_time, zmin, zmax)

    def clear_growth_functions(self):
        self.lib().tfr_clear_growth_functions(self.h)

    def set_grid_mode(self, interpolation=1, pinned=False):
        self.lib().tfr_set_grid_mode(self.h, int(interpolation), 1 if pinned else 0)

    def repin_grid_growth(self):
        self.lib().tfr_repin_grid_growth(self.h)

    @property
    def time(self):
        return self.lib().tfr_get_time(self.h)

    @time.setter
    def time(self, value):
        self.lib().tfr_set_time(self.h, float(value))

    def grid_positions(self):
        """(relz (ne,), pinned (ne, 2), current (ne, 2))."""
        z = np.zeros(self.ne)
        p0 = np.zeros(2 * self.ne)
        p = np.zeros(2 * self.ne)
        self.lib().tfr_grid_positions(self.h, z, p0, p)
        return z, p0.reshape(2, -1).T.copy(), p.reshape(2, -1).T.copy()

    def step(self, dt, rates=None):
        it = C.c_int(0)
        hist = np.zeros(64)
        r = _f64(rates) if rates is not None else None
        rc = self.lib().tfr_step(self.h, dt, _nullable(r), C.byref(it), hist, 64)
        return {"iters": it.value, "dunorm": hist[: min(it.value, 64)].copy(), "capped": bool(rc == 1)}
