"""ctypes loader of the CPU oracle liborc.so (test infrastructure only).

liborc.so is the plain-C restatement of the reference's DGSEM residual,
Riemann solvers, time step and Runge-Kutta steppers (see orc.h for the
reference file:line of every routine).  It is the checker of the GPU library
and the timed CPU baseline, never the thing measured as the product.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "liborc.so"

EXACT, HLLC, AUSM, ROE, RUSANOV = range(5)
BC_NONE, BC_INVISCID_WALL, BC_SUPERSONIC_INLET, BC_SUPERSONIC_OUTLET, BC_SUBSONIC_INLET, \
    BC_SUBSONIC_OUTLET, BC_SMART, BC_NO_SLIP_WALL = range(8)
STATE_CONSTANT, STATE_MOVING_SPLIT, STATE_OBLIQUE_SPLIT, STATE_TABLE = 0, 1, 2, 3

_D = C.POINTER(C.c_double)


class OrcBc(C.Structure):
    _fields_ = [("kind", C.c_int), ("program", C.c_int), ("axis", C.c_int),
                ("position", C.c_double), ("speed", C.c_double),
                ("a", C.c_double * 5), ("b", C.c_double * 5),
                ("normal", C.c_double * 3), ("table", _D)]


def build(force: bool = False) -> Path:
    """make -C oracle (portable flags; rebuilt on each host)."""
    srcs = list(HERE.glob("*.c")) + list(HERE.glob("*.h")) + [HERE / "Makefile"]
    if force or not LIB.exists() or any(p.stat().st_mtime > LIB.stat().st_mtime for p in srcs):
        subprocess.run(["make", "-s", "-B" if force else "-s", "-C", str(HERE)], check=True)
    return LIB


_lib = None


def load() -> C.CDLL:
    global _lib
    if _lib is None:
        build()
        lib = C.CDLL(str(LIB))
        sig = {
            "orc_cons_to_prim": (None, [_D, _D]),
            "orc_prim_to_cons": (None, [_D, _D]),
            "orc_flux_matrix": (None, [_D, _D]),
            "orc_max_speed": (C.c_double, [_D]),
            "orc_flux_1d": (None, [C.c_int, _D, _D, _D]),
            "orc_flux_rotated": (None, [C.c_int, _D, _D, _D, _D]),
            "orc_flux_boundary": (None, [C.c_int, C.c_int, _D, _D, _D, _D]),
            "orc_mesh_create": (C.c_void_p, [C.c_int64, _D, C.c_int64, C.POINTER(C.c_int64),
                                             C.POINTER(C.c_int32), C.c_int32, C.c_int64,
                                             C.POINTER(C.c_int64), C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                                             _D, C.c_int]),
            "orc_mesh_destroy": (None, [C.c_void_p]),
            "orc_column_size": (C.c_int64, [C.c_void_p]),
            "orc_nodes_per_cell": (C.c_int, [C.c_void_p]),
            "orc_face_node_maps": (C.c_int, [C.c_void_p, C.POINTER(C.c_int16), C.POINTER(C.c_int16)]),
            "orc_node_geometry": (C.c_int, [C.c_void_p, _D, _D]),
            "orc_face_geometry": (C.c_int, [C.c_void_p, _D, _D, _D]),
            "orc_cell_length": (C.c_double, [C.c_void_p, C.c_int64]),
            "orc_set_threads": (None, [C.c_int]),
            "orc_get_threads": (C.c_int, []),
            "orc_dgsem_residual": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.POINTER(OrcBc), C.c_double, _D, _D]),
            "orc_time_step": (C.c_double, [C.c_void_p, _D, C.c_double, C.c_int, C.c_double]),
            "orc_rk_update": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.POINTER(OrcBc), C.c_int, C.c_double,
                                        C.c_double, _D]),
            "orc_rk_update_linear": (C.c_int, [C.c_int, C.c_int64, _D, C.c_double, C.c_double, _D]),
            "orc_mesh_set_scheme": (None, [C.c_void_p, C.c_int]),
            "orc_vtk_sample": (C.c_int, [C.c_void_p, _D, _D, _D]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


def _p(a: np.ndarray):
    return a.ctypes.data_as(_D)


def cons_to_prim(u) -> np.ndarray:
    u = np.ascontiguousarray(u, dtype=np.float64)
    out = np.empty(5)
    load().orc_cons_to_prim(_p(u), _p(out))
    return out


def prim_to_cons(w) -> np.ndarray:
    w = np.ascontiguousarray(w, dtype=np.float64)
    out = np.empty(5)
    load().orc_prim_to_cons(_p(w), _p(out))
    return out


def flux_matrix(u) -> np.ndarray:
    u = np.ascontiguousarray(u, dtype=np.float64)
    out = np.empty(15)
    load().orc_flux_matrix(_p(u), _p(out))
    return out.reshape(5, 3)


def max_speed(u) -> float:
    u = np.ascontiguousarray(u, dtype=np.float64)
    return float(load().orc_max_speed(_p(u)))


def flux_1d(kind: int, prim_l, prim_r) -> np.ndarray:
    """Normal-frame flux from primitive (rho, u, v, w, p) states."""
    l = np.ascontiguousarray(prim_l, dtype=np.float64)
    r = np.ascontiguousarray(prim_r, dtype=np.float64)
    out = np.empty(5)
    load().orc_flux_1d(kind, _p(l), _p(r), _p(out))
    return out


def flux_rotated(kind: int, frame, cons_l, cons_r) -> np.ndarray:
    f = np.ascontiguousarray(frame, dtype=np.float64).reshape(9)
    l = np.ascontiguousarray(cons_l, dtype=np.float64)
    r = np.ascontiguousarray(cons_r, dtype=np.float64)
    out = np.empty(5)
    load().orc_flux_rotated(kind, _p(f), _p(l), _p(r), _p(out))
    return out


def flux_boundary(riemann: int, bc_kind: int, frame, cons_in, given) -> np.ndarray:
    f = np.ascontiguousarray(frame, dtype=np.float64).reshape(9)
    u = np.ascontiguousarray(cons_in, dtype=np.float64)
    g = np.ascontiguousarray(given, dtype=np.float64)
    out = np.empty(5)
    load().orc_flux_boundary(riemann, bc_kind, _p(f), _p(u), _p(g), _p(out))
    return out


def make_bcs(specs: dict[int, tuple], face_points=None) -> tuple[int, C.Array]:
    """specs: group -> (kind, value) with value None, a 5-vector, an object
    with axis/position/speed/a/b (moving split), one with
    normal/position/speed/a/b (oblique split), or a callable of the points
    [n, 3] -> states [n, 5] (sampled at face_points, every face point of the
    mesh by global index, into a table)."""
    n = max(specs) + 1 if specs else 1
    arr = (OrcBc * n)()
    keep = []
    for g, (kind, value) in specs.items():
        b = arr[g]
        b.kind = kind
        if value is None:
            b.program = STATE_CONSTANT
        elif callable(value):
            table = np.ascontiguousarray(value(np.asarray(face_points).reshape(-1, 3)), dtype=np.float64)
            keep.append(table)
            b.program = STATE_TABLE
            b.table = table.ctypes.data_as(_D)
        elif hasattr(value, "normal"):
            b.program = STATE_OBLIQUE_SPLIT
            b.position, b.speed = float(value.position), float(value.speed)
            for k in range(3):
                b.normal[k] = float(value.normal[k])
            for k in range(5):
                b.a[k] = float(value.a[k])
                b.b[k] = float(value.b[k])
        elif hasattr(value, "axis"):
            b.program = STATE_MOVING_SPLIT
            b.axis, b.position, b.speed = int(value.axis), float(value.position), float(value.speed)
            for k in range(5):
                b.a[k] = float(value.a[k])
                b.b[k] = float(value.b[k])
        else:
            b.program = STATE_CONSTANT
            for k in range(5):
                b.a[k] = float(value[k])
    arr._keep = keep  # the tables live as long as the array
    return n, arr


class Mesh:
    """Oracle-side mesh + DGSEM system built from the same description."""

    def __init__(self, mesh, degree: int, scheme: str = "dgsem"):
        lib = load()
        self._keep = [np.ascontiguousarray(mesh.xyz, dtype=np.float64),
                      np.ascontiguousarray(mesh.cell_nodes, dtype=np.int64),
                      np.ascontiguousarray(mesh.face_cells, dtype=np.int64),
                      np.ascontiguousarray(mesh.face_sides, dtype=np.int32),
                      np.ascontiguousarray(mesh.face_group, dtype=np.int32),
                      np.ascontiguousarray(mesh.face_shift, dtype=np.float64)]
        xyz, cn, fc, fs, fg, fsh = self._keep
        self._ct = None if mesh.cell_type is None else np.ascontiguousarray(mesh.cell_type, dtype=np.int32)
        ct_p = None if self._ct is None else self._ct.ctypes.data_as(C.POINTER(C.c_int32))
        self._m = lib.orc_mesh_create(xyz.shape[0], _p(xyz), cn.shape[0], cn.ctypes.data_as(C.POINTER(C.c_int64)),
                                      ct_p, cn.shape[1], fc.shape[0], fc.ctypes.data_as(C.POINTER(C.c_int64)),
                                      fs.ctypes.data_as(C.POINTER(C.c_int32)),
                                      fg.ctypes.data_as(C.POINTER(C.c_int32)), _p(fsh), degree)
        if not self._m:
            raise RuntimeError("oracle rejected the mesh (unmatched face point or bad index)")
        self.lib = lib
        self.degree = degree
        self.n_faces = fc.shape[0]
        self.n_cells = cn.shape[0]
        self.column_size = int(lib.orc_column_size(self._m))
        self.bcs = make_bcs({})
        if scheme == "fr":
            lib.orc_mesh_set_scheme(self._m, 1)

    def __del__(self):
        if getattr(self, "_m", None):
            self.lib.orc_mesh_destroy(self._m)
            self._m = None

    def set_bcs(self, specs: dict[int, tuple]) -> None:
        pts = None
        if any(callable(v) for _, v in specs.values()):
            qf = (self.degree + 1) ** 2
            pts = np.empty((self.n_faces * qf, 3))
            self.lib.orc_face_geometry(self._m, _p(pts), None, None)
        self.bcs = make_bcs(specs, pts)

    def face_node_maps(self):
        qf = (self.degree + 1) ** 2
        h = np.empty((self.n_faces, qf), dtype=np.int16)
        s = np.empty((self.n_faces, qf), dtype=np.int16)
        self.lib.orc_face_node_maps(self._m, h.ctypes.data_as(C.POINTER(C.c_int16)),
                                    s.ctypes.data_as(C.POINTER(C.c_int16)))
        return h, s

    def node_geometry(self):
        n = (self.degree + 1) ** 3
        xyz = np.empty((self.n_cells, n, 3))
        w = np.empty((self.n_cells, n))
        self.lib.orc_node_geometry(self._m, _p(xyz), _p(w))
        return xyz, w

    def residual(self, riemann: int, u: np.ndarray, t: float = 0.0) -> np.ndarray:
        u = np.ascontiguousarray(u, dtype=np.float64)
        r = np.empty_like(u)
        n, arr = self.bcs
        self.lib.orc_dgsem_residual(self._m, riemann, n, arr, t, _p(u), _p(r))
        return r

    def time_step(self, u: np.ndarray, dt_guess: float, rk_order: int, cfl: float = 0.0) -> float:
        u = np.ascontiguousarray(u, dtype=np.float64)
        return float(self.lib.orc_time_step(self._m, _p(u), dt_guess, rk_order, cfl))

    def rk_update(self, riemann: int, order: int, t: float, dt: float, u: np.ndarray) -> np.ndarray:
        u = np.array(u, dtype=np.float64, copy=True)
        n, arr = self.bcs
        self.lib.orc_rk_update(self._m, riemann, n, arr, order, t, dt, _p(u))
        return u

    def vtk_sample(self, u: np.ndarray):
        """Writer<Part>::Prepare: (xyz [P, 3], values [P, 5], types [cells])."""
        u = np.ascontiguousarray(u, dtype=np.float64)
        xyz = np.empty((self.n_cells * 27, 3))
        v = np.empty((self.n_cells * 27, 5))
        self.lib.orc_vtk_sample(self._m, _p(u), _p(xyz), _p(v))
        return xyz, v, np.full(self.n_cells, 29, dtype=np.uint8)


def set_threads(n: int) -> None:
    load().orc_set_threads(n)


def rk_update_linear(order: int, a: np.ndarray, t: float, dt: float, u: np.ndarray) -> np.ndarray:
    a = np.ascontiguousarray(a, dtype=np.float64)
    u = np.array(u, dtype=np.float64, copy=True)
    load().orc_rk_update_linear(order, u.size, _p(a), t, dt, _p(u))
    return u


LIMITER_NONE, LIMITER_LAZY, LIMITER_DETECT_LAZY, LIMITER_EIGEN, LIMITER_EIGEN_ALL = 0, 1, 2, 3, 4


def eigen_matrices(cons, frame):
    """EigenMatrices (riemann/euler/eigen.hpp:27-56): L, R of a conservative
    state in the frame rows (normal, tangent, bitangent)."""
    lib = load()
    lib.orc_eigen_matrices.restype = None
    lib.orc_eigen_matrices.argtypes = [_D, _D, _D, _D]
    cons = np.ascontiguousarray(cons, dtype=np.float64)
    frame = np.ascontiguousarray(frame, dtype=np.float64)
    L, R = np.empty((5, 5)), np.empty((5, 5))
    lib.orc_eigen_matrices(_p(cons), _p(frame), _p(L), _p(R))
    return L, R


def _limiter_sigs(lib):
    sig = {
        "orc_limiter_create": (C.c_void_p, [C.c_void_p]),
        "orc_limiter_destroy": (None, [C.c_void_p]),
        "orc_modal_count": (C.c_int, [C.c_int]),
        "orc_limiter_modal": (None, [C.c_void_p, _D, _D]),
        "orc_limit": (C.c_int64, [C.c_void_p, C.c_int, C.c_double, C.c_double, _D]),
        "orc_limiter_troubled": (C.c_int64, [C.c_void_p, _D, C.c_char_p]),
        "orc_limiter_smoothness": (None, [C.c_void_p, C.c_int64, _D, _D]),
        "orc_rk_update_limited": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.POINTER(OrcBc), C.c_int, C.c_double,
                                            C.c_double, _D, C.c_void_p, C.c_int, C.c_double, C.c_double]),
        "orc_modal_limiter_create": (C.c_void_p, [C.c_void_p]),
        "orc_modal_rk_update_limited": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.POINTER(OrcBc), C.c_int,
                                                  C.c_double, C.c_double, _D, C.c_void_p, C.c_int, C.c_double,
                                                  C.c_double]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args


class Limiter:
    """WENO limiter (weno::Lazy reconstruct, optional weno::Eigen detector) on
    the DGSEM cells of an oracle Mesh."""

    def __init__(self, mesh: "Mesh", mode: int = LIMITER_LAZY, w0: float = 0.001, eps: float = 1e-6):
        self.lib = load()
        _limiter_sigs(self.lib)
        self.mesh = mesh
        self._l = self.lib.orc_limiter_create(mesh._m)
        self.mode, self.w0, self.eps = mode, w0, eps
        self.m = int(self.lib.orc_modal_count(mesh.degree))

    def __del__(self):
        if getattr(self, "_l", None):
            self.lib.orc_limiter_destroy(self._l)
            self._l = None

    def modal(self, u: np.ndarray) -> np.ndarray:
        u = np.ascontiguousarray(u, dtype=np.float64)
        out = np.empty((self.mesh.n_cells, 5, self.m))
        self.lib.orc_limiter_modal(self._l, _p(u), _p(out))
        return out

    def limit(self, u: np.ndarray) -> tuple[np.ndarray, int]:
        u = np.array(u, dtype=np.float64, copy=True)
        n = self.lib.orc_limit(self._l, self.mode, self.w0, self.eps, _p(u))
        return u, int(n)

    def troubled(self, u: np.ndarray) -> np.ndarray:
        u = np.ascontiguousarray(u, dtype=np.float64)
        flags = C.create_string_buffer(self.mesh.n_cells)
        self.lib.orc_limiter_troubled(self._l, _p(u), flags)
        return np.frombuffer(flags.raw, dtype=np.int8).astype(bool)

    def smoothness(self, cell: int, modal_coeff: np.ndarray) -> np.ndarray:
        cm = np.ascontiguousarray(modal_coeff, dtype=np.float64)
        beta = np.empty(5)
        self.lib.orc_limiter_smoothness(self._l, cell, _p(cm), _p(beta))
        return beta

    def rk_update(self, riemann: int, order: int, t: float, dt: float, u: np.ndarray) -> np.ndarray:
        u = np.array(u, dtype=np.float64, copy=True)
        n, arr = self.mesh.bcs
        self.lib.orc_rk_update_limited(self.mesh._m, riemann, n, arr, order, t, dt, _p(u), self._l,
                                       self.mode, self.w0, self.eps)
        return u


class ModalLimiter(Limiter):
    """The same WENO limiter on the cells of an oracle Modal system
    (WithLimiter<dg::General> over Projection): the column holds the modal
    coefficients, [cells][M][5]."""

    def __init__(self, modal: "Modal", mode: int = LIMITER_LAZY, w0: float = 0.001, eps: float = 1e-6):
        self.lib = load()
        _limiter_sigs(self.lib)
        self.mesh = modal
        self._l = self.lib.orc_modal_limiter_create(modal._m)
        self.mode, self.w0, self.eps = mode, w0, eps
        self.m = modal.m

    def rk_update(self, riemann: int, order: int, t: float, dt: float, u: np.ndarray) -> np.ndarray:
        u = np.array(u, dtype=np.float64, copy=True)
        n, arr = self.mesh.bcs
        self.lib.orc_modal_rk_update_limited(self.mesh._m, riemann, n, arr, order, t, dt, _p(u), self._l,
                                             self.mode, self.w0, self.eps)
        return u


def _visc_sigs(lib):
    sig = {
        "orc_visc_create": (C.c_void_p, [C.c_void_p, C.c_double, C.c_double, C.c_double]),
        "orc_visc_destroy": (None, [C.c_void_p]),
        "orc_visc_damping": (_D, [C.c_void_p]),
        "orc_visc_jumps": (None, [C.c_void_p, _D, _D]),
        "orc_visc_properties": (None, [C.c_void_p, _D, _D, _D]),
        "orc_visc_residual": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.POINTER(OrcBc), C.c_double, _D, _D, _D]),
        "orc_visc_time_step": (C.c_double, [C.c_void_p, _D, C.c_double, C.c_int, C.c_double]),
        "orc_visc_rk_update": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.POINTER(OrcBc), C.c_int, C.c_double,
                                         C.c_double, _D]),
        "orc_visc_node_derivatives": (None, [C.c_void_p, _D, C.c_int64, C.c_int, _D, _D]),
        "orc_initial_limiter": (C.c_int64, [C.c_void_p, C.c_int, _D]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args


INIT_AVERAGE, INIT_MAJORITY = 1, 2


class Viscosity:
    """EnergyBasedViscosity on the fr::Lobatto system of an oracle Mesh built
    with scheme="fr" (WithViscosity<fr::Lobatto>, Hex8 cells)."""

    def __init__(self, mesh: "Mesh", beta0: float = 2.0, beta1: float = 1.0 / 12, time_scale: float = 1.0):
        self.lib = load()
        _visc_sigs(self.lib)
        self.mesh = mesh
        self._v = self.lib.orc_visc_create(mesh._m, beta0, beta1, time_scale)
        if not self._v:
            raise RuntimeError("oracle viscosity needs an fr mesh of Hex8 cells")
        self.n = (mesh.degree + 1) ** 3

    def __del__(self):
        if getattr(self, "_v", None):
            self.lib.orc_visc_destroy(self._v)
            self._v = None

    def damping(self) -> np.ndarray:
        n, nc = self.n, self.mesh.n_cells
        ptr = self.lib.orc_visc_damping(self._v)
        return np.ctypeslib.as_array(ptr, shape=(nc, n, n)).copy()

    def jumps(self, u: np.ndarray) -> np.ndarray:
        u = np.ascontiguousarray(u, dtype=np.float64)
        out = np.empty((self.mesh.n_cells, 5))
        self.lib.orc_visc_jumps(self._v, _p(u), _p(out))
        return out

    def properties(self, u: np.ndarray) -> tuple[np.ndarray, float]:
        u = np.ascontiguousarray(u, dtype=np.float64)
        nu = np.empty((self.mesh.n_cells, 5))
        dt = np.zeros(1)
        self.lib.orc_visc_properties(self._v, _p(u), _p(nu), _p(dt))
        return nu, float(dt[0])

    def residual(self, riemann: int, u: np.ndarray, nu: np.ndarray | None = None, t: float = 0.0) -> np.ndarray:
        u = np.ascontiguousarray(u, dtype=np.float64)
        if nu is None:
            nu = self.properties(u)[0]
        nu = np.ascontiguousarray(nu, dtype=np.float64)
        r = np.empty_like(u)
        n, arr = self.mesh.bcs
        self.lib.orc_visc_residual(self._v, riemann, n, arr, t, _p(u), _p(nu), _p(r))
        return r

    def time_step(self, u: np.ndarray, dt_guess: float, rk_order: int, cfl: float = 0.0) -> float:
        u = np.ascontiguousarray(u, dtype=np.float64)
        return float(self.lib.orc_visc_time_step(self._v, _p(u), dt_guess, rk_order, cfl))

    def rk_update(self, riemann: int, order: int, t: float, dt: float, u: np.ndarray) -> np.ndarray:
        u = np.array(u, dtype=np.float64, copy=True)
        n, arr = self.mesh.bcs
        self.lib.orc_visc_rk_update(self._v, riemann, n, arr, order, t, dt, _p(u))
        return u

    def node_derivatives(self, u: np.ndarray, cell: int, node: int) -> tuple[np.ndarray, np.ndarray]:
        u = np.ascontiguousarray(u, dtype=np.float64)
        g = np.empty((3, 5))
        h = np.empty((6, 5))
        self.lib.orc_visc_node_derivatives(self._v, _p(u), cell, node, _p(g), _p(h))
        return g, h


def initial_limiter(mesh: "Mesh", kind: int, u: np.ndarray) -> tuple[np.ndarray, int]:
    """limiter::average / limiter::majority Reconstruct on a copy of u."""
    lib = load()
    _visc_sigs(lib)
    u = np.array(u, dtype=np.float64, copy=True)
    missing = lib.orc_initial_limiter(mesh._m, kind, _p(u))
    return u, int(missing)


def _modal_sigs(lib):
    P64, P32 = C.POINTER(C.c_int64), C.POINTER(C.c_int32)
    sig = {
        "orc_modal_create": (C.c_void_p, [C.c_int64, _D, C.c_int64, P64, P32, C.c_int32, C.c_int64, P64, P32,
                                          P32, _D, C.c_int]),
        "orc_modal_destroy": (None, [C.c_void_p]),
        "orc_modal_column_size": (C.c_int64, [C.c_void_p]),
        "orc_modal_basis_count": (C.c_int, [C.c_void_p]),
        "orc_modal_point_count": (C.c_int64, [C.c_void_p]),
        "orc_modal_points": (C.c_int, [C.c_void_p, _D, _D]),
        "orc_modal_face_point_count": (C.c_int64, [C.c_void_p]),
        "orc_modal_face_points": (C.c_int, [C.c_void_p, _D, _D, _D]),
        "orc_modal_cell_length": (C.c_double, [C.c_void_p, C.c_int64]),
        "orc_modal_values": (C.c_int, [C.c_void_p, _D, _D]),
        "orc_modal_project": (C.c_int, [C.c_void_p, _D, _D]),
        "orc_modal_residual": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.POINTER(OrcBc), C.c_double, _D, _D]),
        "orc_modal_time_step": (C.c_double, [C.c_void_p, _D, C.c_double, C.c_int, C.c_double]),
        "orc_modal_rk_update": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.POINTER(OrcBc), C.c_int, C.c_double,
                                          C.c_double, _D]),
        "orc_modal_vtk_sample": (C.c_int64, [C.c_void_p, _D, _D, _D, C.POINTER(C.c_uint8)]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args


class Modal:
    """Oracle-side modal DG system (dg::General over Projection) on a Hex8 /
    Tet4 mesh description; column layout per cell [M][5]."""

    def __init__(self, mesh, degree: int):
        lib = load()
        _modal_sigs(lib)
        ct = mesh.cell_type if mesh.cell_type is not None else np.zeros(mesh.n_cells, np.int32)
        self._keep = [np.ascontiguousarray(mesh.xyz, dtype=np.float64),
                      np.ascontiguousarray(mesh.cell_nodes, dtype=np.int64),
                      np.ascontiguousarray(ct, dtype=np.int32),
                      np.ascontiguousarray(mesh.face_cells, dtype=np.int64),
                      np.ascontiguousarray(mesh.face_sides, dtype=np.int32),
                      np.ascontiguousarray(mesh.face_group, dtype=np.int32),
                      np.ascontiguousarray(mesh.face_shift, dtype=np.float64)]
        xyz, cn, ct, fc, fs, fg, fsh = self._keep
        P64, P32 = C.POINTER(C.c_int64), C.POINTER(C.c_int32)
        self._m = lib.orc_modal_create(xyz.shape[0], _p(xyz), cn.shape[0], cn.ctypes.data_as(P64),
                                       ct.ctypes.data_as(P32), cn.shape[1], fc.shape[0], fc.ctypes.data_as(P64),
                                       fs.ctypes.data_as(P32), fg.ctypes.data_as(P32), _p(fsh), degree)
        if not self._m:
            raise RuntimeError("oracle rejected the modal mesh")
        self.lib = lib
        self.degree = degree
        self.n_cells = cn.shape[0]
        self.m = int(lib.orc_modal_basis_count(self._m))
        self.column_size = int(lib.orc_modal_column_size(self._m))
        self.n_points = int(lib.orc_modal_point_count(self._m))
        self.bcs = make_bcs({})

    def __del__(self):
        if getattr(self, "_m", None):
            self.lib.orc_modal_destroy(self._m)
            self._m = None

    def set_bcs(self, specs: dict[int, tuple]) -> None:
        pts = self.face_points()[0] if any(callable(v) for _, v in specs.values()) else None
        self.bcs = make_bcs(specs, pts)

    def points(self):
        xyz = np.empty((self.n_points, 3))
        w = np.empty(self.n_points)
        self.lib.orc_modal_points(self._m, _p(xyz), _p(w))
        return xyz, w

    def face_points(self):
        n = int(self.lib.orc_modal_face_point_count(self._m))
        xyz, w, fr = np.empty((n, 3)), np.empty(n), np.empty((n, 3, 3))
        self.lib.orc_modal_face_points(self._m, _p(xyz), _p(w), _p(fr))
        return xyz, w, fr

    def cell_length(self, c: int) -> float:
        return float(self.lib.orc_modal_cell_length(self._m, c))

    def values(self, u: np.ndarray) -> np.ndarray:
        u = np.ascontiguousarray(u, dtype=np.float64)
        v = np.empty((self.n_points, 5))
        self.lib.orc_modal_values(self._m, _p(u), _p(v))
        return v

    def project(self, values: np.ndarray) -> np.ndarray:
        values = np.ascontiguousarray(values, dtype=np.float64).reshape(self.n_points, 5)
        u = np.empty(self.column_size)
        self.lib.orc_modal_project(self._m, _p(values), _p(u))
        return u

    def residual(self, riemann: int, u: np.ndarray, t: float = 0.0) -> np.ndarray:
        u = np.ascontiguousarray(u, dtype=np.float64)
        r = np.empty_like(u)
        n, arr = self.bcs
        self.lib.orc_modal_residual(self._m, riemann, n, arr, t, _p(u), _p(r))
        return r

    def time_step(self, u: np.ndarray, dt_guess: float, rk_order: int, cfl: float = 0.0) -> float:
        u = np.ascontiguousarray(u, dtype=np.float64)
        return float(self.lib.orc_modal_time_step(self._m, _p(u), dt_guess, rk_order, cfl))

    def rk_update(self, riemann: int, order: int, t: float, dt: float, u: np.ndarray) -> np.ndarray:
        u = np.array(u, dtype=np.float64, copy=True)
        n, arr = self.bcs
        self.lib.orc_modal_rk_update(self._m, riemann, n, arr, order, t, dt, _p(u))
        return u

    def vtk_sample(self, u: np.ndarray):
        """Writer<Part>::Prepare: (xyz [P, 3], values [P, 5], types [cells])."""
        u = np.ascontiguousarray(u, dtype=np.float64)
        cap = self.n_cells * 27
        xyz, v = np.empty((cap, 3)), np.empty((cap, 5))
        types = np.empty(self.n_cells, dtype=np.uint8)
        n = int(self.lib.orc_modal_vtk_sample(self._m, _p(u), _p(xyz), _p(v),
                                              types.ctypes.data_as(C.POINTER(C.c_uint8))))
        if n < 0:
            raise RuntimeError("the VTK writer has no pyramid cell")
        return xyz[:n].copy(), v[:n].copy(), types


# ---------------------------------------------------------------------------
# Writer<Part>::WriteSolutions (mesh/vtk.hpp:526-669), restated in Python:
# the text of the .pvtu index and the .vtu piece written by one rank.

FIELD_NAMES = ("Density", "MomentumX", "MomentumY", "MomentumZ", "EnergyStagnationDensity")


def _fmt(x) -> str:
    """operator<< of a double at the stream defaults (%g, 6 digits)."""
    return "%g" % x


def vtk_inline_binary(data: bytes) -> str:
    """EncodeBase64 of the UInt64 byte count, then of the bytes (vtk.hpp:641-648)."""
    import base64
    import struct
    return base64.b64encode(struct.pack("<Q", len(data))).decode() + base64.b64encode(data).decode()


def pvtu_text(soln_name: str) -> str:
    lines = ['<VTKFile type="PUnstructuredGrid" version="1.0" byte_order="LittleEndian" header_type="UInt64">',
             '  <PUnstructuredGrid GhostLevel="1">', "    <PPointData>"]
    lines += [f'      <PDataArray type="Float64" Name="{f}"/>' for f in FIELD_NAMES]
    lines += ["    </PPointData>", "    <PCellData>", "    </PCellData>", "    <PPoints>",
              '      <PDataArray type="Float64" Name="Points" NumberOfComponents="3"/>', "    </PPoints>",
              f'    <Piece Source="./{soln_name}/0.vtu"/>', "  </PUnstructuredGrid>", "</VTKFile>"]
    return "\n".join(lines) + "\n"


def vtu_text(xyz: np.ndarray, values: np.ndarray, types: np.ndarray) -> str:
    n_points, n_cells = len(xyz), len(types)
    out = ['<VTKFile type="UnstructuredGrid" version="1.0" byte_order="LittleEndian" header_type="UInt64">\n',
           "  <UnstructuredGrid>\n", f'    <Piece NumberOfPoints="{n_points}" NumberOfCells="{n_cells}">\n',
           "      <PointData>\n"]
    for k, f in enumerate(FIELD_NAMES):
        out.append(f'        <DataArray type="Float64" Name="{f}" format="ascii">\n')
        out.append("".join(_fmt(v) + " " for v in values[:, k]))
        out.append("\n        </DataArray>\n")
    out += ["      </PointData>\n", "      <CellData>\n", "      </CellData>\n", "      <Points>\n",
            '        <DataArray type="Float64" Name="Points" NumberOfComponents="3" format="binary">\n',
            vtk_inline_binary(np.ascontiguousarray(xyz, dtype="<f8").tobytes()),
            "\n        </DataArray>\n", "      </Points>\n", "      <Cells>\n",
            '        <DataArray type="Int32" Name="connectivity" format="ascii">\n',
            "".join(f"{i} " for i in range(n_points)), "\n        </DataArray>\n",
            '        <DataArray type="Int32" Name="offsets" format="ascii">\n']
    t_ = np.asarray(types)
    sizes = np.where(t_ == 29, 27, np.where(t_ == 26, 15, 10))
    out.append("".join(f"{o} " for o in np.cumsum(sizes)))
    out += ["\n        </DataArray>\n", '        <DataArray type="UInt8" Name="types" format="ascii">\n',
            "".join(f"{int(t)} " for t in types), "\n        </DataArray>\n", "      </Cells>\n",
            "    </Piece>\n", "  </UnstructuredGrid>\n", "</VTKFile>\n"]
    return "".join(out)
