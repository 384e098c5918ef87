"""Host-side mirror of the reference's temporal / spatial interface.

``Lobatto`` plays the role of ``mini::spatial::dg::Lobatto`` (a
``mini::temporal::System``) and ``RungeKutta`` the role of
``mini::temporal::RungeKutta<order>``; both drive the GPU library through the
C ABI of include/mcfd.h.  Method names and argument meanings follow the
reference:

  System::SetTime / SetSolutionColumn / GetSolutionColumn / GetResidualColumn
      include/mini/temporal/ode.hpp:17-48
  FiniteElement::GetTimeStep(dt_guess, rk_order)      spatial/fem.hpp:417-435
  FiniteElement::Set<Boundary>(name, func)            spatial/fem.hpp:196-222
  FiniteElement::Approximate(func)                    spatial/fem.hpp:147-154
  Solver::Update(system, t_curr, dt)                  temporal/ode.hpp:92-105

Boundary "names" are the integer face groups of the mesh description.  A
boundary value is a constant conservative state, or a ``MovingSplit``
(value = a if x[axis] - speed * t < position else b), the two forms the
reference's drivers use (demo/euler/shock_tube.cpp, demo/euler/riemann2d.cpp).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import Callable

import numpy as np

from . import capi
from .mesh import Mesh, node_coordinates


@dataclass
class MovingSplit:
    axis: int
    position: float
    speed: float
    a: np.ndarray
    b: np.ndarray


@dataclass
class ObliqueSplit:
    """value(x, t) = (normal . x - speed t) < position ? a : b, e.g. the
    oblique moving shock of demo/euler/double_mach.cpp:28-31."""
    normal: np.ndarray
    position: float
    speed: float
    a: np.ndarray
    b: np.ndarray


def _bc_state(kind: int, value) -> capi.BcState:
    s = capi.BcState()
    s.kind = kind
    if value is None:
        s.program = capi.STATE_CONSTANT
    elif callable(value):
        s.program = capi.STATE_TABLE  # values set by _set_bc afterwards
    elif isinstance(value, ObliqueSplit):
        s.program = capi.STATE_OBLIQUE_SPLIT
        s.position = float(value.position)
        s.speed = float(value.speed)
        for k in range(3):
            s.normal[k] = float(value.normal[k])
        for k in range(5):
            s.a[k] = float(value.a[k])
            s.b[k] = float(value.b[k])
    elif isinstance(value, MovingSplit):
        s.program = capi.STATE_MOVING_SPLIT
        s.axis = int(value.axis)
        s.position = float(value.position)
        s.speed = float(value.speed)
        for k in range(5):
            s.a[k] = float(value.a[k])
            s.b[k] = float(value.b[k])
    else:
        v = np.asarray(value, dtype=np.float64)
        if v.shape != (5,):
            raise ValueError("a boundary value is a 5-component state")
        s.program = capi.STATE_CONSTANT
        for k in range(5):
            s.a[k] = float(v[k])
    return s


class Lobatto:
    """DGSEM (dg::Lobatto, kLocal = false) Euler system on one GPU."""

    def __init__(self, mesh: Mesh, degree: int, riemann: str | int = "rusanov",
                 cfl: float = 0.0, device: int = 0, precision: str = "fp64",
                 limiter: str = "none", weno_w0: float = 0.001, weno_eps: float = 1e-6,
                 scheme: str = "dgsem", contraction: str = "simt", shock_cells_fp64: int = 0):
        """precision: "fp64" (plain form) or "mixed" (FP32 volume flux and
        contraction; FP64 Riemann fluxes, lift and RK accumulation).
        limiter: "none", "lazy" (weno::Lazy on every cell) or "detect_lazy"
        (weno::Lazy on the cells the weno::Eigen jump detector flags), run
        after every solution update as WithLimiter does.
        contraction: "simt" (FP32 SIMT) or "tensor" (TF32x3 on the tensor
        cores; mixed DGSEM at p = 3) for the mixed form's differentiation.
        shock_cells_fp64 (mixed form with a limiter): 1 or 2 — the cells the
        last limiter pass flagged and that many layers of face neighbours take
        the FP64 cell update, the rest stays mixed."""
        lib = capi.load()
        self.mesh = mesh
        self.degree = int(degree)
        if precision not in ("fp64", "mixed"):
            raise ValueError("precision must be 'fp64' or 'mixed'")
        self.precision = precision
        self.riemann = capi.RIEMANN[riemann] if isinstance(riemann, str) else int(riemann)
        self._keep = [
            np.ascontiguousarray(mesh.xyz, dtype=np.float64),
            np.ascontiguousarray(mesh.cell_nodes, dtype=np.int64),
            np.ascontiguousarray(mesh.face_cells, dtype=np.int64),
            np.ascontiguousarray(mesh.face_sides, dtype=np.int32),
            np.ascontiguousarray(mesh.face_group, dtype=np.int32),
            np.ascontiguousarray(mesh.face_shift, dtype=np.float64),
            None if mesh.cell_type is None else np.ascontiguousarray(mesh.cell_type, dtype=np.int32),
        ]
        xyz, cn, fc, fs, fg, fsh, ct = self._keep
        desc = capi.MeshDesc()
        desc.n_nodes = xyz.shape[0]
        desc.xyz = capi.dptr(xyz)
        desc.n_cells = cn.shape[0]
        desc.cell_nodes = cn.ctypes.data_as(C.POINTER(C.c_int64))
        desc.cell_type = None if ct is None else ct.ctypes.data_as(C.POINTER(C.c_int32))
        desc.n_faces = fc.shape[0]
        desc.face_cells = fc.ctypes.data_as(C.POINTER(C.c_int64))
        desc.face_sides = fs.ctypes.data_as(C.POINTER(C.c_int32))
        desc.face_group = fg.ctypes.data_as(C.POINTER(C.c_int32))
        desc.face_shift = capi.dptr(fsh)
        desc.cell_node_stride = cn.shape[1]
        opt = capi.Options()
        opt.degree = self.degree
        if scheme not in capi.SCHEME:
            raise ValueError("scheme must be 'dgsem' (dg::Lobatto), 'fr' (fr::Lobatto) "
                             "or 'modal' (dg::General over Projection)")
        self.scheme = scheme
        opt.scheme = capi.SCHEME[scheme]
        opt.riemann = self.riemann
        opt.precision = capi.FP64 if precision == "fp64" else capi.MIXED
        opt.cfl = float(cfl)
        opt.device = int(device)
        opt.limiter = capi.LIMITER[limiter]
        opt.weno_w0 = float(weno_w0)
        opt.weno_eps = float(weno_eps)
        opt.contraction = capi.CONTRACTION[contraction]
        opt.shock_cells_fp64 = int(shock_cells_fp64)
        self.limiter = limiter
        h = C.c_void_p()
        capi.check(lib.mcfd_create(C.byref(desc), C.byref(opt), C.byref(h)), None)
        self._h = h
        self._lib = lib
        self.column_size = int(lib.mcfd_column_size(h))
        self.n_nodes_per_cell = (self.degree + 1) ** 3
        if scheme == "modal":
            self.n_nodes_per_cell = (self.degree + 1) * (self.degree + 2) * (self.degree + 3) // 6

    # -- lifetime
    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.mcfd_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def handle(self):
        return self._h

    def _check(self, code: int) -> None:
        capi.check(code, self._h)

    # -- boundary registration (fem.hpp:196-222).  value: a 5-component
    # state, a MovingSplit or ObliqueSplit (moving shocks, evaluated on the
    # device at every stage time), or a callable of the points [n, 3] ->
    # states [n, 5], sampled once at the group's face points (bc_points).
    def _set_bc(self, kind: int, group: int, value) -> None:
        self._check(self._lib.mcfd_set_bc(self._h, group, C.byref(_bc_state(kind, value))))
        if callable(value):
            pts = self.bc_points(group)
            vals = np.ascontiguousarray(value(pts), dtype=np.float64)
            if vals.shape != (pts.shape[0], 5):
                raise ValueError("a boundary function maps points [n, 3] to states [n, 5]")
            self._check(self._lib.mcfd_set_bc_table(self._h, group, capi.dptr(vals), pts.shape[0]))

    def bc_points(self, group: int) -> np.ndarray:
        """Face points [n, 3] of a boundary group (mcfd_bc_points)."""
        n = C.c_int64()
        self._check(self._lib.mcfd_bc_point_count(self._h, group, C.byref(n)))
        out = np.empty((n.value, 3))
        self._check(self._lib.mcfd_bc_points(self._h, group, capi.dptr(out), n.value))
        return out

    def SetInviscidWall(self, group: int) -> None:
        self._set_bc(capi.BC_INVISCID_WALL, group, None)

    def SetSupersonicOutlet(self, group: int) -> None:
        self._set_bc(capi.BC_SUPERSONIC_OUTLET, group, None)

    def SetSupersonicInlet(self, group: int, value) -> None:
        self._set_bc(capi.BC_SUPERSONIC_INLET, group, value)

    def SetSubsonicInlet(self, group: int, value) -> None:
        self._set_bc(capi.BC_SUBSONIC_INLET, group, value)

    def SetSubsonicOutlet(self, group: int, value) -> None:
        self._set_bc(capi.BC_SUBSONIC_OUTLET, group, value)

    def SetSmartBoundary(self, group: int, value) -> None:
        self._set_bc(capi.BC_SMART, group, value)

    def SetNoSlipWall(self, group: int) -> None:
        """fr::Lobatto only; with the artificial viscosity the wall flux minus
        nu n . grad(u) (fr/general.hpp:460-476), without it no correction."""
        self._check(self._lib.mcfd_set_bc(self._h, group, C.byref(_bc_state(capi.BC_NO_SLIP_WALL, None))))

    # -- energy-based artificial viscosity (spatial/viscosity.hpp, with_viscosity.hpp)
    def SetViscosity(self, ddg_beta0: float = 2.0, ddg_beta1: float = 1.0 / 12, time_scale: float = 1.0) -> None:
        """Direct::SetBetaValues + EnergyBasedViscosity::SetTimeScale + the
        WithViscosity construction (demo/euler/sourceless.cpp:117-121)."""
        self._check(self._lib.mcfd_set_viscosity(self._h, float(ddg_beta0), float(ddg_beta1), float(time_scale)))

    def GetViscosity(self) -> np.ndarray:
        """[cells, 5] viscosity of the current solution (GetPropertyOnCell)."""
        out = np.empty((self.mesh.n_cells, 5), dtype=np.float64)
        self._check(self._lib.mcfd_get_viscosity(self._h, capi.dptr(out), out.size))
        return out

    def InitialLimiter(self, kind: str) -> None:
        """limiter::average ("average") or limiter::majority ("majority")
        Reconstruct on the current solution."""
        code = {"average": capi.INIT_AVERAGE, "majority": capi.INIT_MAJORITY}[kind]
        self._check(self._lib.mcfd_initial_limiter(self._h, code))

    # -- System quartet (ode.hpp:17-48)
    def SetTime(self, t_curr: float) -> None:
        self._check(self._lib.mcfd_set_time(self._h, float(t_curr)))

    def SetSolutionColumn(self, column: np.ndarray) -> None:
        col = np.ascontiguousarray(column, dtype=np.float64)
        self._check(self._lib.mcfd_set_solution(self._h, capi.dptr(col), col.size))

    def GetSolutionColumn(self) -> np.ndarray:
        out = np.empty(self.column_size, dtype=np.float64)
        self._check(self._lib.mcfd_get_solution(self._h, capi.dptr(out), out.size))
        return out

    def get_solution_into(self, out: np.ndarray) -> None:
        """GetSolutionColumn into a caller-owned (e.g. pinned) float64 buffer."""
        if out.dtype != np.float64 or not out.flags.c_contiguous or out.size != self.column_size:
            raise ValueError("out must be a contiguous float64 array of the column size")
        self._check(self._lib.mcfd_get_solution(self._h, capi.dptr(out), out.size))

    def GetResidualColumn(self) -> np.ndarray:
        out = np.empty(self.column_size, dtype=np.float64)
        self._check(self._lib.mcfd_residual(self._h, capi.dptr(out), out.size))
        return out

    # -- device-pointer variants (torch tensors or raw addresses)
    def set_solution_device(self, ptr: int, n: int) -> None:
        self._check(self._lib.mcfd_set_solution_device(self._h, C.c_void_p(ptr), n))

    def get_solution_device(self, ptr: int, n: int) -> None:
        self._check(self._lib.mcfd_get_solution_device(self._h, C.c_void_p(ptr), n))

    def residual_device(self, ptr: int, n: int) -> None:
        self._check(self._lib.mcfd_residual_device(self._h, C.c_void_p(ptr), n))

    # -- spatial extras
    def GetTimeStep(self, dt_guess: float, rk_order: int) -> float:
        dt = C.c_double()
        self._check(self._lib.mcfd_time_step(self._h, float(dt_guess), int(rk_order), C.byref(dt)))
        return dt.value

    def Approximate(self, func: Callable[[np.ndarray], np.ndarray]) -> None:
        """Interpolate func (vectorised over [M, 3] points -> [M, 5]) at the
        GLL nodes (polynomial/hexahedron.hpp:642-648) and load it."""
        x = node_coordinates(self.mesh, self.degree).reshape(-1, 3)
        self.SetSolutionColumn(np.ascontiguousarray(func(x), dtype=np.float64).ravel())

    def node_coordinates(self) -> np.ndarray:
        return node_coordinates(self.mesh, self.degree)

    def face_node_maps(self) -> tuple[np.ndarray, np.ndarray]:
        qf = (self.degree + 1) ** 2
        h = np.empty((self.mesh.n_faces, qf), dtype=np.int16)
        s = np.empty((self.mesh.n_faces, qf), dtype=np.int16)
        self._check(self._lib.mcfd_face_node_maps(
            self._h, h.ctypes.data_as(C.POINTER(C.c_int16)), s.ctypes.data_as(C.POINTER(C.c_int16))))
        return h, s

    def launch_count(self) -> int:
        return int(self._lib.mcfd_launch_count(self._h))

    def advance(self, n_steps: int, dt_guess: float, rk_order: int, t: float) -> float:
        """n_steps x {dt = GetTimeStep; Update(t, dt)} with dt, t on device."""
        tt = C.c_double(float(t))
        self._check(self._lib.mcfd_advance(self._h, int(n_steps), float(dt_guess), int(rk_order), C.byref(tt)))
        return tt.value

    # -- output and restart (mesh/vtk.hpp Writer, mesh/part.hpp Gather/Scatter/Write/ReadSolutions)
    def vtk_sample(self) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
        """Writer<Part>::Prepare on the current solution: (xyz [P, 3],
        values [P, 5], VTK cell types [cells]), hexahedra as Hexahedron27,
        tetrahedra as Tetrahedron10, wedges as Wedge15 (pyramids: refused, the
        reference's writer has none), points cell by cell."""
        n = C.c_int64()
        self._check(self._lib.mcfd_vtk_point_count(self._h, C.byref(n)))
        xyz = np.empty((n.value, 3))
        values = np.empty((n.value, 5))
        types = np.empty(self.mesh.n_cells, dtype=np.uint8)
        self._check(self._lib.mcfd_vtk_sample(self._h, capi.dptr(xyz), capi.dptr(values),
                                              types.ctypes.data_as(C.POINTER(C.c_uint8)), n.value))
        return xyz, values, types

    def WriteSolutions(self, directory: str, soln_name: str, binary: bool = False) -> None:
        """<directory>/<soln_name>.pvtu + <directory>/<soln_name>/0.vtu."""
        self._check(self._lib.mcfd_write_vtu(self._h, str(directory).encode(), soln_name.encode(),
                                             int(bool(binary))))

    def gather_fields_device(self, ptr: int, n: int) -> None:
        self._check(self._lib.mcfd_gather_fields(self._h, C.c_void_p(ptr), n))

    def scatter_fields_device(self, ptr: int, n: int) -> None:
        self._check(self._lib.mcfd_scatter_fields(self._h, C.c_void_p(ptr), n))

    def write_restart(self, path: str, t: float) -> None:
        self._check(self._lib.mcfd_write_restart(self._h, str(path).encode(), float(t)))

    def read_restart(self, path: str) -> float:
        t = C.c_double()
        self._check(self._lib.mcfd_read_restart(self._h, str(path).encode(), C.byref(t)))
        return t.value

    # -- streamed stepping (uploads/downloads overlap the neighbouring jobs' compute)
    def stream_begin(self) -> None:
        self._check(self._lib.mcfd_stream_begin(self._h))

    def stream_step(self, host_in: np.ndarray, host_out: np.ndarray, t: float, n_steps: int,
                    dt_guess: float, rk_order: int) -> None:
        """Enqueue one job: load host_in at time t, advance n_steps, store into
        host_out.  Both arrays must stay alive (and host_in unchanged) until
        stream_end; page-locked arrays make the copies asynchronous."""
        for a in (host_in, host_out):
            if a.dtype != np.float64 or not a.flags.c_contiguous or a.size != self.column_size:
                raise ValueError("stream buffers must be contiguous float64 arrays of the column size")
        self._check(self._lib.mcfd_stream_step(self._h, capi.dptr(host_in), capi.dptr(host_out), host_in.size,
                                               float(t), int(n_steps), float(dt_guess), int(rk_order)))

    def stream_end(self) -> None:
        self._check(self._lib.mcfd_stream_end(self._h))

    def Limit(self) -> int:
        """limiter::Reconstruct on the current solution; returns the number of
        reconstructed cells."""
        n = C.c_int64()
        self._check(self._lib.mcfd_limit(self._h, C.byref(n)))
        return n.value

    def troubled_cells(self) -> int:
        """Cells reconstructed since the previous call."""
        n = C.c_int64()
        self._check(self._lib.mcfd_troubled_cells(self._h, C.byref(n)))
        return n.value

    def kernel_times(self, reps: int = 10) -> dict:
        """Average CUDA-event milliseconds per launch of each stage kernel."""
        out = (C.c_double * 4)()
        self._check(self._lib.mcfd_kernel_times(self._h, int(reps), out))
        return {"dt": out[0], "face_flux": out[1], "cell_update": out[2], "rk3_step": out[3]}

    def synchronize(self) -> None:
        self._check(self._lib.mcfd_synchronize(self._h))

    def autotune(self, cache_path: str | None = None) -> dict:
        """mcfd_autotune: pick the fastest launch shapes on this mesh and
        solution (optionally through a JSON-lines cache file)."""
        out = (C.c_int32 * 4)()
        path = cache_path.encode() if cache_path else None
        self._check(self._lib.mcfd_autotune(self._h, path, out))
        return {"face_block": out[0], "dt_block": out[1], "limiter_blocks_per_sm": out[2],
                "from_cache": bool(out[3])}

    # -- batching: independent cases inside this handle
    def set_cases(self, case_offsets) -> None:
        """Cells [offsets[k], offsets[k+1]) form case k, with its own dt and t."""
        off = np.ascontiguousarray(case_offsets, dtype=np.int64)
        self._check(self._lib.mcfd_set_cases(self._h, off.size - 1, off.ctypes.data_as(C.POINTER(C.c_int64))))
        self.n_cases = off.size - 1

    def case_times(self) -> tuple[np.ndarray, np.ndarray]:
        """(t, last dt) of every case."""
        t = np.empty(self.n_cases)
        dt = np.empty(self.n_cases)
        self._check(self._lib.mcfd_case_times(self._h, capi.dptr(t), capi.dptr(dt), self.n_cases))
        return t, dt

    def set_stream(self, stream_ptr: int | None) -> None:
        self._check(self._lib.mcfd_set_stream(self._h, C.c_void_p(stream_ptr or 0)))


class General(Lobatto):
    """Modal DG (dg::General over polynomial::Projection) Euler system on one
    GPU, on every cell type (hexahedra, tetrahedra, wedges, pyramids).  The column holds, per cell, the M x 5
    coefficients on the cell's orthonormal Taylor basis (m-major)."""

    def __init__(self, mesh: Mesh, degree: int, riemann: str | int = "rusanov",
                 cfl: float = 0.0, device: int = 0, precision: str = "fp64",
                 limiter: str = "none", weno_w0: float = 0.001, weno_eps: float = 1e-6):
        """precision: "fp64", or "mixed" (FP32 contractions on FP32 copies of
        the basis and point offsets; FP64 face states, Riemann fluxes and RK
        accumulation).  limiter: as for Lobatto, on the cells' own bases
        (WithLimiter<dg::General> over Projection, every cell type); it runs
        after every solution update and after Approximate / project."""
        super().__init__(mesh, degree, riemann, cfl=cfl, device=device, scheme="modal",
                         precision=precision, limiter=limiter, weno_w0=weno_w0, weno_eps=weno_eps)
        self.n_points = int(self._lib.mcfd_point_count(self._h))

    def points(self) -> np.ndarray:
        """Global coordinates [n_points, 3] of the volume quadrature points."""
        out = np.empty((self.n_points, 3), dtype=np.float64)
        self._check(self._lib.mcfd_points(self._h, capi.dptr(out), self.n_points))
        return out

    def project(self, values: np.ndarray) -> None:
        """Load the projection of values [n_points, 5] given at points()."""
        v = np.ascontiguousarray(values, dtype=np.float64)
        if v.size != self.n_points * 5:
            raise ValueError("values must hold 5 components per quadrature point")
        self._check(self._lib.mcfd_project(self._h, capi.dptr(v), self.n_points))

    def Approximate(self, func: Callable[[np.ndarray], np.ndarray]) -> None:
        """Projection::Approximate (polynomial/projection.hpp:28-42) of func
        (vectorised over [M, 3] points -> [M, 5])."""
        self.project(func(self.points()))

    def node_coordinates(self) -> np.ndarray:
        raise NotImplementedError("the modal scheme has no nodes; use points()")

    def face_node_maps(self):
        raise NotImplementedError("the modal scheme evaluates both sides at each face point")


class Ensemble:
    """Several systems stepped by one CUDA graph per step (mcfd_ensemble)."""

    def __init__(self, systems):
        self._lib = capi.load()
        self.systems = list(systems)
        arr = (C.c_void_p * len(self.systems))(*[s.handle.value for s in self.systems])
        e = C.c_void_p()
        code = self._lib.mcfd_ensemble_create(arr, len(self.systems), C.byref(e))
        if code != capi.OK:
            msg = self._lib.mcfd_ensemble_last_error(None)
            raise capi.McfdError(code, msg.decode() if msg else "")
        self._e = e

    def advance(self, n_steps: int, dt_guess: float, rk_order: int) -> None:
        code = self._lib.mcfd_ensemble_advance(self._e, int(n_steps), float(dt_guess), int(rk_order))
        if code != capi.OK:
            msg = self._lib.mcfd_ensemble_last_error(self._e)
            raise capi.McfdError(code, msg.decode() if msg else "")

    def _ens_check(self, code: int) -> None:
        if code != capi.OK:
            msg = self._lib.mcfd_ensemble_last_error(self._e)
            raise capi.McfdError(code, msg.decode() if msg else "")

    def stream_begin(self) -> None:
        self._ens_check(self._lib.mcfd_ensemble_stream_begin(self._e))

    def stream_step(self, host_in, host_out, n_steps: int, dt_guess: float, rk_order: int) -> None:
        """Enqueue one job: every member's column from host_in[i], n_steps
        ensemble steps, the columns into host_out[i] (arrays kept alive and
        unread until stream_end; page-locked for asynchronous copies)."""
        n = len(self.systems)
        if len(host_in) != n or len(host_out) != n:
            raise ValueError("one input and one output column per member")
        for s, a, b in zip(self.systems, host_in, host_out):
            for x in (a, b):
                if x.dtype != np.float64 or not x.flags.c_contiguous or x.size != s.column_size:
                    raise ValueError("stream buffers must be contiguous float64 arrays of each column size")
        ins = (capi._D * n)(*[capi.dptr(a) for a in host_in])
        outs = (capi._D * n)(*[capi.dptr(b) for b in host_out])
        self._ens_check(self._lib.mcfd_ensemble_stream_step(self._e, ins, outs, int(n_steps), float(dt_guess),
                                                            int(rk_order)))

    def stream_end(self) -> None:
        self._ens_check(self._lib.mcfd_ensemble_stream_end(self._e))

    def set_stream(self, stream_ptr: int) -> None:
        code = self._lib.mcfd_ensemble_set_stream(self._e, C.c_void_p(stream_ptr))
        if code != capi.OK:
            msg = self._lib.mcfd_ensemble_last_error(self._e)
            raise capi.McfdError(code, msg.decode() if msg else "")

    def close(self) -> None:
        if getattr(self, "_e", None):
            self._lib.mcfd_ensemble_destroy(self._e)
            self._e = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class RungeKutta:
    """mini::temporal::RungeKutta<order> (rk.hpp:10-57) over a Lobatto system:
    the whole update runs as fused device stages."""

    def __init__(self, order: int):
        if order not in (1, 2, 3):
            raise ValueError("order must be 1, 2 or 3")
        self.order = order

    def Update(self, system: Lobatto, t_curr: float, dt: float) -> None:
        system._check(system._lib.mcfd_rk_step(system.handle, float(t_curr), float(dt), self.order))


def write_vtu_arrays(directory: str, soln_name: str, xyz: np.ndarray, values: np.ndarray,
                     types: np.ndarray, binary: bool = False) -> None:
    """The .pvtu / .vtu writer on host arrays (no device needed)."""
    lib = capi.load()
    xyz = np.ascontiguousarray(xyz, dtype=np.float64)
    values = np.ascontiguousarray(values, dtype=np.float64)
    types = np.ascontiguousarray(types, dtype=np.uint8)
    capi.check(lib.mcfd_write_vtu_arrays(str(directory).encode(), soln_name.encode(), len(xyz),
                                         capi.dptr(xyz), capi.dptr(values), len(types),
                                         types.ctypes.data_as(C.POINTER(C.c_uint8)), int(bool(binary))))


def base64_encode(data: bytes) -> str:
    """The library's base64 of VTK binary arrays."""
    lib = capi.load()
    buf = (C.c_uint8 * max(len(data), 1)).from_buffer_copy(data if data else b"\0")
    n = C.c_int64()
    capi.check(lib.mcfd_base64_encode(buf, len(data), None, 0, C.byref(n)))
    out = C.create_string_buffer(n.value + 1)
    capi.check(lib.mcfd_base64_encode(buf, len(data), out, n.value + 1, C.byref(n)))
    return out.value.decode()
