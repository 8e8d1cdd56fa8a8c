"""MAC_CylinderFlow / GhostCellIntegrator for the ghost-cell AB2/CN path on the GPU.

Drop-in for the reference's ``MAC_CylinderFlow(boundary='ghost_cell',
time_scheme='ab2_cn')`` (solver/main.py) and its ``gg`` integrator
(solver/optimized_ghost_cell.py): same constructor keywords, ``solve``
signature, ``last_step_diagnostics`` keys, checkpoint schema and exceptions.
All arithmetic runs in libghostmac.so on the GPU; this module only moves
arrays and maps status codes to exceptions.  numpy arrays (host) and CUDA
torch tensors (device) are both accepted by the integrator methods.
"""
from __future__ import annotations

import ctypes as C
import hashlib
import json
import os
import tempfile
import time as _time
import weakref
from pathlib import Path
from types import SimpleNamespace

import numpy as np

from . import _lib
from ._args import check_reference_arguments
from ._lib import check, lib, ptr

_PKG = Path(__file__).resolve().parent


def pinned_empty(shape):
    """A float64 numpy array in page-locked host memory (gm_host_alloc), so that the state
    copies of every solve() run by DMA; an ordinary np.empty when none can be had.  The
    memory is freed when the last array viewing it is collected."""
    n = int(np.prod(shape))
    p = C.c_void_p()
    if n == 0 or lib.gm_host_alloc(C.c_size_t(n * 8), C.byref(p)) != _lib.GM_OK or not p.value:
        return np.empty(shape)
    buf = (C.c_double * n).from_address(p.value)
    fin = weakref.finalize(buf, lib.gm_host_free, C.c_void_p(p.value))
    fin.atexit = False  # the CUDA runtime may be gone by then; the process exit frees it
    return np.frombuffer(buf, dtype=np.float64).reshape(shape)


def _f64(a):
    if hasattr(a, 'data_ptr'):
        return a.contiguous()
    return np.ascontiguousarray(a, dtype=np.float64)


def _like(x, n):
    """Output buffer matching the input's residence (torch device tensor or numpy)."""
    if hasattr(x, 'data_ptr'):
        import torch
        return torch.empty(n, dtype=torch.float64, device=x.device)
    return np.empty(n)


class PointOperator:
    """A sparse operator in CSR form (rows = sample points, columns = flat grid indices) with
    ``op @ x`` for a flat host array: what the reference keeps as a scipy CSR matrix."""

    def __init__(self, indptr, indices, data, ncols):
        self.indptr, self.indices, self.data = indptr, indices, data
        self.shape = (len(indptr) - 1, int(ncols))

    def __matmul__(self, x):
        x = np.asarray(x, dtype=np.float64).ravel()
        if x.size != self.shape[1]:
            raise ValueError('operand size does not match the operator')
        prod = self.data * x[self.indices]
        out = np.zeros(self.shape[0])
        rows = np.repeat(np.arange(self.shape[0]), np.diff(self.indptr))
        np.add.at(out, rows, prod)
        return out

    def toarray(self):
        a = np.zeros(self.shape)
        rows = np.repeat(np.arange(self.shape[0]), np.diff(self.indptr))
        np.add.at(a, (rows, self.indices), self.data)
        return a


def pressure_reconstruction(handle, points, ncols):
    """Quadratic point-pressure operator at (y, x) points through gm_pressure_reconstruction
    (solver/cut_cell_solver.py:25-55); invalid points raise the reference's ValueError."""
    pts = np.ascontiguousarray(points, dtype=np.float64)
    if pts.ndim != 2 or pts.shape[1] != 2 or not np.isfinite(pts).all():
        raise ValueError('Pressure sample points must be finite (y, x) pairs')
    nnz = C.c_int64()
    check(lib.gm_pressure_reconstruction(handle, ptr(pts), len(pts), C.byref(nnz), None, None, None), handle)
    indptr = np.empty(len(pts) + 1, np.int64)
    cols = np.empty(nnz.value, np.int64)
    vals = np.empty(nnz.value)
    check(lib.gm_pressure_reconstruction(handle, ptr(pts), len(pts), C.byref(nnz), ptr(indptr), ptr(cols),
                                         ptr(vals)), handle)
    return PointOperator(indptr, cols, vals, ncols)


class GhostCellIntegrator:
    """GPU counterpart of solver/optimized_ghost_cell.py:GhostCellIntegrator for one case."""

    def __init__(self, handle, solver):
        self._h = handle
        self.solver = solver
        s = _lib.Sizes()
        check(lib.gm_get_sizes(handle, C.byref(s)), handle)
        self.sizes = s
        self.ui = np.empty(s.nu_active, np.int64)
        self.vi = np.empty(s.nv_active, np.int64)
        self.pi = np.empty(s.np_active, np.int64)
        check(lib.gm_get_indices(handle, ptr(self.ui), ptr(self.vi), ptr(self.pi)), handle)
        self.qsize = int(s.qsize)
        self.usize = int(s.usize)
        self.nx, self.ny = int(s.nx), int(s.ny)
        pts = np.empty((s.n_surface, 2))
        check(lib.gm_get_surface_points(handle, ptr(pts)), handle)
        self.surface_points = pts
        self.geom = SimpleNamespace(nx=solver.nx, ny=solver.ny, dx=solver.dx, dy=solver.dy, Lx=solver.Lx,
                                    Ly=solver.Ly, xc=solver.xc, yc=solver.yc, R=solver.D / 2)
        self.last_diagnostics = {}
        self.pressure_inverse_info = dict(backend='fft_boundary_schur', rank=int(s.rank_p))
        self.reconstruction_info = dict(velocity=solver.ghost_velocity_interpolation,
                                        pressure=solver.ghost_pressure_extension)

    # -- packing (solver/optimized_ghost_cell.py:174-184)
    def pack(self, u, v, out=None):
        f = np.concatenate((np.ascontiguousarray(u, np.float64).ravel(), np.ascontiguousarray(v, np.float64).ravel())) \
            if not hasattr(u, 'data_ptr') else __import__('torch').cat((u.reshape(-1), v.reshape(-1)))
        y = _like(f, self.qsize) if out is None else out
        check(lib.gm_apply(self._h, _lib.OP_PACK, 0.0, ptr(f), ptr(y)), self._h)
        return y

    def unpack(self, q):
        q = _f64(q)
        y = _like(q, self.usize + (self.ny + 1) * self.nx)
        check(lib.gm_apply(self._h, _lib.OP_UNPACK, 0.0, ptr(q), ptr(y)), self._h)
        return y[:self.usize].reshape(self.ny, self.nx + 1), y[self.usize:].reshape(self.ny + 1, self.nx)

    def _op(self, op, x, n, param=0.0):
        x = _f64(x)
        y = _like(x, n)
        check(lib.gm_apply(self._h, op, float(param), ptr(x), ptr(y)), self._h)
        return y

    # -- operators (solver/optimized_ghost_cell.py:186-234)
    def advection(self, q, compiled=True, out=None):
        return self._op(_lib.OP_ADVECTION, q, self.qsize)

    def diffusion(self, q, out=None):
        return self._op(_lib.OP_DIFFUSION, q, self.qsize)

    def gradient(self, p, out=None):
        # a full pressure grid acts through its first len(pi) raveled entries, as in the
        # reference's unchecked CSR kernel (solver/numba_kernels.py:347-354)
        x = p.reshape(-1)[:len(self.pi)] if p.ndim > 1 else p
        return self._op(_lib.OP_GRADIENT, x, self.qsize)

    def divergence(self, q, out=None):
        return self._op(_lib.OP_DIVERGENCE, q, len(self.pi))

    def H_matvec(self, q, dt, out=None):
        return self._op(_lib.OP_H_MATVEC, q, self.qsize, dt)

    def pressure_extend(self, p_packed):
        return self._op(_lib.OP_PRESSURE_EXTEND, p_packed, self.nx * self.ny).reshape(self.ny, self.nx)

    def project(self, q, dt, out=None):
        q = _f64(q)
        qo = _like(q, self.qsize)
        phi = _like(q, len(self.pi))
        info = _lib.SolveInfo()
        check(lib.gm_project(self._h, float(dt), ptr(q), ptr(qo), ptr(phi), C.byref(info)), self._h)
        self.pressure_inverse_info['last_solve'] = _solve_dict(info)
        return qo, phi

    def pressure_solve(self, rhs):
        rhs = _f64(rhs)
        phi = _like(rhs, len(self.pi))
        info = _lib.SolveInfo()
        check(lib.gm_pressure_solve(self._h, ptr(rhs), ptr(phi), C.byref(info)), self._h)
        self.pressure_inverse_info['last_solve'] = _solve_dict(info)
        return phi

    def rectangle_solve(self, kind, b, dt=0.0):
        """Separable inverse of solver/rectangular_inverse.py:8-58 on a rectangle grid."""
        k = {'pressure': 0, 'u': 1, 'v': 2}[kind]
        b = _f64(b)
        x = _like(b, b.size if hasattr(b, 'size') and not callable(b.size) else b.numel())
        check(lib.gm_rectangle_solve(self._h, k, float(dt), ptr(b), ptr(x)), self._h)
        return x.reshape(b.shape)

    def surface_forces(self, u, v, p, mu):
        out = np.empty(6)
        u, v, p = _f64(u), _f64(v), _f64(p)
        check(lib.gm_surface_forces(self._h, ptr(u), ptr(v), ptr(p), float(mu), ptr(out)), self._h)
        return tuple(float(x) for x in out)

    def pressure_reconstruction(self, points):
        """Quadratic point-pressure operator at (y, x) points (rows) over the flat pressure grid
        (build_pressure_reconstruction of solver/cut_cell_solver.py:25-55)."""
        return pressure_reconstruction(self._h, points, self.nx * self.ny)

    def ghost_stencils(self, which):
        """(rows, ptr, cols, vals) of the ghost rows of E_u (0), E_v (1) or P (2), grid flat indices."""
        n, nnz = C.c_int64(), C.c_int64()
        check(lib.gm_get_ghost_stencils(self._h, which, C.byref(n), C.byref(nnz), None, None, None, None), self._h)
        rows, p_ = np.empty(n.value, np.int64), np.empty(n.value + 1, np.int64)
        cols, vals = np.empty(nnz.value, np.int64), np.empty(nnz.value)
        check(lib.gm_get_ghost_stencils(self._h, which, None, None, ptr(rows), ptr(p_), ptr(cols), ptr(vals)), self._h)
        return rows, p_, cols, vals

    def schur_rows(self, which):
        n = C.c_int64()
        check(lib.gm_get_schur_rows(self._h, which, C.byref(n), None), self._h)
        if n.value < 0:
            return None
        rows = np.empty(n.value, np.int64)
        check(lib.gm_get_schur_rows(self._h, which, None, ptr(rows)), self._h)
        return rows

    # -- AB2 history (solver/optimized_ghost_cell.py:129, 266)
    def history(self):
        has = C.c_int32()
        dt = C.c_double()
        adv = np.empty(self.qsize)
        half = np.empty(len(self.pi))
        check(lib.gm_get_history(self._h, C.byref(has), ptr(adv), ptr(half), C.byref(dt)), self._h)
        if not has.value:
            return None, None, None
        return adv, half, dt.value

    @property
    def previous_advection(self):
        return self.history()[0]

    @property
    def half_pressure(self):
        return self.history()[1]

    @property
    def previous_dt(self):
        return self.history()[2]

    def set_history(self, previous_advection, half_pressure, previous_dt):
        if previous_advection is None:
            check(lib.gm_set_history(self._h, 0, None, None, 0.0), self._h)
            return
        a, h = _f64(previous_advection), _f64(half_pressure)
        check(lib.gm_set_history(self._h, 1, ptr(a), ptr(h), float(previous_dt)), self._h)


def _solve_dict(info):
    return dict(iterations=int(info.iterations), residual_linf=float(info.residual_linf),
                residual_relative_l2=float(info.residual_relative_l2),
                refinement_iterations=int(info.refinement_iterations),
                residual_target_linf=float(info.residual_target_linf),
                roundoff_bound_linf=float(info.roundoff_bound_linf), status=int(info.status))


class MAC_CylinderFlow:
    """Cylinder flow on the GPU with the reference's MAC_CylinderFlow constructor
    (solver/main.py:19-617), defaults included (boundary='immersed', time_scheme='legacy').  This
    class runs the ghost-cell AB2/CN path; the other paths are other classes, which the
    constructor returns: boundary='cut_cell' (either time scheme) cutcell.CutCellFlow,
    boundary='staircase' staircase.StaircaseFlow, boundary='ghost_cell' with
    time_scheme='legacy' staircase.LegacyGhostFlow.  boundary='immersed' is not built."""

    def __new__(cls, *args, **kwargs):
        import inspect
        bound = inspect.signature(cls.__init__).bind_partial(None, *args, **kwargs).arguments
        boundary, scheme = bound.get('boundary', 'immersed'), bound.get('time_scheme', 'legacy')
        if boundary == 'cut_cell':
            from .cutcell import CutCellFlow
            return CutCellFlow(*args, **kwargs)
        if boundary == 'staircase':
            from .staircase import StaircaseFlow
            return StaircaseFlow(*args, **kwargs)
        if boundary == 'ghost_cell' and scheme == 'legacy':
            from .staircase import LegacyGhostFlow
            return LegacyGhostFlow(*args, **kwargs)
        return super().__new__(cls)

    def __init__(self, nx=400, ny=100, Lx=20.0, Ly=5.0, D=1.0, xc=5.0, yc=2.5,
                 nu=0.01, rho=1.0, U_inf=1.0, inflow='uniform', U_m=None,
                 slip_walls=False, verbose=True, boundary='immersed', transport='centered',
                 pressure_solver='direct', marker_spacing_factor=1.5, time_scheme='legacy',
                 ghost_pressure_extension='neumann', ghost_velocity_interpolation='bilinear', precision='fp64'):
        """Keywords and defaults of solver/main.py:40-44.  ``precision`` (this library only): 'fp64'
        runs the plain FP64 method; 'fp32' runs the separable inverses and the momentum stencils in
        FP32 and refines every solve against the FP64 operator until the reference's residual
        targets hold."""
        check_reference_arguments(boundary, transport, pressure_solver, time_scheme, ghost_pressure_extension,
                                  ghost_velocity_interpolation)
        if boundary != 'ghost_cell' or time_scheme != 'ab2_cn':
            raise NotImplementedError(f'boundary={boundary!r} with time_scheme={time_scheme!r} is not built here '
                                      '(the immersed-boundary projection is outside this library)')
        if pressure_solver not in ('direct', 'iterative') or slip_walls:
            raise ValueError('Ghost AB2/CN requires direct/iterative pressure and no-slip channel walls')
        if any(isinstance(n, bool) or not isinstance(n, (int, np.integer)) or n < 4 for n in (nx, ny)):
            raise ValueError('nx and ny must be integers >= 4')
        if U_m is not None and (not np.isfinite(U_m) or U_m <= 0):
            raise ValueError('U_m must be finite and positive')
        if precision not in ('fp64', 'fp32'):
            raise ValueError("precision must be 'fp64' or 'fp32'")
        self.precision = precision
        self.configuration = dict(nx=nx, ny=ny, Lx=Lx, Ly=Ly, D=D, xc=xc, yc=yc, nu=nu, rho=rho, U_inf=U_inf,
                                  inflow=inflow, U_m=U_m, slip_walls=slip_walls, boundary=boundary,
                                  transport=transport, pressure_solver=pressure_solver,
                                  marker_spacing_factor=marker_spacing_factor, time_scheme=time_scheme,
                                  verbose=False, ghost_pressure_extension=ghost_pressure_extension,
                                  ghost_velocity_interpolation=ghost_velocity_interpolation, precision=precision)
        self.boundary, self.transport, self.pressure_solver, self.time_scheme = boundary, transport, pressure_solver, time_scheme
        self.ghost_pressure_extension = ghost_pressure_extension
        self.ghost_velocity_interpolation = ghost_velocity_interpolation
        self.verbose = verbose
        self.nx, self.ny, self.Lx, self.Ly = int(nx), int(ny), float(Lx), float(Ly)
        self.D, self.xc, self.yc, self.nu, self.rho, self.U_inf = D, xc, yc, nu, rho, U_inf
        self.inflow, self.slip_walls = inflow, slip_walls
        cfg = _lib.Config(nx=int(nx), ny=int(ny), Lx=float(Lx), Ly=float(Ly), D=float(D), xc=float(xc),
                          yc=float(yc), nu=float(nu), rho=float(rho), U_inf=float(U_inf),
                          inflow={'uniform': 0, 'parabolic': 1}.get(inflow, -1),
                          U_m=float(U_m) if U_m is not None else 0.0,
                          pressure_solver=0 if pressure_solver == 'direct' else 1,
                          pressure_extension=0 if ghost_pressure_extension == 'neumann' else 1,
                          velocity_interpolation=0 if ghost_velocity_interpolation == 'bilinear' else 1,
                          precision=0 if precision == 'fp64' else 1)
        h = C.c_void_p()
        t0 = _time.time()
        check(lib.gm_create(C.byref(cfg), C.byref(h)))
        self._h = h
        self.dx, self.dy = self.Lx / self.nx, self.Ly / self.ny
        if inflow == 'parabolic':
            self.U_m = 1.5 * U_inf if U_m is None else U_m
            self.U_ref = (2.0 / 3.0) * self.U_m
        else:
            self.U_m = self.U_ref = U_inf
        self.Re = self.U_ref * self.D / self.nu
        self.y_centers = (np.arange(self.ny) + 0.5) * self.dy
        self.x_centers = (np.arange(self.nx) + 0.5) * self.dx
        rr = (((self.x_centers - xc) / (D / 2.0)) ** 2)[None, :] + (((self.y_centers - yc) / (D / 2.0)) ** 2)[:, None]
        self.mask = rr <= (1.0 + 1e-13)
        if inflow == 'parabolic':
            y = self.y_centers
            self.u_inlet = 4.0 * self.U_m * y * (self.Ly - y) / (self.Ly ** 2)
        else:
            self.u_inlet = np.full(self.ny, float(U_inf))
        self.u_inlet_base = self.u_inlet.copy()
        self.u = pinned_empty((self.ny, self.nx + 1))
        self.v = pinned_empty((self.ny + 1, self.nx))
        self.p = pinned_empty((self.ny, self.nx))
        self.phi = np.zeros((self.ny, self.nx))
        self.gg = GhostCellIntegrator(h, self)
        self._pull()
        self.time = 0.0
        self.run_options = {}
        self.last_step_diagnostics = {}
        if verbose:
            print(f"Ghost AB2/CN on the GPU ready in {_time.time() - t0:.3f}s (Re={self.Re:.1f}).")

    def __del__(self):
        h = getattr(self, '_h', None)
        if h:
            lib.gm_destroy(h)
            self._h = None

    # -- state transfer
    def _pull(self):
        check(lib.gm_get_state(self._h, ptr(self.u), ptr(self.v), ptr(self.p)), self._h)

    def _push(self):
        for name in ('u', 'v', 'p'):
            a = getattr(self, name)
            if not (isinstance(a, np.ndarray) and a.dtype == np.float64 and a.flags['C_CONTIGUOUS']):
                setattr(self, name, np.ascontiguousarray(a, dtype=np.float64))
        check(lib.gm_set_state(self._h, ptr(self.u), ptr(self.v), ptr(self.p)), self._h)

    def _set_inlet(self):
        self.u_inlet = np.ascontiguousarray(self.u_inlet, dtype=np.float64)
        check(lib.gm_set_inlet(self._h, ptr(self.u_inlet)), self._h)

    def _diag_dict(self, d):
        solves = [dict(iterations=0, residual_linf=float(d.pressure_residual_linf),
                       residual_relative_l2=float(d.pressure_residual_relative_l2), status=0)
                  for _ in range(d.pressure_solve_count)]
        return dict(momentum_iterations=0, momentum_residual_linf=d.momentum_residual_linf,
                    coupled_momentum_residual_linf=d.coupled_momentum_residual_linf,
                    pressure_backend='gmres_rectangle' if self.pressure_solver == 'iterative' else 'fft_boundary_schur',
                    pressure_solve_count=int(d.pressure_solve_count),
                    pressure_iterations=int(d.pressure_iterations),
                    pressure_refinement_iterations=int(d.pressure_refinement_iterations),
                    pressure_residual_linf=d.pressure_residual_linf,
                    pressure_residual_relative_l2=d.pressure_residual_relative_l2, pressure_seconds=0.0,
                    pressure_solves=solves, time=d.time, dt=d.dt, max_divergence=d.max_divergence, cfl=d.cfl,
                    cd=d.cd, cl=d.cl, cd_pressure=d.cd_pressure, cd_viscous=d.cd_viscous,
                    cl_pressure=d.cl_pressure, cl_viscous=d.cl_viscous)

    def step_raw(self, dt, n_steps, first_index=0, start_time=None):
        """n_steps on the device state without host transfers; returns the diag records."""
        diag = (_lib.StepDiag * n_steps)()
        t = self.time if start_time is None else start_time
        rc = lib.gm_step(self._h, float(dt), int(n_steps), int(first_index), float(t), diag)
        return rc, diag

    def solve(self, n_steps=25000, dt=0.002, perturb_transient=True, perturb_duration=None, perturb_amp=0.15,
              save_artifacts=True, verbose=None, step_callback=None):
        """Step loop of solver/main.py:245-501 for the ghost-cell AB2/CN path."""
        if isinstance(n_steps, bool) or not isinstance(n_steps, (int, np.integer)) or n_steps <= 0:
            raise ValueError('n_steps must be a positive integer')
        if not np.isfinite(dt) or dt <= 0:
            raise ValueError('dt must be finite and positive')
        if perturb_duration is None:
            perturb_duration = 2.5 * (self.D / self.U_ref)
        if not np.isfinite(perturb_duration) or perturb_duration <= 0 or not np.isfinite(perturb_amp) or abs(perturb_amp) >= 1:
            raise ValueError('Require perturb_duration > 0 and finite |perturb_amp| < 1')
        self.run_options = dict(perturb_transient=perturb_transient, perturb_duration=perturb_duration,
                                perturb_amp=perturb_amp)
        verbose = self.verbose if verbose is None else verbose
        for name in ('u', 'v', 'p'):
            a = getattr(self, name)
            if not (isinstance(a, np.ndarray) and a.dtype == np.float64 and a.flags['C_CONTIGUOUS']):
                setattr(self, name, np.ascontiguousarray(a, dtype=np.float64))
        t0 = _time.time()
        start = self.time
        ts, cds, cls = [], [], []
        s = 0
        pushed = False
        while s < n_steps:
            now_t = start + (s + 1) * dt
            perturbing = perturb_transient and self.inflow == 'uniform' and now_t <= perturb_duration
            if perturbing:
                decay = 1.0 - (now_t / perturb_duration)
                pert = perturb_amp * np.sin(2.0 * np.pi * self.y_centers / self.Ly) * decay
                self.u_inlet[:] = self.u_inlet_base * (1.0 + pert)
                chunk = 1
            else:
                self.u_inlet[:] = self.u_inlet_base
                if step_callback is not None:
                    chunk = 1
                elif verbose:
                    # up to the next printed step: 0, 1000, 2000, ... and the last one
                    chunk = min(n_steps - s, 1001 - s % 1000 if s % 1000 else 1)
                else:
                    chunk = n_steps - s
            # one call per chunk: the state in (first chunk), the inlet, the steps, the state out
            # (last chunk, or when a callback or the verbose report reads it)
            self.u_inlet = np.ascontiguousarray(self.u_inlet, dtype=np.float64)
            pull = s + chunk >= n_steps or step_callback is not None or verbose
            diag = (_lib.StepDiag * chunk)()
            st_in = (None, None, None) if pushed else (ptr(self.u), ptr(self.v), ptr(self.p))
            st_out = (ptr(self.u), ptr(self.v), ptr(self.p)) if pull else (None, None, None)
            rc = lib.gm_solve_io(self._h, *st_in, ptr(self.u_inlet), float(dt), int(chunk), int(s),
                                 float(start + s * dt), diag, *st_out)
            pushed = True
            done = chunk
            if rc != _lib.GM_OK:
                done = next((k for k in range(chunk) if diag[k].status), chunk)
            for k in range(done):
                d = diag[k]
                self.time = d.time
                self.last_step_diagnostics = self._diag_dict(d)
                ts.append(d.time)
                cds.append(d.cd)
                cls.append(d.cl)
            if rc != _lib.GM_OK:
                self._pull()
                check(rc, self._h)
            s += chunk
            if step_callback is not None:
                step_callback(self, dict(self.last_step_diagnostics))
            if verbose and ((s - 1) % 1000 == 0 or s == n_steps):
                # Div_RMS over every fluid cell: sqrt(sum div^2 / count) (solver/main.py:445)
                stats = self.divergence_stats()
                rms = np.sqrt(stats[1] / stats[2]) if stats[2] > 0 else 0.0
                flux_in, flux_out = np.sum(self.u[:, 0]) * self.dy, np.sum(self.u[:, self.nx]) * self.dy
                print(f"Step {s - 1:5d} | Div_RMS: {rms:.2e} | Div_Max: {stats[0]:.2e} | "
                      f"FluxErr: {abs(flux_out - flux_in) / flux_in:.2e} | "
                      f"Cd: {self.last_step_diagnostics['cd']:.4f} | Cl: {self.last_step_diagnostics['cl']:.4f}")
        if verbose:
            elapsed = _time.time() - t0
            print(f"Simulation completed in {elapsed:.2f}s ({elapsed / n_steps * 1000:.2f} ms/step)")
        return np.array(ts), np.array(cds), np.array(cls)

    def helmholtz_solver_info(self):
        """How the FP32 mode applies its CN Helmholtz inverse for the current dt: the FP32 Jacobi
        iterations per application (0: the FFT + boundary Schur inverse) and the row-sum norm
        of the Jacobi iteration matrix that chose them."""
        it, rho = C.c_int32(), C.c_double()
        check(lib.gm_solver_info(self._h, C.byref(it), C.byref(rho)), self._h)
        return dict(jacobi_iters=int(it.value), jacobi_rho=float(rho.value))

    def divergence_stats(self):
        """mac_engine.calculate_mac_divergence_cpp statistics (solver/src/bindings.cpp:343-390):
        (max, sum div^2, count, core sum div^2, core count)."""
        out = np.empty(3)
        counts = np.empty(2, np.int64)
        u, v = _f64(self.u), _f64(self.v)
        check(lib.gm_divergence_stats(self._h, ptr(u), ptr(v), ptr(out), ptr(counts)), self._h)
        return float(out[0]), float(out[1]), int(counts[0]), float(out[2]), int(counts[1])

    # -- checkpoints (solver/main.py:503-585), schema 1
    def _source_hashes(self):
        files = ['ghost.py', '_lib.py', 'csrc/ghostmac.cu', 'csrc/kernels.cu', 'csrc/kernels.cuh',
                 'csrc/transforms.cuh', 'csrc/geometry.cpp', 'csrc/geometry.hpp']
        return {name: hashlib.sha256((_PKG / name).read_bytes()).hexdigest() for name in files}

    def metadata(self, dt, n_steps, perturb_transient=True, perturb_duration=None, perturb_amp=.15):
        if perturb_duration is None:
            perturb_duration = 2.5 * self.D / self.U_ref
        return dict(nx=self.nx, ny=self.ny, Lx=self.Lx, Ly=self.Ly, D=self.D, xc=self.xc, yc=self.yc, nu=self.nu,
                    rho=self.rho, U_ref=self.U_ref, U_inf=self.U_inf, U_m=self.U_m, inflow=self.inflow,
                    slip_walls=self.slip_walls, dt=dt, n_steps=n_steps, end_time=self.time, boundary=self.boundary,
                    transport=self.transport, time_integrator='AB2_CN_discrete_incremental',
                    time_scheme=self.time_scheme, pressure_solver=self.pressure_solver,
                    pressure_backend='ghost_fft_boundary_schur', ghost_pressure_extension=self.ghost_pressure_extension,
                    ghost_velocity_interpolation=self.ghost_velocity_interpolation,
                    pressure_preconditioner=self.gg.pressure_inverse_info, perturb_transient=perturb_transient,
                    perturb_duration=perturb_duration, perturb_amp=perturb_amp, source_sha256=self._source_hashes())

    def save_checkpoint(self, path, *, overwrite=False):
        """Atomic schema-1 checkpoint with the AB2 history (solver/main.py:503-530)."""
        path = Path(path)
        if path.exists() and not overwrite:
            raise FileExistsError(path)
        path.parent.mkdir(parents=True, exist_ok=True)
        adv, half, prev_dt = self.gg.history()
        arrays = dict(u=self.u, v=self.v, p=self.p, phi=self.phi, u_inlet=self.u_inlet)
        if adv is not None:
            arrays.update(previous_advection=adv, half_pressure=half)
        meta = dict(schema=1, configuration=self.configuration, time=self.time, run_options=self.run_options,
                    prev_dt=prev_dt, cn_dt=prev_dt, diagnostics=self.last_step_diagnostics,
                    source_sha256=self._source_hashes())
        tmp = None
        try:
            with tempfile.NamedTemporaryFile(dir=path.parent, suffix='.npz', delete=False) as stream:
                tmp = Path(stream.name)
                np.savez(stream, checkpoint_metadata=json.dumps(meta), **arrays)
                stream.flush()
                os.fsync(stream.fileno())
            os.replace(tmp, path)
        finally:
            if tmp is not None and tmp.exists():
                tmp.unlink()

    @classmethod
    def from_checkpoint(cls, path, *, check_sources=True, accept_reference=False, precision=None):
        """Resume a schema-1 checkpoint; reject foreign sources or incomplete AB2 history (solver/main.py:532-567).

        A checkpoint written by the reference solver's own save_checkpoint (ghost-cell AB2/CN:
        the same arrays, packed history layouts and metadata keys) is imported when
        ``accept_reference`` is set, and rejected as a source mismatch otherwise.  ``precision``
        overrides the checkpoint's precision mode ('fp64' for a reference checkpoint)."""
        with np.load(path, allow_pickle=False) as data:
            meta = json.loads(str(data['checkpoint_metadata']))
            if meta.get('schema') != 1 or meta['configuration'].get('boundary') not in ('cut_cell', 'ghost_cell'):
                raise ValueError('Unsupported checkpoint')
            if meta['configuration'].get('boundary') == 'cut_cell':
                from .cutcell import CutCellFlow
                return CutCellFlow.from_checkpoint(path, check_sources=check_sources,
                                                   accept_reference=accept_reference)
            sources = meta.get('source_sha256') or {}
            from_reference = 'optimized_ghost_cell.py' in sources and 'compiled_engine' in sources
            if from_reference and not accept_reference:
                raise ValueError('Checkpoint source mismatch: written by the reference solver '
                                 '(from_checkpoint(..., accept_reference=True) imports it)')
            config = dict(meta['configuration'])
            config['verbose'] = False
            if precision is not None:
                config['precision'] = precision
            solver = cls(**config)
            if check_sources and not from_reference and sources != solver._source_hashes():
                raise ValueError('Checkpoint source mismatch')
            solver.restored_from = 'reference' if from_reference else 'library'
            for name in ('u', 'v', 'p', 'phi', 'u_inlet'):
                value = data[name]
                target = getattr(solver, name)
                if value.shape != target.shape or not np.isfinite(value).all():
                    raise ValueError(f'Invalid checkpoint field: {name}')
                target[:] = value
            solver.time = float(meta['time'])
            if not np.isfinite(solver.time) or solver.time < 0:
                raise ValueError('Invalid checkpoint time')
            solver.run_options = meta['run_options']
            solver.last_step_diagnostics = meta['diagnostics']
            hist = {}
            for name, shape in (('previous_advection', (solver.gg.qsize,)), ('half_pressure', (len(solver.gg.pi),))):
                value = data[name].copy() if name in data else None
                if solver.time > 0 and (value is None or value.shape != shape or not np.isfinite(value).all()):
                    raise ValueError(f'Incomplete Ghost AB2/CN history: {name}')
                hist[name] = value
            prev_dt = meta['prev_dt']
            if solver.time > 0 and (prev_dt is None or not np.isfinite(prev_dt) or prev_dt <= 0):
                raise ValueError('Invalid Ghost timestep history')
            solver._push()
            if hist['previous_advection'] is not None:
                solver.gg.set_history(hist['previous_advection'], hist['half_pressure'], prev_dt)
            return solver


def _constructor_signature(cls):
    """The constructor keywords of cls.__init__ (without self), so that inspect.signature of the
    class reports them rather than the dispatching __new__'s (*args, **kwargs)."""
    import inspect
    sig = inspect.signature(cls.__init__)
    return sig.replace(parameters=list(sig.parameters.values())[1:])


MAC_CylinderFlow.__signature__ = _constructor_signature(MAC_CylinderFlow)


class CylinderBatch:
    """Independent ``MAC_CylinderFlow`` cases advanced together on one GPU.

    Every steady step of all cases is one CUDA graph launch in which each case is a
    concurrent branch with its own refinement loops (gm_batch_step).  The reference steps
    one case per process; a batch gives the same per-case results as stepping each case
    alone (the same kernels in the same order per case).  Cases may differ in grid size,
    geometry, viscosity and precision mode.  The inlet is held at its base profile (no
    start-up perturbation) while the batch steps.
    """

    def __init__(self, cases):
        cases = list(cases)
        if not cases or not all(isinstance(c, MAC_CylinderFlow) for c in cases):
            raise ValueError('CylinderBatch takes a non-empty list of MAC_CylinderFlow cases')
        if len({id(c) for c in cases}) != len(cases):
            raise ValueError('a case appears twice in the batch')
        self.cases = cases
        arr = (C.c_void_p * len(cases))(*[c._h.value for c in cases])
        b = C.c_void_p()
        check(lib.gm_batch_create(arr, len(cases), C.byref(b)))
        self._b = b

    def close(self):
        b = getattr(self, '_b', None)
        if b:
            lib.gm_batch_destroy(b)
            self._b = None

    def __del__(self):
        self.close()

    def _check(self, rc):
        if rc != _lib.GM_OK:
            msg = (lib.gm_batch_last_error(self._b) or b'').decode(errors='replace')
            raise _lib.error_for(rc, msg)

    def launch_shapes(self):
        """(gthreads, groups per block, columns per block) the batch chose by timing, and the
        probe times of its candidates in ms (-1: did not fit); zeros before the first steady step."""
        shape = (C.c_int32 * 3)()
        ms = (C.c_float * 8)()
        check(lib.gm_batch_shapes(self._b, shape, ms, 8))
        return tuple(shape), [float(x) for x in ms]

    def step_raw(self, dt, n_steps, first_index=0):
        """n_steps of every case on the device state; returns (rc, diag[n_cases][n_steps], steps_done)."""
        n = len(self.cases)
        diag = (_lib.StepDiag * (n * n_steps))()
        done = np.zeros(n, np.int32)
        t0 = np.array([c.time for c in self.cases], np.float64)
        rc = lib.gm_batch_step(self._b, float(dt), int(n_steps), int(first_index), ptr(t0), diag, ptr(done))
        return rc, diag, done

    def solve(self, n_steps, dt=0.002, first_index=0):
        """Advance every case n_steps (the loop of solver/main.py:245-501 without the inlet
        perturbation); returns per case (times, C_D, C_L)."""
        if isinstance(n_steps, bool) or not isinstance(n_steps, (int, np.integer)) or n_steps <= 0:
            raise ValueError('n_steps must be a positive integer')
        if not np.isfinite(dt) or dt <= 0:
            raise ValueError('dt must be finite and positive')
        for c in self.cases:
            c._push()
            c.u_inlet[:] = c.u_inlet_base
            c._set_inlet()
        rc, diag, done = self.step_raw(dt, n_steps, first_index)
        out = []
        for i, c in enumerate(self.cases):
            recs = [diag[i * n_steps + k] for k in range(int(done[i]))]
            for d in recs:
                c.time = d.time
                c.last_step_diagnostics = c._diag_dict(d)
            c._pull()
            out.append((np.array([d.time for d in recs]), np.array([d.cd for d in recs]),
                        np.array([d.cl for d in recs])))
        self._check(rc)
        return out
