"""MAC_CylinderFlow(boundary='cut_cell') on the GPU, with either time scheme.

The reference's cut-cell path (CutCellBoundary, solver/cut_cell_solver.py:370-1015, stepped by
solver/main.py:245-501) with the same constructor keywords, ``solve`` loop, diagnostics keys and
exceptions: the AB2/CN step (time_scheme='ab2_cn', advance_ab2_cn) and the legacy step
(time_scheme='legacy': advance_momentum_predictor with centred transport and AB2 or upwind
transport and forward Euler, then compute_rhs, solve_pressure and apply_corrector).  The geometry-dependent setup runs once on the host (cutcell_geometry.py); the
pressure operator, its boundary-corrected inverse and every step run in libghostmac.so
(gm_cc_* entry points, csrc/cutcell.cu).  All three pressure_solver choices of the reference
('direct' sparse LU, 'iterative' ILU-GMRES, 'cg_dct' CG with the boundary-Schur DCT
preconditioner) solve the same cut-cell Poisson system to the same 1e-10 divergence budget;
here each is the boundary-corrected separable inverse with residual refinement, which solves it
to rounding.
"""
from __future__ import annotations

import ctypes as C
import hashlib
import json
import os
import tempfile
import time as _time
from pathlib import Path

import numpy as np

from . import _lib
from ._args import check_reference_arguments
from ._lib import lib, ptr
from .cutcell_geometry import CutCellSetup

FAMILIES = (('u', 'x'), ('u', 'y'), ('v', 'x'), ('v', 'y'))
_PKG = Path(__file__).resolve().parent


def _check(rc, handle=None):
    if rc != _lib.GM_OK:
        raise _lib.error_for(rc, lib.gm_cc_last_error(handle).decode(errors='replace'))


def _i64(a):
    return np.ascontiguousarray(a, dtype=np.int64)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


class _Keep:
    """Host arrays referenced by a gm_cc_config while the handle is built."""

    def __init__(self):
        self.arrays = []

    def __call__(self, a, kind='f'):
        a = _f64(a) if kind == 'f' else (_i64(a) if kind == 'i' else np.ascontiguousarray(a, dtype=np.int32))
        self.arrays.append(a)
        return a.ctypes.data

    def csr(self, m):
        m = m.tocsr()
        return _lib.Csr(self(m.indptr, 'i'), self(m.indices, 'i'), self(m.data))


def _viscous_rows(setup, key):
    """Viscous override rows of one family: the reconstruction and ring faces with their
    gradient rows, then any fitted face of the momentum stencil the reconstruction misses
    (its flux stays rho nu times the momentum stencil's gradient row)."""
    from scipy.sparse import vstack
    df, mf = setup.diffusion_faces[key], setup.momentum_faces[key]
    have = set(int(f) for f in df.indices)
    extra = [k for k, f in enumerate(mf.indices) if int(f) not in have]
    if not extra:
        return df.indices, df.gradient
    return np.r_[df.indices, mf.indices[extra]], vstack((df.gradient, mf.gradient[extra]), format='csr')


class CutCellIntegrator:
    """The cut-cell integrator's operators on the GPU (CutCellBoundary methods and the closures
    of advance_ab2_cn, solver/cut_cell_solver.py:640-1002) over packed vectors q."""

    def __init__(self, handle, solver, setup):
        self._h = handle
        self._s = solver
        self.setup = setup
        self.geom = setup.geom
        self.nx, self.ny, self.dx, self.dy = solver.nx, solver.ny, solver.dx, solver.dy
        self.wall = setup.wall
        self.momentum_faces = setup.momentum_faces
        self.diffusion_faces = setup.diffusion_faces
        self.u_vol, self.u_covered, self.u_owner = setup.u_vol, setup.u_covered, setup.u_owner
        self.v_vol, self.v_covered, self.v_owner = setup.v_vol, setup.v_covered, setup.v_owner
        self.u_vol_eff, self.v_vol_eff = setup.u_vol_eff, setup.v_vol_eff
        sz = _lib.Sizes()
        _check(lib.gm_cc_get_sizes(handle, C.byref(sz)), handle)
        self.sizes = sz
        self.ui = np.empty(sz.nu_active, np.int64)
        self.vi = np.empty(sz.nv_active, np.int64)
        self.pi = np.empty(sz.np_active, np.int64)
        _check(lib.gm_cc_get_indices(handle, ptr(self.ui), ptr(self.vi), ptr(self.pi)), handle)
        self.qsize = int(sz.qsize)
        pts = np.empty((sz.n_surface, 2))
        _check(lib.gm_cc_get_surface_points(handle, ptr(pts)), handle)
        self.pressure_points = pts
        self.pressure_inverse_info = dict(kind='dct_boundary_schur', rank=int(sz.rank_p))
        self.last_pressure_diagnostics = {}

    # -- packing (advance_ab2_cn's pack / unpack, :962-971)
    def pack(self, u, v):
        return np.r_[np.asarray(u).ravel()[self.ui], np.asarray(v).ravel()[self.vi]]

    def unpack(self, q, u_inlet=None):
        u = np.zeros((self.ny, self.nx + 1))
        v = np.zeros((self.ny + 1, self.nx))
        u[:, 0] = self._s.u_inlet if u_inlet is None else u_inlet
        n = len(self.ui)
        u.ravel()[self.ui] = q[:n]
        v.ravel()[self.vi] = q[n:]
        return u, v

    def _apply(self, op, param, x, n_out, n_out2=0):
        x = _f64(x)
        y = np.empty(n_out)
        y2 = np.empty(n_out2) if n_out2 else None
        _check(lib.gm_cc_apply(self._h, op, float(param), ptr(x), ptr(y), ptr(y2) if n_out2 else None), self._h)
        return (y, y2) if n_out2 else y

    def compute_momentum_rhs(self, u, v, nu, rho, transport='upwind', include_advection=True):
        """(a_u, a_v, rhs_u, rhs_v) of CutCellBoundary.compute_momentum_rhs
        (solver/cut_cell_solver.py:790-957): the advective form (centred or upwind transport)
        and the viscous form, each one device evaluation; with advection and nu != 0 the two
        are added (the reference adds the fluxes before differencing, which agrees to
        rounding)."""
        if transport not in ('centered', 'upwind'):
            raise ValueError('transport must be centered or upwind')
        if float(rho) != float(self._s.rho):
            raise ValueError('rho must be the case density')
        field = np.r_[_f64(u).ravel(), _f64(v).ravel()]
        n = field.size
        a = r = None
        if include_advection:
            op = _lib.CC_OP_MOMENTUM_ADVECTION if transport == 'centered' else _lib.CC_OP_MOMENTUM_ADVECTION_UPWIND
            a, r = self._apply(op, 0.0, field, n, n)
        if nu != 0 or not include_advection:
            ad, rd = self._apply(_lib.CC_OP_MOMENTUM_DIFFUSION, nu, field, n, n)
            a, r = (ad, rd) if a is None else (a + ad, r + rd)
        us = (self.ny) * (self.nx + 1)
        shp_u, shp_v = (self.ny, self.nx + 1), (self.ny + 1, self.nx)
        return a[:us].reshape(shp_u), a[us:].reshape(shp_v), r[:us].reshape(shp_u), r[us:].reshape(shp_v)

    def advection(self, q):
        return self._apply(_lib.CC_OP_ADVECTION, 0.0, q, self.qsize)

    def diffusion(self, q):
        return self._apply(_lib.CC_OP_DIFFUSION, 0.0, q, self.qsize)

    def H_matvec(self, q, dt):
        return self._apply(_lib.CC_OP_H_MATVEC, dt, q, self.qsize)

    def project(self, q, dt):
        """(projected q, phi) of advance_ab2_cn's project (solver/cut_cell_solver.py:993-1002)."""
        y, phi = self._apply(_lib.CC_OP_PROJECT, dt, q, self.qsize, self.nx * self.ny)
        return y, phi.reshape(self.ny, self.nx)

    def solve_pressure(self, rhs, dt, rho, divergence_tolerance=1e-10):
        """CutCellBoundary.solve_pressure (solver/cut_cell_solver.py:688-730)."""
        rhs = np.asarray(rhs, dtype=float)
        if (rhs.shape != (self.ny, self.nx) or not np.isfinite(rhs).all()
                or not np.isfinite([dt, rho, divergence_tolerance]).all()
                or min(dt, rho, divergence_tolerance) <= 0):
            raise ValueError('Invalid pressure solve inputs')
        if float(rho) != float(self._s.rho) or divergence_tolerance != 1e-10:
            raise NotImplementedError('the case density and the 1e-10 divergence budget are built in')
        return self._apply(_lib.CC_OP_PRESSURE_SOLVE, dt, rhs, self.nx * self.ny).reshape(self.ny, self.nx)

    def extract_true_surface_forces(self, u, v, p, mu):
        out = np.empty(6)
        _check(lib.gm_cc_surface_forces(self._h, ptr(_f64(u)), ptr(_f64(v)), ptr(_f64(p)), float(mu), ptr(out)),
               self._h)
        return tuple(float(x) for x in out)

    def divergence_stats(self, u=None, v=None):
        """(max |div|, rms div, max |net flux|) of calculate_cut_cell_divergence."""
        out = np.empty(3)
        _check(lib.gm_cc_divergence_stats(self._h, ptr(_f64(u)) if u is not None else None,
                                          ptr(_f64(v)) if v is not None else None, ptr(out)), self._h)
        return tuple(float(x) for x in out)

    # -- restart history (cn_advection, cn_pressure, cn_dt)
    def history(self):
        has = C.c_int32()
        dtp = C.c_double()
        adv = np.empty(self.qsize)
        half = np.empty((self.ny, self.nx))
        _check(lib.gm_cc_get_history(self._h, C.byref(has), ptr(adv), ptr(half), C.byref(dtp)), self._h)
        if not has.value:
            return None, None, None
        return adv, half, float(dtp.value)

    @property
    def cn_advection(self):
        return self.history()[0]

    @property
    def cn_pressure(self):
        return self.history()[1]

    @property
    def cn_dt(self):
        return self.history()[2]

    def set_history(self, cn_advection, cn_pressure, cn_dt):
        if cn_advection is None:
            _check(lib.gm_cc_set_history(self._h, 0, None, None, 0.0), self._h)
            return
        _check(lib.gm_cc_set_history(self._h, 1, ptr(_f64(cn_advection)), ptr(_f64(cn_pressure)), float(cn_dt)),
               self._h)


class CutCellFlow:
    """The cut-cell MAC_CylinderFlow on the GPU (solver/main.py:19-501 with boundary='cut_cell'):
    the AB2/CN step (time_scheme='ab2_cn', centred transport) or the legacy step
    (time_scheme='legacy', centred or upwind transport)."""

    def __init__(self, nx=400, ny=100, Lx=20.0, Ly=5.0, D=1.0, xc=5.0, yc=2.5, nu=0.01, rho=1.0, U_inf=1.0,
                 inflow='uniform', U_m=None, slip_walls=False, verbose=True, boundary='cut_cell',
                 transport='centered', pressure_solver='direct', marker_spacing_factor=1.5, time_scheme='legacy',
                 ghost_pressure_extension='neumann', ghost_velocity_interpolation='bilinear', precision='fp64'):
        # argument checks of solver/main.py:45-129
        check_reference_arguments(boundary, transport, pressure_solver, time_scheme, ghost_pressure_extension,
                                  ghost_velocity_interpolation)
        if boundary != 'cut_cell':
            raise NotImplementedError('CutCellFlow implements boundary="cut_cell"')
        if precision != 'fp64':
            raise NotImplementedError('the cut-cell path runs in FP64')
        if any(isinstance(n, bool) or not isinstance(n, (int, np.integer)) or n < 4 for n in (nx, ny)):
            raise ValueError('nx and ny must be integers >= 4')
        if not all(np.isfinite(x) and x > 0 for x in (Lx, Ly, D, nu, rho, U_inf)):
            raise ValueError('Domain lengths, D, nu, rho and U_inf must be finite and positive')
        if inflow not in ('uniform', 'parabolic'):
            raise ValueError('inflow must be uniform or parabolic')
        if U_m is not None and (not np.isfinite(U_m) or U_m <= 0):
            raise ValueError('U_m must be finite and positive')
        if not (D / 2 < xc < Lx - D / 2 and D / 2 < yc < Ly - D / 2):
            raise ValueError('Cylinder must lie strictly inside the channel')
        self.configuration = dict(nx=nx, ny=ny, Lx=Lx, Ly=Ly, D=D, xc=xc, yc=yc, nu=nu, rho=rho, U_inf=U_inf,
                                  inflow=inflow, U_m=U_m, slip_walls=slip_walls, boundary=boundary,
                                  transport=transport, pressure_solver=pressure_solver,
                                  marker_spacing_factor=marker_spacing_factor, time_scheme=time_scheme,
                                  verbose=False, ghost_pressure_extension=ghost_pressure_extension,
                                  ghost_velocity_interpolation=ghost_velocity_interpolation)
        self.boundary, self.transport, self.pressure_solver, self.time_scheme = boundary, transport, pressure_solver, time_scheme
        self.verbose = verbose
        self.nx, self.ny, self.Lx, self.Ly = int(nx), int(ny), float(Lx), float(Ly)
        self.dx, self.dy = self.Lx / self.nx, self.Ly / self.ny
        self.D, self.xc, self.yc, self.nu, self.rho, self.U_inf = D, xc, yc, nu, rho, U_inf
        self.inflow, self.slip_walls = inflow, slip_walls
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
        if not self.mask.any() or self.mask[[0, -1], :].any() or self.mask[:, [0, -1]].any():
            raise ValueError('Grid must resolve the cylinder and a fluid layer at every outer boundary')
        t0 = _time.time()
        setup = CutCellSetup(self.nx, self.ny, self.Lx, self.Ly, xc, yc, D / 2.0)
        self._h = self._create(setup, inflow, U_m)
        self.cc = CutCellIntegrator(self._h, self, setup)
        self.cut_geom = setup.geom
        if inflow == 'parabolic':
            y = self.y_centers
            self.u_inlet = 4.0 * self.U_m * y * (self.Ly - y) / (self.Ly ** 2)
        else:
            self.u_inlet = np.full(self.ny, float(U_inf))
        self.u_inlet_base = self.u_inlet.copy()
        self.u = np.empty((self.ny, self.nx + 1))
        self.v = np.empty((self.ny + 1, self.nx))
        self.p = np.empty((self.ny, self.nx))
        self.phi = np.zeros((self.ny, self.nx))
        self.time = 0.0
        self._pull()
        if time_scheme == 'legacy':
            # the legacy loop starts from the unprojected field of solver/main.py:166-177: inlet
            # rows, the faces of covered cells zero, closed faces zero
            g = self.cut_geom
            self.u[:, :] = self.u_inlet[:, None]
            self.v[:, :] = 0.0
            self.p[:, :] = 0.0
            js, is_ = np.nonzero(g.cell_type == -1)
            self.u[js, is_] = 0.0
            self.u[js, is_ + 1] = 0.0
            self.u[g.ax == 0] = 0.0
            self.v[g.ay == 0] = 0.0
            self._push()
        self.time = 0.0
        self.run_options = {}
        self.last_step_diagnostics = {}
        if verbose:
            scheme = 'AB2/CN' if time_scheme == 'ab2_cn' else 'legacy'
            print(f"Cut-cell {scheme} on the GPU ready in {_time.time() - t0:.3f}s (Re={self.Re:.1f}).")

    def _create(self, st, inflow, U_m):
        g = st.geom
        keep = _Keep()
        cfg = _lib.CcConfig()
        cfg.nx, cfg.ny = self.nx, self.ny
        cfg.Lx, cfg.Ly, cfg.D, cfg.xc, cfg.yc = self.Lx, self.Ly, float(self.D), float(self.xc), float(self.yc)
        cfg.nu, cfg.rho, cfg.U_inf = float(self.nu), float(self.rho), float(self.U_inf)
        cfg.inflow = 1 if inflow == 'parabolic' else 0
        cfg.U_m = float(U_m) if U_m is not None else 0.0
        cfg.slip_walls = 1 if self.slip_walls else 0
        for name in ('ax', 'ay', 'ax_mid', 'ay_mid', 'ay_u', 'ax_v', 'volume_fraction', 'u_volume_fraction',
                     'v_volume_fraction'):
            setattr(cfg, name, keep(getattr(g, name)))
        cfg.cell_type = keep(g.cell_type, 'i32')
        cfg.u_vol, cfg.v_vol = keep(st.u_vol), keep(st.v_vol)
        cfg.u_vol_eff, cfg.v_vol_eff = keep(st.u_vol_eff), keep(st.v_vol_eff)
        um = np.array(g.u_merge_list, dtype=np.int64).reshape(-1, 4)
        vm = np.array(g.v_merge_list, dtype=np.int64).reshape(-1, 4)
        cfg.n_u_merge, cfg.n_v_merge = len(um), len(vm)
        cfg.u_merge, cfg.v_merge = keep(um, 'i'), keep(vm, 'i')
        cfg.n_u_covered, cfg.n_v_covered = len(st.u_covered), len(st.v_covered)
        cfg.u_covered, cfg.u_owner = keep(st.u_covered, 'i'), keep(st.u_owner, 'i')
        cfg.v_covered, cfg.v_owner = keep(st.v_covered, 'i'), keep(st.v_owner, 'i')
        w = st.wall
        cfg.n_wall = len(w.ds)
        cfg.wall_rate = keep.csr(w.rate)
        cfg.wall_tx, cfg.wall_ty, cfg.wall_ds = keep(w.tx), keep(w.ty), keep(w.ds)
        cfg.wall_u, cfg.wall_v = keep(w.u_indices, 'i'), keep(w.v_indices, 'i')
        for k, key in enumerate(FAMILIES):
            mf = st.momentum_faces[key]
            fc = cfg.faces[k]
            fc.n_adv, fc.n_adv_points = len(mf.indices), len(mf.patch)
            if np.any(np.diff(mf.patch) < 0):
                raise ValueError('face stencil points must be grouped by face')
            fc.adv_face, fc.adv_patch = keep(mf.indices, 'i'), keep(mf.patch, 'i')
            fc.adv_u, fc.adv_v = keep.csr(mf.u), keep.csr(mf.v)
            fc.adv_len = keep(mf.lengths)
            idx, grad = _viscous_rows(st, key)
            fc.n_dif = len(idx)
            fc.dif_face = keep(idx, 'i')
            fc.dif_grad = keep.csr(grad)
        h = C.c_void_p()
        _check(lib.gm_cc_create(C.byref(cfg), C.byref(h)))
        return h

    def __del__(self):
        h = getattr(self, '_h', None)
        if h:
            lib.gm_cc_destroy(h)
            self._h = None

    def _pull(self):
        _check(lib.gm_cc_get_state(self._h, ptr(self.u), ptr(self.v), ptr(self.p)), self._h)
        if self.time_scheme == 'legacy' and self.time > 0:
            self.phi[...] = self.p  # the legacy loop keeps p = phi (solver/main.py:377-378)

    def _push(self):
        for name in ('u', 'v', 'p'):
            a = getattr(self, name)
            if not (isinstance(a, np.ndarray) and a.dtype == np.float64 and a.flags['C_CONTIGUOUS']):
                setattr(self, name, np.ascontiguousarray(a, dtype=np.float64))
        _check(lib.gm_cc_set_state(self._h, ptr(self.u), ptr(self.v), ptr(self.p)), self._h)

    def _set_inlet(self):
        self.u_inlet = np.ascontiguousarray(self.u_inlet, dtype=np.float64)
        _check(lib.gm_cc_set_inlet(self._h, ptr(self.u_inlet)), self._h)

    def _diag_dict(self, d):
        if self.time_scheme == 'legacy':
            # solve_pressure's record (solver/cut_cell_solver.py:723-728); the inverse is direct,
            # so no Krylov iterations
            pd = dict(residual_linf=d.pressure_residual_linf, residual_l2=d.pressure_residual_l2, iterations=0,
                      predicted_divergence=d.predicted_divergence, seconds=0.0)
            if self.pressure_solver == 'cg_dct':
                pd['preconditioner'] = dict(self.cc.pressure_inverse_info)
            self.cc.last_pressure_diagnostics = dict(pd)
            return dict(pd, time=d.time, dt=d.dt, max_divergence=d.max_divergence, cfl=d.cfl, cd=d.cd, cl=d.cl,
                        cd_pressure=d.cd_pressure, cd_viscous=d.cd_viscous, cl_pressure=d.cl_pressure,
                        cl_viscous=d.cl_viscous)
        pd = dict(residual_linf=float('nan'), residual_l2=float('nan'), iterations=0,
                  predicted_divergence=d.predicted_divergence, seconds=0.0,
                  preconditioner=dict(self.cc.pressure_inverse_info),
                  pressure_solves=int(d.pressure_solves), momentum_iterations=int(d.momentum_iterations),
                  momentum_residual_linf=d.momentum_residual_linf,
                  coupled_momentum_residual_linf=d.coupled_momentum_residual_linf)
        self.cc.last_pressure_diagnostics = dict(pd)
        return dict(pd, time=d.time, dt=d.dt, max_divergence=d.max_divergence, cfl=d.cfl, cd=d.cd, cl=d.cl,
                    cd_pressure=d.cd_pressure, cd_viscous=d.cd_viscous, cl_pressure=d.cl_pressure,
                    cl_viscous=d.cl_viscous)

    def step_raw(self, dt, n_steps, start_time=None):
        """n_steps on the device state without host transfers; (status, diag records)."""
        diag = (_lib.CcStepDiag * n_steps)()
        t = self.time if start_time is None else start_time
        if self.time_scheme == 'legacy':
            rc = lib.gm_cc_legacy_step(self._h, float(dt), int(n_steps), float(t),
                                       1 if self.transport == 'centered' else 0, diag)
        else:
            rc = lib.gm_cc_step(self._h, float(dt), int(n_steps), float(t), diag)
        return rc, diag

    def solve(self, n_steps=25000, dt=0.002, perturb_transient=True, perturb_duration=None, perturb_amp=0.15,
              save_artifacts=True, verbose=None, step_callback=None):
        """Step loop of solver/main.py:245-501 for the cut-cell path."""
        if isinstance(n_steps, bool) or not isinstance(n_steps, (int, np.integer)) or n_steps <= 0:
            raise ValueError('n_steps must be a positive integer')
        if not np.isfinite(dt) or dt <= 0:
            raise ValueError('dt must be finite and positive')
        if perturb_duration is None:
            perturb_duration = 2.5 * (self.D / self.U_ref)
        if not np.isfinite(perturb_duration) or perturb_duration <= 0 or not np.isfinite(perturb_amp) or \
                abs(perturb_amp) >= 1:
            raise ValueError('Require perturb_duration > 0 and finite |perturb_amp| < 1')
        self.run_options = dict(perturb_transient=perturb_transient, perturb_duration=perturb_duration,
                                perturb_amp=perturb_amp)
        verbose = self.verbose if verbose is None else verbose
        self._push()
        t0 = _time.time()
        start = self.time
        ts, cds, cls = [], [], []
        s = 0
        while s < n_steps:
            now_t = start + (s + 1) * dt
            if s % 100 == 0:
                # explicit advection (and, legacy, diffusion) screen of solver/main.py:273-278
                self._pull()
                legacy = self.time_scheme == 'legacy'
                rate = (np.max(np.abs(self.u)) / self.dx + np.max(np.abs(self.v)) / self.dy
                        + (2 * self.nu * (self.dx ** -2 + self.dy ** -2) if legacy else 0.))
                if not np.isfinite(rate) or dt * rate > (1. if legacy else .5):
                    raise RuntimeError(f'Explicit timestep unsafe at t={self.time:g}: dt*rate={dt * rate:g}; reduce dt')
            perturbing = perturb_transient and self.inflow == 'uniform' and now_t <= perturb_duration
            if perturbing:
                decay = 1.0 - (now_t / perturb_duration)
                pert = perturb_amp * np.sin(2.0 * np.pi * self.y_centers / self.Ly) * decay
                self.u_inlet[:] = self.u_inlet_base * (1.0 + pert)
                chunk = 1
            else:
                self.u_inlet[:] = self.u_inlet_base
                chunk = 1 if step_callback is not None else min(n_steps - s, 100 - s % 100)
                if verbose:
                    chunk = min(chunk, 1001 - s % 1000 if s % 1000 else 1)
            self._set_inlet()
            rc, diag = self.step_raw(dt, chunk, start_time=start + s * dt)
            done = chunk
            if rc != _lib.GM_OK:
                done = min(chunk, next((k for k in range(chunk) if diag[k].status), chunk) + 1)
            for k in range(done):
                d = diag[k]
                self.time = d.time
                self.last_step_diagnostics = self._diag_dict(d)
                ts.append(d.time)
                cds.append(d.cd)
                cls.append(d.cl)
            if rc != _lib.GM_OK:
                self._pull()
                _check(rc, self._h)
            s += chunk
            if step_callback is not None or verbose:
                self._pull()
            if step_callback is not None:
                step_callback(self, dict(self.last_step_diagnostics))
            if verbose and ((s - 1) % 1000 == 0 or s == n_steps):
                max_div, div_all, _ = self.cc.divergence_stats()
                flux_in, flux_out = np.sum(self.u[:, 0]) * self.dy, np.sum(self.u[:, self.nx]) * self.dy
                print(f"Step {s - 1:5d} | Div_RMS: {div_all:.2e} | Div_Max: {max_div:.2e} | "
                      f"FluxErr: {abs(flux_out - flux_in) / flux_in:.2e} | "
                      f"Cd: {self.last_step_diagnostics['cd']:.4f} | Cl: {self.last_step_diagnostics['cl']:.4f}")
        self._pull()
        if verbose:
            elapsed = _time.time() - t0
            print(f"Simulation completed in {elapsed:.2f}s ({elapsed / n_steps * 1000:.2f} ms/step)")
        return np.array(ts), np.array(cds), np.array(cls)

    def divergence_stats(self):
        """(max |div|, rms div, max |net flux|) of the state (calculate_cut_cell_divergence)."""
        return self.cc.divergence_stats()

    # -- checkpoints (schema 1, solver/main.py:503-567)
    def _source_hashes(self):
        files = ['cutcell.py', 'cutcell_geometry.py', '_lib.py', 'csrc/cutcell.cu', 'csrc/ghostmac.cu',
                 'csrc/kernels.cu', 'csrc/kernels.cuh', 'csrc/transforms.cuh', 'csrc/geometry.cpp',
                 'csrc/geometry.hpp', 'csrc/internal.hpp']
        return {name: hashlib.sha256((_PKG / name).read_bytes()).hexdigest() for name in files}

    def metadata(self, dt, n_steps, perturb_transient=True, perturb_duration=None, perturb_amp=.15):
        if perturb_duration is None:
            perturb_duration = 2.5 * self.D / self.U_ref
        return dict(nx=self.nx, ny=self.ny, Lx=self.Lx, Ly=self.Ly, D=self.D, xc=self.xc, yc=self.yc, nu=self.nu,
                    rho=self.rho, U_ref=self.U_ref, U_inf=self.U_inf, U_m=self.U_m, inflow=self.inflow,
                    slip_walls=self.slip_walls, dt=dt, n_steps=n_steps, end_time=self.time, boundary=self.boundary,
                    transport=self.transport,
                    time_integrator=('AB2_CN_discrete_incremental' if self.time_scheme == 'ab2_cn'
                                     else 'AB2' if self.transport == 'centered' else 'Euler'),
                    time_scheme=self.time_scheme, pressure_solver=self.pressure_solver,
                    pressure_backend='cut_cell_fft_boundary_schur',
                    pressure_preconditioner=self.cc.pressure_inverse_info, perturb_transient=perturb_transient,
                    perturb_duration=perturb_duration, perturb_amp=perturb_amp, source_sha256=self._source_hashes())

    def legacy_history(self):
        """(prev_au, prev_av, prev_dt) of the legacy predictor, or (None, None, None)."""
        has = C.c_int32()
        dtp = C.c_double()
        buf = np.empty(self.u.size + self.v.size)
        _check(lib.gm_cc_get_legacy_history(self._h, C.byref(has), ptr(buf), C.byref(dtp)), self._h)
        if not has.value:
            return None, None, None
        return (buf[:self.u.size].reshape(self.u.shape).copy(), buf[self.u.size:].reshape(self.v.shape).copy(),
                float(dtp.value))

    def set_legacy_history(self, prev_au, prev_av, prev_dt):
        if prev_au is None:
            _check(lib.gm_cc_set_legacy_history(self._h, 0, None, 0.0), self._h)
            return
        buf = np.r_[_f64(prev_au).ravel(), _f64(prev_av).ravel()]
        _check(lib.gm_cc_set_legacy_history(self._h, 1, ptr(buf), float(prev_dt)), self._h)

    def save_checkpoint(self, path, *, overwrite=False):
        """Atomic schema-1 checkpoint with the cut-cell history (solver/main.py:503-530): the
        state, the inlet, and cn_advection (packed), cn_pressure, cn_dt (AB2/CN) or prev_au,
        prev_av, prev_dt (legacy)."""
        path = Path(path)
        if path.exists() and not overwrite:
            raise FileExistsError(path)
        path.parent.mkdir(parents=True, exist_ok=True)
        arrays = dict(u=self.u, v=self.v, p=self.p, phi=self.phi, u_inlet=self.u_inlet)
        prev_dt = cn_dt = None
        if self.time_scheme == 'legacy':
            au, av, prev_dt = self.legacy_history()
            if au is not None:
                arrays.update(prev_au=au, prev_av=av)
        else:
            adv, half, cn_dt = self.cc.history()
            if adv is not None:
                arrays.update(cn_advection=adv, cn_pressure=half)
        meta = dict(schema=1, configuration=self.configuration, time=self.time, run_options=self.run_options,
                    prev_dt=prev_dt, cn_dt=cn_dt, diagnostics=self.last_step_diagnostics,
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
    def from_checkpoint(cls, path, *, check_sources=True, accept_reference=False):
        """Resume a schema-1 cut-cell checkpoint (solver/main.py:532-567, cut-cell branch); one
        written by the reference's own save_checkpoint is imported when ``accept_reference`` is
        set and rejected as a source mismatch otherwise."""
        with np.load(path, allow_pickle=False) as data:
            meta = json.loads(str(data['checkpoint_metadata']))
            if meta.get('schema') != 1 or meta['configuration'].get('boundary') != 'cut_cell':
                raise ValueError('Unsupported checkpoint')
            sources = meta.get('source_sha256') or {}
            from_reference = 'cut_cell_solver.py' in sources and 'compiled_engine' in sources
            if from_reference and not accept_reference:
                raise ValueError('Checkpoint source mismatch: written by the reference solver '
                                 '(from_checkpoint(..., accept_reference=True) imports it)')
            config = dict(meta['configuration'])
            config['verbose'] = False
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
            for name in ('prev_au', 'prev_av', 'cn_advection', 'cn_pressure'):
                value = data[name].copy() if name in data else None
                if value is not None and not np.isfinite(value).all():
                    raise ValueError(f'Invalid checkpoint history: {name}')
                hist[name] = value
            cn_dt = meta['cn_dt']
            if solver.time_scheme == 'legacy':
                au, av, prev_dt = hist['prev_au'], hist['prev_av'], meta['prev_dt']
                if solver.time > 0 and (au is None or au.shape != solver.u.shape or av is None
                                        or av.shape != solver.v.shape or prev_dt is None
                                        or not np.isfinite(prev_dt) or prev_dt <= 0):
                    raise ValueError('Incomplete predictor checkpoint history')
                solver._push()
                if au is not None and prev_dt is not None:
                    solver.set_legacy_history(au, av, prev_dt)
                return solver
            if solver.time > 0:
                adv, half = hist['cn_advection'], hist['cn_pressure']
                if (adv is None or adv.shape != (solver.cc.qsize,) or half is None or half.shape != solver.p.shape
                        or cn_dt is None or not np.isfinite(cn_dt) or cn_dt <= 0):
                    raise ValueError('Incomplete AB2/CN checkpoint history')
            solver._push()
            if hist['cn_advection'] is not None:
                solver.cc.set_history(hist['cn_advection'], hist['cn_pressure'], cn_dt)
            return solver
