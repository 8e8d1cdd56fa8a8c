"""MAC_CylinderFlow(boundary='staircase' | 'ghost_cell', time_scheme='legacy') on the GPU.

The reference's legacy loop (solver/main.py:245-501): the native predictor (predictor_rhs_cpp),
for the ghost-cell branch the image-point ghost velocities of GhostCellBoundary
(solver/ghost_cell.py), the loop's own AB2 step for centred transport and its recomputed
Poisson right-hand side, a pressure solve of the staircase Poisson matrix (build_poisson_matrix,
solver/mac_solver.py:5-87, which the reference factors with a sparse LU or solves by
ILU-GMRES), the native corrector (or the ghost-cell branch's) and the force sums (staircase
sums, or the integral on the true circle).  One library call (gm_poisson_legacy_step) runs a
chunk of steps on the device with one synchronisation per step; the state stays on the device
between calls (torch tensors serve as device buffers), and the host arrays u, v, p are written
back after each solve() call.  The staircase Poisson matrix is the aperture-weighted cut-cell matrix with
open fractions 0 or 1 taken from the cell mask, solved to rounding by the boundary-corrected
separable inverse; both pressure_solver choices of the reference solve that system (the LU
exactly, ILU-GMRES to rtol 1e-8).
"""
from __future__ import annotations

import ctypes as C
import hashlib
import time as _time
from pathlib import Path

import numpy as np

from . import _lib
from ._args import check_reference_arguments
from ._lib import lib, ptr


def _check_mac(rc):
    if rc != _lib.GM_OK:
        raise _lib.error_for(rc, lib.gm_last_error(None).decode(errors='replace'))


class StaircaseFlow:
    """The legacy staircase MAC_CylinderFlow on the GPU (solver/main.py:19-501, boundary='staircase',
    time_scheme='legacy')."""

    _boundary = 'staircase'

    def __init__(self, nx=400, ny=100, Lx=20.0, Ly=5.0, D=1.0, xc=5.0, yc=2.5, nu=0.01, rho=1.0, U_inf=1.0,
                 inflow='uniform', U_m=None, slip_walls=False, verbose=True, boundary=None,
                 transport='centered', pressure_solver='direct', marker_spacing_factor=1.5, time_scheme='legacy',
                 ghost_pressure_extension='neumann', ghost_velocity_interpolation='bilinear', precision='fp64'):
        """Keywords of solver/main.py:40-44; boundary defaults to the class's own."""
        import torch
        boundary = self._boundary if boundary is None else boundary
        check_reference_arguments(boundary, transport, pressure_solver, time_scheme, ghost_pressure_extension,
                                  ghost_velocity_interpolation)
        if boundary != self._boundary or time_scheme != 'legacy':
            raise NotImplementedError(f'{type(self).__name__} implements boundary="{self._boundary}", '
                                      'time_scheme="legacy"')
        if precision != 'fp64':
            raise NotImplementedError('the legacy loop runs in FP64')
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
        # solid mask of solver/main.py:123-129
        rr = (((self.x_centers - xc) / (D / 2.0)) ** 2)[None, :] + (((self.y_centers - yc) / (D / 2.0)) ** 2)[:, None]
        self.mask = rr <= (1.0 + 1e-13)
        if not self.mask.any() or self.mask[[0, -1], :].any() or self.mask[:, [0, -1]].any():
            raise ValueError('Grid must resolve the cylinder and a fluid layer at every outer boundary')
        t0 = _time.time()
        self.u_inlet = np.empty(self.ny)
        for j in range(self.ny):
            y = self.y_centers[j]
            self.u_inlet[j] = 4.0 * self.U_m * y * (self.Ly - y) / (self.Ly ** 2) if inflow == 'parabolic' else self.U_inf
        self.u_inlet_base = self.u_inlet.copy()
        # initial field (solver/main.py:166-177): inlet rows, faces of masked cells zero
        self.u = np.zeros((self.ny, self.nx + 1))
        self.v = np.zeros((self.ny + 1, self.nx))
        self.p = np.zeros((self.ny, self.nx))
        self.phi = np.zeros((self.ny, self.nx))
        self.u[:, :] = self.u_inlet[:, None]
        js, is_ = np.nonzero(self.mask)
        self.u[js, is_] = 0.0
        self.u[js, is_ + 1] = 0.0
        self.v[js, is_] = 0.0
        self.v[js + 1, is_] = 0.0
        # the staircase Poisson system: open fractions 0 on faces next to a masked cell
        m = self.mask
        ax = np.ones((self.ny, self.nx + 1))
        ax[:, 1:-1][m[:, :-1] | m[:, 1:]] = 0.0
        ay = np.ones((self.ny + 1, self.nx))
        ay[1:-1][m[:-1] | m[1:]] = 0.0
        ctype = np.where(m, -1, 1).astype(np.int32)
        kappa = np.where(m, 0.0, 1.0)
        h = C.c_void_p()
        rc = lib.gm_poisson_create(self.nx, self.ny, self.Lx, self.Ly, float(D), float(xc), float(yc), ptr(ax),
                                   ptr(ay), ptr(ctype.view(np.int32)), ptr(kappa), C.byref(h))
        if rc != _lib.GM_OK:
            raise _lib.error_for(rc, lib.gm_poisson_last_error(None).decode(errors='replace'))
        self._poisson = h
        dev = torch.device('cuda')
        f64 = dict(dtype=torch.float64, device=dev)
        self._d = dict(u=torch.empty(self.u.shape, **f64), v=torch.empty(self.v.shape, **f64),
                       p=torch.empty(self.p.shape, **f64), us=torch.zeros(self.u.shape, **f64),
                       vs=torch.zeros(self.v.shape, **f64), rhs=torch.zeros(self.p.shape, **f64),
                       phi=torch.zeros(self.p.shape, **f64), zero_p=torch.zeros(self.p.shape, **f64),
                       pdu=torch.zeros(self.u.shape, **f64), pdv=torch.zeros(self.v.shape, **f64),
                       inlet=torch.empty(self.ny, **f64),
                       mask=torch.from_numpy(np.ascontiguousarray(self.mask, dtype=np.uint8)).to(dev))
        st = _lib.LegacyState()
        st.nx, st.ny, st.dx, st.dy = self.nx, self.ny, self.dx, self.dy
        st.nu, st.rho = float(nu), float(rho)
        st.slip_walls = 1 if slip_walls else 0
        st.centered = 1 if transport == 'centered' else 0
        d = self._d
        for name, key in (('u', 'u'), ('v', 'v'), ('p', 'p'), ('u_star', 'us'), ('v_star', 'vs'), ('rhs', 'rhs'),
                          ('phi', 'phi'), ('prev_du', 'pdu'), ('prev_dv', 'pdv'), ('zero_p', 'zero_p'),
                          ('mask', 'mask'), ('inlet', 'inlet')):
            setattr(st, name, d[key].data_ptr())
        self._st = st
        self.time = 0.0
        self.run_options = {}
        self.last_step_diagnostics = {}
        self._setup_boundary()
        if verbose:
            print(f"{self._boundary} legacy MAC on the GPU ready in {_time.time() - t0:.3f}s (Re={self.Re:.1f}).")

    def _setup_boundary(self):
        """Extra boundary tables of a subclass (none for the staircase)."""

    def __del__(self):
        h = getattr(self, '_poisson', None)
        if h:
            lib.gm_poisson_destroy(h)
            self._poisson = None

    def _stream(self):
        import torch
        return C.c_void_p(torch.cuda.current_stream().cuda_stream)

    def _push(self):
        import torch
        for name, key in (('u', 'u'), ('v', 'v'), ('p', 'p')):
            self._d[key].copy_(torch.from_numpy(np.ascontiguousarray(getattr(self, name), dtype=np.float64)))

    def _pull(self):
        for name, key in (('u', 'u'), ('v', 'v'), ('p', 'p'), ('phi', 'phi')):
            getattr(self, name)[...] = self._d[key].cpu().numpy()

    @property
    def _previous_dt(self):
        """dt of the last centred step (the loop's AB2 history), or None."""
        return self._st.prev_dt if self._st.has_prev else None

    def _steps(self, dt, n):
        """n legacy steps with the current inlet on the device (solver/main.py:303-378), one
        library call: per-step (fx_p, fy_p, fx_v, fy_v) and the pressure residual."""
        diag = (_lib.LegacyStepDiag * n)()
        rc = lib.gm_poisson_legacy_step(self._poisson, C.byref(self._st), float(dt), int(n), diag, self._stream())
        if rc != _lib.GM_OK:
            raise _lib.error_for(rc, lib.gm_poisson_last_error(self._poisson).decode(errors='replace'))
        return [(tuple(d.forces), d.pressure_residual_linf) for d in diag]

    def _source_hashes(self):
        root = Path(__file__).resolve().parent
        files = ['staircase.py', '_lib.py', '_args.py', 'csrc/legacy.cu', 'csrc/cutcell.cu', 'csrc/ghostmac.cu',
                 'csrc/kernels.cu', 'csrc/geometry.cpp', 'csrc/internal.hpp']
        return {name: hashlib.sha256((root / name).read_bytes()).hexdigest() for name in files}

    def metadata(self, dt, n_steps, perturb_transient=True, perturb_duration=None, perturb_amp=.15):
        """The run record of solver/main.py:587-617 for this loop."""
        if perturb_duration is None:
            perturb_duration = 2.5 * self.D / self.U_ref
        return dict(nx=self.nx, ny=self.ny, Lx=self.Lx, Ly=self.Ly, D=self.D, xc=self.xc, yc=self.yc, nu=self.nu,
                    rho=self.rho, U_ref=self.U_ref, U_inf=self.U_inf, U_m=self.U_m, inflow=self.inflow,
                    slip_walls=self.slip_walls, dt=dt, n_steps=n_steps, end_time=self.time, boundary=self.boundary,
                    transport=self.transport, time_integrator='AB2' if self.transport == 'centered' else 'Euler',
                    time_scheme=self.time_scheme, pressure_solver=self.pressure_solver,
                    pressure_backend='staircase_fft_boundary_schur', perturb_transient=perturb_transient,
                    perturb_duration=perturb_duration, perturb_amp=perturb_amp, source_sha256=self._source_hashes())

    def save_checkpoint(self, path, *, overwrite=False):
        """The reference keeps no checkpoint of its legacy staircase and ghost-cell loops
        (solver/main.py:503-506)."""
        raise ValueError('Checkpoints require Cut-Cell or Ghost-Cell AB2/CN')

    def divergence_stats(self):
        """calculate_mac_divergence_cpp of the state: (max |div|, sum div^2, fluid count, core sum
        div^2, core count)."""
        d = self._d
        out = np.empty(3)
        counts = np.empty(2, np.int64)
        _check_mac(lib.gm_mac_divergence(ptr(d['u']), ptr(d['v']), ptr(d['mask']), self.nx, self.ny, self.dx,
                                         self.dy, ptr(out), ptr(counts), self._stream()))
        return out[0], out[1], int(counts[0]), out[2], int(counts[1])

    def solve(self, n_steps=25000, dt=0.002, perturb_transient=True, perturb_duration=None, perturb_amp=0.15,
              save_artifacts=True, verbose=None, step_callback=None):
        """Step loop of solver/main.py:245-501 for the legacy staircase path."""
        import torch
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
        d = self._d
        t0 = _time.time()
        start = self.time
        ts, cds, cls = [], [], []
        denom = 0.5 * self.rho * (self.U_ref ** 2) * self.D
        s = 0
        while s < n_steps:
            now_t = start + (s + 1) * dt
            if s % 100 == 0:
                # explicit advection/diffusion screen (solver/main.py:273-278)
                rate = (float(d['u'].abs().max()) / self.dx + float(d['v'].abs().max()) / self.dy
                        + 2 * self.nu * (self.dx ** -2 + self.dy ** -2))
                if not np.isfinite(rate) or dt * rate > 1.:
                    self._pull()
                    raise RuntimeError(f'Explicit timestep unsafe at t={self.time:g}: dt*rate={dt * rate:g}; reduce dt')
            if perturb_transient and self.inflow == 'uniform' and now_t <= perturb_duration:
                decay = 1.0 - (now_t / perturb_duration)
                pert = perturb_amp * np.sin(2.0 * np.pi * self.y_centers / self.Ly) * decay
                self.u_inlet[:] = self.u_inlet_base * (1.0 + pert)
                chunk = 1
            else:
                self.u_inlet[:] = self.u_inlet_base
                chunk = 1 if step_callback is not None else min(n_steps - s, 100 - s % 100)
                if verbose:
                    chunk = min(chunk, 1001 - s % 1000 if s % 1000 else 1)
            d['inlet'].copy_(torch.from_numpy(self.u_inlet))
            for k, ((fx_p, fy_p, fx_v, fy_v), res) in enumerate(self._steps(dt, chunk)):
                t_k = start + (s + k + 1) * dt
                fx, fy = fx_p + fx_v, fy_p + fy_v
                cd, cl = fx / denom, fy / denom
                if not np.isfinite(cd) or not np.isfinite(cl):
                    self._pull()
                    raise FloatingPointError(f'Non-finite force at t={t_k:g}; results not saved')
                self.time = t_k
                self.last_step_diagnostics = dict(time=self.time, dt=dt, cd=float(cd), cl=float(cl),
                                                  cd_pressure=float(fx_p / denom), cd_viscous=float(fx_v / denom),
                                                  cl_pressure=float(fy_p / denom), cl_viscous=float(fy_v / denom),
                                                  pressure_residual_linf=float(res))
                cds.append(cd)
                cls.append(cl)
                ts.append(t_k)
            s += chunk
            if step_callback is not None:
                self._pull()
                step_callback(self, dict(self.last_step_diagnostics))
            if verbose and ((s - 1) % 1000 == 0 or s == n_steps):
                max_div, sum_div2, count, _, _ = self.divergence_stats()
                div_all = np.sqrt(sum_div2 / count) if count > 0 else 0.0
                self._pull()
                in_flux, out_flux = np.sum(self.u[:, 0]) * self.dy, np.sum(self.u[:, self.nx]) * self.dy
                print(f"Step {s - 1:5d} | Div_RMS: {div_all:.2e} | Div_Max: {max_div:.2e} | "
                      f"FluxErr: {abs(out_flux - in_flux) / in_flux:.2e} | Cd: {cds[-1]:.4f} | Cl: {cls[-1]:.4f}")
        self._pull()
        if verbose:
            elapsed = _time.time() - t0
            print(f"Simulation completed in {elapsed:.2f}s ({elapsed / n_steps * 1000:.2f} ms/step)")
        return np.array(ts), np.array(cds), np.array(cls)


def ghost_face_tables(xs, ys, dx, dy, xc, yc, radius, is_u):
    """Ghost faces of one staggered face grid (coordinates xs, ys) and their image-point stencils,
    as GhostCellBoundary builds them (solver/ghost_cell.py:41-157): the faces inside the circle
    (signed distance < 0) with a face outside it among their four neighbours, in row-major order;
    the image point at distance d + max(d, h/2) along the outward normal, its bilinear cell and
    weights (00, 10, 01, 11), and gamma = d / max(d, h/2).  The same elementwise float64
    arithmetic, vectorised.  Returns dict(target, src (n, 4), weights (n, 4), gamma, snap_of (n, 4),
    level, n_levels) with flat indexes into the face grid.

    The reference sets the faces in order, so a corner that is itself a ghost face is read with
    the value it holds at that moment: new if it comes earlier in the order, its value before the
    pass otherwise (snap_of = its ghost index).  A face's level is one above the highest level of
    the earlier ghost faces it reads, so one launch per level reproduces the sequential pass."""
    X, Y = np.meshgrid(xs, ys)
    dist = np.sqrt((X - xc) ** 2 + (Y - yc) ** 2) - radius
    fluid = dist >= 0.0
    near = np.zeros_like(fluid)
    near[:, 1:] |= fluid[:, :-1]
    near[:, :-1] |= fluid[:, 1:]
    near[1:, :] |= fluid[:-1, :]
    near[:-1, :] |= fluid[1:, :]
    js, is_ = np.nonzero(~fluid & near)
    nyf, nxf = fluid.shape
    xg, yg = xs[is_], ys[js]
    d = np.abs(dist[js, is_])
    delta = np.maximum(d, 0.5 * min(dx, dy))
    r = np.maximum(np.sqrt((xg - xc) ** 2 + (yg - yc) ** 2), 1e-14)
    x_ip = xg + (d + delta) * ((xg - xc) / r)
    y_ip = yg + (d + delta) * ((yg - yc) / r)
    if is_u:
        i0 = np.floor(x_ip / dx).astype(np.int64)
        j0 = np.floor((y_ip - 0.5 * dy) / dy).astype(np.int64)
        x0, y0 = i0 * dx, (j0 + 0.5) * dy
    else:
        i0 = np.floor((x_ip - 0.5 * dx) / dx).astype(np.int64)
        j0 = np.floor(y_ip / dy).astype(np.int64)
        x0, y0 = (i0 + 0.5) * dx, j0 * dy
    i0 = np.clip(i0, 0, nxf - 2)
    j0 = np.clip(j0, 0, nyf - 2)
    rx = np.clip((x_ip - x0) / dx, 0.0, 1.0)
    ry = np.clip((y_ip - y0) / dy, 0.0, 1.0)
    weights = np.stack([(1.0 - rx) * (1.0 - ry), rx * (1.0 - ry), (1.0 - rx) * ry, rx * ry], axis=1)
    base = j0 * nxf + i0
    src = np.stack([base, base + 1, base + nxf, base + nxf + 1], axis=1)
    target = js.astype(np.int64) * nxf + is_
    n = target.size
    order = np.full(nyf * nxf, -1, np.int64)
    order[target] = np.arange(n)
    snap_of = np.full((n, 4), -1, np.int32)
    level = np.zeros(n, np.int32)
    for g in range(n):
        lv = 0
        for q in range(4):
            k = order[src[g, q]]
            if k >= g:
                snap_of[g, q] = k
            elif k >= 0:
                lv = max(lv, int(level[k]) + 1)
        level[g] = lv
    return dict(target=target, src=src, weights=weights, gamma=d / delta, snap_of=snap_of, level=level,
                n_levels=int(level.max()) + 1 if n else 0)


class LegacyGhostFlow(StaircaseFlow):
    """MAC_CylinderFlow(boundary='ghost_cell', time_scheme='legacy') on the GPU: the legacy loop of
    solver/main.py:245-501 with the GhostCellBoundary of solver/ghost_cell.py.  Each step runs the
    native predictor on the staircase mask, sets the image-point ghost velocities on u*, v* (again
    after the loop's AB2 step for centred transport), recomputes the Poisson right-hand side,
    solves the staircase Poisson matrix, applies the ghost branch's own corrector, sets the ghost
    velocities of u, v, restores u* on the faces between fluid and masked cells, and integrates
    the forces on the true circle at 360 points.  Fields are bit-identical to the reference's
    arithmetic except for the pressure solve, which agrees with the reference's sparse LU to
    rounding."""

    _boundary = 'ghost_cell'
    n_theta = 360

    def _setup_boundary(self):
        import torch
        dev = torch.device('cuda')
        xu = np.arange(self.nx + 1) * self.dx
        yu = (np.arange(self.ny) + 0.5) * self.dy
        xv = (np.arange(self.nx) + 0.5) * self.dx
        yv = np.arange(self.ny + 1) * self.dy
        self._ghost = {}
        st = self._st
        st.ghost = 1
        st.xc, st.yc, st.radius, st.n_theta = float(self.xc), float(self.yc), float(self.D / 2.0), self.n_theta
        for k, (key, xs, ys, is_u) in enumerate((('u', xu, yu, True), ('v', xv, yv, False))):
            t = ghost_face_tables(xs, ys, self.dx, self.dy, self.xc, self.yc, self.D / 2.0, is_u)
            dt = {name: torch.from_numpy(np.ascontiguousarray(t[name])).to(dev)
                  for name in ('target', 'src', 'weights', 'gamma', 'snap_of', 'level')}
            dt['n'], dt['n_levels'] = int(t['target'].size), t['n_levels']
            self._ghost[key] = dt
            st.n_ghost[k], st.n_levels[k] = dt['n'], dt['n_levels']
            for name in ('target', 'src', 'snap_of', 'weights', 'gamma', 'level'):
                getattr(st, name)[k] = dt[name].data_ptr()

    def ghost_counts(self):
        """Numbers of ghost u and v faces and of launch levels of each."""
        return {k: (t['n'], t['n_levels']) for k, t in self._ghost.items()}
