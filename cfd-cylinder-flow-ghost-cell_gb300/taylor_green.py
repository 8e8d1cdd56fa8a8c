"""Periodic Taylor-Green verification on the GPU (verification/taylor_green.py:14-59).

``run(n, dt, end_time, nu)`` has the reference's signature and return value: the AB2/CN
step from the analytic field at t = 0 to end_time, then the L1/L2/Linf errors of velocity
and (mean-free) pressure against the analytic solution and the largest divergence of any
step.  ``precision='fp32'`` runs the stencils and Fourier solves in FP32 with both solves
refined against the FP64 operators.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import lib, ptr


def exact(n, nu, t):
    """Analytic velocity (u then v) and pressure on the staggered grid at time t
    (verification/taylor_green.py:21-29)."""
    h = 2 * np.pi / n
    yu, xu = np.meshgrid((np.arange(n) + .5) * h, np.arange(n) * h, indexing='ij')
    yv, xv = np.meshgrid(np.arange(n) * h, (np.arange(n) + .5) * h, indexing='ij')
    yp, xp = np.meshgrid((np.arange(n) + .5) * h, (np.arange(n) + .5) * h, indexing='ij')
    a = np.exp(-2 * nu * t)
    q = np.r_[(a * np.sin(xu) * np.cos(yu)).ravel(), (-a * np.cos(xv) * np.sin(yv)).ravel()]
    return q, .25 * a * a * (np.cos(2 * xp) + np.cos(2 * yp))


class TaylorGreen:
    """Device state of one periodic Taylor-Green case (C ABI ``gm_tg_*``)."""

    def __init__(self, n, nu, precision='fp64'):
        if precision not in ('fp64', 'fp32'):
            raise ValueError("precision must be 'fp64' or 'fp32'")
        h = C.c_void_p()
        rc = lib.gm_tg_create(int(n), float(nu), 0 if precision == 'fp64' else 1, C.byref(h))
        if rc != _lib.GM_OK:
            raise _lib.error_for(rc, lib.gm_tg_last_error(None).decode(errors='replace'))
        self._t, self.n, self.nu = h, int(n), float(nu)

    def _check(self, rc):
        if rc != _lib.GM_OK:
            raise _lib.error_for(rc, lib.gm_tg_last_error(self._t).decode(errors='replace'))

    def close(self):
        if getattr(self, '_t', None):
            lib.gm_tg_destroy(self._t)
            self._t = None

    def __del__(self):
        self.close()

    def set_state(self, q, p):
        q = np.ascontiguousarray(q, dtype=np.float64)
        p = np.ascontiguousarray(p, dtype=np.float64)
        if q.size != 2 * self.n * self.n or p.size != self.n * self.n:
            raise ValueError('state sizes do not match the grid')
        self._check(lib.gm_tg_set_state(self._t, ptr(q), ptr(p)))

    def state(self):
        q = np.empty(2 * self.n * self.n)
        half = np.empty((self.n, self.n))
        out = np.empty((self.n, self.n))
        self._check(lib.gm_tg_get_state(self._t, ptr(q), ptr(half), ptr(out)))
        return q, half, out

    def step(self, dt, n_steps):
        md = C.c_double(0.0)
        self._check(lib.gm_tg_step(self._t, float(dt), int(n_steps), C.byref(md)))
        return md.value


def run(n, dt, end_time=.4, nu=.1, precision='fp64'):
    """verification/taylor_green.py:14-59 on the GPU; returns (info, q, pressure - mean)."""
    if n < 8 or not np.isfinite([dt, end_time, nu]).all() or min(dt, end_time, nu) <= 0:
        raise ValueError('Require n>=8 and finite positive dt, end_time and nu')
    steps = round(end_time / dt)
    if steps < 1 or not np.isclose(steps * dt, end_time):
        raise ValueError('end_time must be an integer multiple of dt')
    case = TaylorGreen(n, nu, precision)
    q0, p0 = exact(n, nu, 0.0)
    case.set_state(q0, p0)
    max_divergence = case.step(dt, steps)
    q, _, output = case.state()
    case.close()
    q_exact, p_exact = exact(n, nu, end_time)
    p_error = output - output.mean() - p_exact
    norms = lambda a: dict(l1=float(np.mean(abs(a))), l2=float(np.sqrt(np.mean(a * a))), linf=float(np.max(abs(a))))
    return dict(n=n, dt=dt, end_time=end_time, velocity=norms(q - q_exact), pressure=norms(p_error),
                max_divergence=max_divergence), q, output - output.mean()
