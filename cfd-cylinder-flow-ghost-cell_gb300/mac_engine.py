"""The reference's native module ``mac_engine`` (solver/src/bindings.cpp) on the GPU.

Same function names, arguments, in-place outputs, return values and ValueError messages as the
pybind11 module, so the reference's legacy staircase loop (solver/main.py:303-381) can import
this instead.  Arrays are numpy (C order, float64; the mask bool) or CUDA torch tensors; the
library stages host arrays through the device itself.  predictor_rhs_cpp and corrector_cpp are
bit-identical to the reference's compiled loops; the force and divergence sums are reduced on
the GPU in a fixed order.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import lib, ptr

_MSG_GRID = 'MAC arrays must have matching staggered shapes, C layout, and float64/bool dtype'


def _is_tensor(a):
    return hasattr(a, 'data_ptr')


def _grid(a, rows, cols, boolean=False):
    """check_grid of solver/src/bindings.cpp:10-16."""
    if _is_tensor(a):
        import torch
        ok = (a.dim() == 2 and tuple(a.shape) == (rows, cols) and a.is_contiguous()
              and a.dtype == (torch.bool if boolean else torch.float64))
    else:
        ok = (isinstance(a, np.ndarray) and a.ndim == 2 and a.shape == (rows, cols) and a.flags['C_CONTIGUOUS']
              and a.dtype == (np.bool_ if boolean else np.float64))
    if not ok:
        raise ValueError(_MSG_GRID)


def _fields(u, v, mask, dx, dy):
    """check_fields of solver/src/bindings.cpp:18-27; returns (ny, nx)."""
    shape = tuple(mask.shape)
    if len(shape) != 2 or shape[0] < 2 or shape[1] < 2:
        raise ValueError('mask must be a 2D grid with at least 2 cells per direction')
    ny, nx = shape
    _grid(mask, ny, nx, True)
    _grid(u, ny, nx + 1)
    _grid(v, ny + 1, nx)
    if not (np.isfinite(dx) and dx > 0 and np.isfinite(dy) and dy > 0):
        raise ValueError('dx and dy must be finite and positive')
    return ny, nx


def _step(inlet, ny, dt, rho):
    """check_step of solver/src/bindings.cpp:29-35."""
    if _is_tensor(inlet):
        import torch
        ok = inlet.dim() == 1 and inlet.shape[0] == ny and inlet.is_contiguous() and inlet.dtype == torch.float64
    else:
        ok = (isinstance(inlet, np.ndarray) and inlet.ndim == 1 and inlet.shape[0] == ny
              and inlet.flags['C_CONTIGUOUS'] and inlet.dtype == np.float64)
    if not ok:
        raise ValueError('inlet must be a contiguous float64 vector of length ny')
    if not (np.isfinite(dt) and dt > 0 and np.isfinite(rho) and rho > 0):
        raise ValueError('dt and rho must be finite and positive')


def _mask_ptr(mask):
    return mask.data_ptr() if _is_tensor(mask) else mask.ctypes.data


def _check(rc):
    if rc != _lib.GM_OK:
        raise _lib.error_for(rc, lib.gm_last_error(None).decode(errors='replace'))


def predictor_rhs_cpp(u, v, u_star, v_star, rhs, p, mask, inlet, dx, dy, dt, nu, rho, slip_walls, centered=False):
    """u*, v* and rho/dt div u* in place (solver/src/bindings.cpp:47-216)."""
    ny, nx = _fields(u, v, mask, dx, dy)
    _grid(u_star, ny, nx + 1)
    _grid(v_star, ny + 1, nx)
    _grid(rhs, ny, nx)
    _grid(p, ny, nx)
    _step(inlet, ny, dt, rho)
    if not (np.isfinite(nu) and nu >= 0):
        raise ValueError('nu must be finite and nonnegative')
    _check(lib.gm_mac_predictor_rhs(ptr(u), ptr(v), ptr(u_star), ptr(v_star), ptr(rhs), ptr(p), _mask_ptr(mask),
                                    ptr(inlet), nx, ny, float(dx), float(dy), float(dt), float(nu), float(rho),
                                    1 if slip_walls else 0, 1 if centered else 0, None))


def corrector_cpp(u, v, u_star, v_star, phi, mask, inlet, dx, dy, dt, rho, slip_walls):
    """u = u* - dt/rho grad phi in place, exact Dirichlet outlet (solver/src/bindings.cpp:218-282)."""
    ny, nx = _fields(u, v, mask, dx, dy)
    _grid(u_star, ny, nx + 1)
    _grid(v_star, ny + 1, nx)
    _grid(phi, ny, nx)
    _step(inlet, ny, dt, rho)
    _check(lib.gm_mac_corrector(ptr(u), ptr(v), ptr(u_star), ptr(v_star), ptr(phi), _mask_ptr(mask), ptr(inlet),
                                nx, ny, float(dx), float(dy), float(dt), float(rho), 1 if slip_walls else 0, None))


def calculate_mac_forces_cpp(u, v, p, mask, dx, dy, mu):
    """(fx_p, fy_p, fx_v, fy_v) of the staircase solid cells (solver/src/bindings.cpp:284-341)."""
    ny, nx = _fields(u, v, mask, dx, dy)
    _grid(p, ny, nx)
    if not (np.isfinite(mu) and mu >= 0):
        raise ValueError('mu must be finite and nonnegative')
    out = np.empty(4)
    _check(lib.gm_mac_forces(ptr(u), ptr(v), ptr(p), _mask_ptr(mask), nx, ny, float(dx), float(dy), float(mu),
                             out.ctypes.data, None))
    return tuple(float(x) for x in out)


def calculate_mac_divergence_cpp(u, v, mask, dx, dy):
    """(max |div|, sum div^2, count, core sum div^2, core count) over the fluid cells
    (solver/src/bindings.cpp:343-390)."""
    ny, nx = _fields(u, v, mask, dx, dy)
    out = np.empty(3)
    counts = np.empty(2, np.int64)
    _check(lib.gm_mac_divergence(ptr(u), ptr(v), _mask_ptr(mask), nx, ny, float(dx), float(dy), out.ctypes.data,
                                 counts.ctypes.data, None))
    return float(out[0]), float(out[1]), int(counts[0]), float(out[2]), int(counts[1])
