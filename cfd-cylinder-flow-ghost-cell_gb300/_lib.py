"""ctypes binding of libghostmac.so (declarations in include/ghostmac.h).

The library is loaded from this package directory.  There is no fallback:
if it is missing or cannot be loaded the import fails loudly.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / 'libghostmac.so'

GM_OK, GM_EVALUE, GM_ERUNTIME, GM_EFLOAT, GM_ECUDA, GM_ENOTIMPL = range(6)
OP_PACK, OP_UNPACK, OP_ADVECTION, OP_DIFFUSION, OP_GRADIENT, OP_DIVERGENCE, OP_H_MATVEC, OP_PRESSURE_EXTEND = range(1, 9)
GATE_NAMES = {1: 'projection', 2: 'momentum', 3: 'pressure', 4: 'pressure_rhs', 5: 'step', 6: 'force',
              7: 'cfl_screen', 8: 'finite'}

SYMBOLS = ('gm_create', 'gm_create_host', 'gm_prepare_dt', 'gm_destroy', 'gm_last_error', 'gm_get_sizes',
           'gm_set_stream', 'gm_get_indices', 'gm_get_ghost_stencils', 'gm_get_schur_rows',
           'gm_get_surface_points', 'gm_set_state', 'gm_get_state', 'gm_set_inlet', 'gm_set_history',
           'gm_get_history', 'gm_step', 'gm_solve_io', 'gm_apply', 'gm_project', 'gm_pressure_solve', 'gm_rectangle_solve',
           'gm_surface_forces', 'gm_divergence_stats', 'gm_kernel_launches', 'gm_kernel_timing',
           'gm_divergence_stats_noalloc', 'gm_batch_create', 'gm_batch_destroy', 'gm_batch_last_error',
           'gm_batch_step', 'gm_phase_timing', 'gm_tg_create', 'gm_tg_destroy', 'gm_tg_last_error',
           'gm_tg_set_state', 'gm_tg_get_state', 'gm_tg_step', 'gm_unet_layers', 'gm_unet_create',
           'gm_unet_destroy', 'gm_unet_last_error', 'gm_unet_input', 'gm_unet_forward', 'gm_unet_backward',
           'gm_set_learned_preconditioner', 'gm_set_pressure_recorder', 'gm_pressure_recorded',
           'gm_host_alloc', 'gm_host_free', 'gm_solver_info', 'gm_pressure_reconstruction',
           'gm_mac_predictor_rhs', 'gm_mac_corrector', 'gm_mac_forces', 'gm_mac_divergence',
           'gm_pod_create', 'gm_pod_destroy', 'gm_pod_last_error', 'gm_pod_gram', 'gm_pod_modes', 'gm_batch_shapes',
           'gm_cc_create', 'gm_cc_destroy', 'gm_cc_last_error', 'gm_cc_get_sizes', 'gm_cc_get_indices',
           'gm_cc_get_surface_points', 'gm_cc_set_state', 'gm_cc_get_state', 'gm_cc_set_inlet',
           'gm_cc_set_history', 'gm_cc_get_history', 'gm_cc_step', 'gm_cc_apply', 'gm_cc_surface_forces',
           'gm_cc_divergence_stats', 'gm_cc_phase_timing', 'gm_cc_legacy_step', 'gm_cc_set_legacy_history',
           'gm_cc_get_legacy_history', 'gm_mac_ab2_rhs', 'gm_mac_ghost_apply',
           'gm_mac_ghost_correct', 'gm_mac_ghost_forces', 'gm_poisson_create',
           'gm_poisson_destroy', 'gm_poisson_last_error', 'gm_poisson_solve',
           'gm_poisson_legacy_step')
CC_OP_MOMENTUM_ADVECTION, CC_OP_MOMENTUM_DIFFUSION, CC_OP_ADVECTION, CC_OP_DIFFUSION, CC_OP_H_MATVEC, CC_OP_PROJECT, \
    CC_OP_PRESSURE_SOLVE, CC_OP_MOMENTUM_ADVECTION_UPWIND = range(1, 9)
MAC_AB2, MAC_RHS = 1, 2
NOALLOC_MAX_CELLS = 1048576


class Config(C.Structure):
    _fields_ = [('nx', C.c_int32), ('ny', C.c_int32), ('Lx', C.c_double), ('Ly', C.c_double), ('D', C.c_double),
                ('xc', C.c_double), ('yc', C.c_double), ('nu', C.c_double), ('rho', C.c_double),
                ('U_inf', C.c_double), ('inflow', C.c_int32), ('U_m', C.c_double),
                ('pressure_solver', C.c_int32), ('pressure_extension', C.c_int32),
                ('velocity_interpolation', C.c_int32), ('precision', C.c_int32)]


class Sizes(C.Structure):
    _fields_ = [(n, C.c_int64) for n in ('nx', 'ny', 'usize', 'vsize', 'psize', 'nu_active', 'nv_active',
                                         'np_active', 'qsize', 'n_surface', 'rank_p', 'rank_u', 'rank_v',
                                         'ghost_u', 'ghost_v', 'ghost_p')] + \
               [('dx', C.c_double), ('dy', C.c_double), ('U_ref', C.c_double)]


class StepDiag(C.Structure):
    _fields_ = [(n, C.c_double) for n in ('time', 'dt', 'max_divergence', 'cfl', 'cd', 'cl', 'cd_pressure',
                                          'cd_viscous', 'cl_pressure', 'cl_viscous', 'momentum_residual_linf',
                                          'coupled_momentum_residual_linf', 'pressure_residual_linf',
                                          'pressure_residual_relative_l2')] + \
               [('forces', C.c_double * 6)] + \
               [(n, C.c_int32) for n in ('pressure_solve_count', 'pressure_iterations',
                                         'pressure_refinement_iterations', 'momentum_refinement_iterations',
                                         'status', 'gate')]


class SolveInfo(C.Structure):
    _fields_ = [(n, C.c_double) for n in ('residual_linf', 'residual_relative_l2', 'residual_target_linf',
                                          'roundoff_bound_linf', 'backward_error_linf')] + \
               [(n, C.c_int32) for n in ('iterations', 'refinement_iterations', 'status', 'rank')]


class Csr(C.Structure):
    _fields_ = [('ptr', C.c_void_p), ('col', C.c_void_p), ('val', C.c_void_p)]


class CcFaces(C.Structure):
    _fields_ = [('n_adv', C.c_int64), ('n_adv_points', C.c_int64), ('adv_face', C.c_void_p),
                ('adv_patch', C.c_void_p), ('adv_u', Csr), ('adv_v', Csr), ('adv_len', C.c_void_p),
                ('n_dif', C.c_int64), ('dif_face', C.c_void_p), ('dif_grad', Csr)]


class CcConfig(C.Structure):
    _fields_ = [('nx', C.c_int32), ('ny', C.c_int32)] + \
               [(n, C.c_double) for n in ('Lx', 'Ly', 'D', 'xc', 'yc', 'nu', 'rho', 'U_inf')] + \
               [('inflow', C.c_int32), ('U_m', C.c_double), ('slip_walls', C.c_int32)] + \
               [(n, C.c_void_p) for n in ('ax', 'ay', 'ax_mid', 'ay_mid', 'ay_u', 'ax_v', 'cell_type',
                                          'volume_fraction', 'u_volume_fraction', 'v_volume_fraction', 'u_vol',
                                          'v_vol', 'u_vol_eff', 'v_vol_eff')] + \
               [('n_u_merge', C.c_int64), ('n_v_merge', C.c_int64), ('u_merge', C.c_void_p), ('v_merge', C.c_void_p),
                ('n_u_covered', C.c_int64), ('n_v_covered', C.c_int64)] + \
               [(n, C.c_void_p) for n in ('u_covered', 'u_owner', 'v_covered', 'v_owner')] + \
               [('n_wall', C.c_int64), ('wall_rate', Csr)] + \
               [(n, C.c_void_p) for n in ('wall_tx', 'wall_ty', 'wall_ds', 'wall_u', 'wall_v')] + \
               [('faces', CcFaces * 4)]


class CcStepDiag(C.Structure):
    _fields_ = [(n, C.c_double) for n in ('time', 'dt', 'max_divergence', 'cfl', 'cd', 'cl', 'cd_pressure',
                                          'cd_viscous', 'cl_pressure', 'cl_viscous', 'momentum_residual_linf',
                                          'coupled_momentum_residual_linf', 'predicted_divergence')] + \
               [('forces', C.c_double * 6)] + \
               [(n, C.c_int32) for n in ('momentum_iterations', 'pressure_solves', 'status', 'gate')] + \
               [(n, C.c_double) for n in ('pressure_residual_linf', 'pressure_residual_l2')]


class LegacyState(C.Structure):
    _fields_ = [('nx', C.c_int32), ('ny', C.c_int32), ('dx', C.c_double), ('dy', C.c_double), ('nu', C.c_double),
                ('rho', C.c_double), ('slip_walls', C.c_int32), ('centered', C.c_int32), ('ghost', C.c_int32)] + \
               [(n, C.c_void_p) for n in ('u', 'v', 'p', 'u_star', 'v_star', 'rhs', 'phi', 'prev_du', 'prev_dv',
                                          'zero_p', 'mask', 'inlet')] + \
               [('n_ghost', C.c_int64 * 2)] + \
               [(n, C.c_void_p * 2) for n in ('target', 'src', 'snap_of', 'weights', 'gamma', 'level')] + \
               [('n_levels', C.c_int32 * 2), ('xc', C.c_double), ('yc', C.c_double), ('radius', C.c_double),
                ('n_theta', C.c_int32), ('has_prev', C.c_int32), ('prev_dt', C.c_double)]


class LegacyStepDiag(C.Structure):
    _fields_ = [('forces', C.c_double * 4), ('pressure_residual_linf', C.c_double)]


def _load():
    if not LIB_PATH.exists():
        raise ImportError(f'{LIB_PATH} is missing: build it with cfd-cylinder-flow-ghost-cell_gb300/build.py')
    lib = C.CDLL(str(LIB_PATH))
    P, I32, I64, D = C.c_void_p, C.c_int32, C.c_int64, C.c_double
    pp = C.POINTER(C.c_void_p)
    sig = {
        'gm_create': ([C.POINTER(Config), pp], C.c_int),
        'gm_create_host': ([C.POINTER(Config), pp], C.c_int),
        'gm_prepare_dt': ([P, D], C.c_int),
        'gm_destroy': ([P], C.c_int),
        'gm_last_error': ([P], C.c_char_p),
        'gm_get_sizes': ([P, C.POINTER(Sizes)], C.c_int),
        'gm_set_stream': ([P, P], C.c_int),
        'gm_get_indices': ([P, P, P, P], C.c_int),
        'gm_get_ghost_stencils': ([P, I32, C.POINTER(I64), C.POINTER(I64), P, P, P, P], C.c_int),
        'gm_get_schur_rows': ([P, I32, C.POINTER(I64), P], C.c_int),
        'gm_get_surface_points': ([P, P], C.c_int),
        'gm_pressure_reconstruction': ([P, P, I32, C.POINTER(I64), P, P, P], C.c_int),
        'gm_mac_predictor_rhs': ([P, P, P, P, P, P, P, P, I32, I32, D, D, D, D, D, I32, I32, P], C.c_int),
        'gm_mac_corrector': ([P, P, P, P, P, P, P, I32, I32, D, D, D, D, I32, P], C.c_int),
        'gm_mac_forces': ([P, P, P, P, I32, I32, D, D, D, P, P], C.c_int),
        'gm_mac_divergence': ([P, P, P, I32, I32, D, D, P, P, P], C.c_int),
        'gm_pod_create': ([I32, I64, P], C.c_int),
        'gm_batch_shapes': ([P, P, P, I32], C.c_int),
        'gm_pod_destroy': ([P], C.c_int),
        'gm_pod_last_error': ([P], C.c_char_p),
        'gm_pod_gram': ([P, P, P, P, P], C.c_int),
        'gm_pod_modes': ([P, P, P, I32, P, P, P], C.c_int),
        'gm_set_state': ([P, P, P, P], C.c_int),
        'gm_get_state': ([P, P, P, P], C.c_int),
        'gm_set_inlet': ([P, P], C.c_int),
        'gm_set_history': ([P, I32, P, P, D], C.c_int),
        'gm_get_history': ([P, C.POINTER(I32), P, P, C.POINTER(D)], C.c_int),
        'gm_step': ([P, D, I32, I64, D, C.POINTER(StepDiag)], C.c_int),
        'gm_solve_io': ([P, P, P, P, P, D, I32, I64, D, C.POINTER(StepDiag), P, P, P], C.c_int),
        'gm_apply': ([P, I32, D, P, P], C.c_int),
        'gm_project': ([P, D, P, P, P, C.POINTER(SolveInfo)], C.c_int),
        'gm_pressure_solve': ([P, P, P, C.POINTER(SolveInfo)], C.c_int),
        'gm_rectangle_solve': ([P, I32, D, P, P], C.c_int),
        'gm_surface_forces': ([P, P, P, P, D, P], C.c_int),
        'gm_divergence_stats': ([P, P, P, P, P], C.c_int),
        'gm_kernel_launches': ([], I64),
        'gm_kernel_timing': ([I32, I32, C.POINTER(D), C.POINTER(I64), C.POINTER(D)], C.c_int),
        'gm_divergence_stats_noalloc': ([P, P, P, I32, I32, D, D, P, P, P], C.c_int),
        'gm_batch_create': ([C.POINTER(C.c_void_p), I32, pp], C.c_int),
        'gm_batch_destroy': ([P], C.c_int),
        'gm_batch_last_error': ([P], C.c_char_p),
        'gm_batch_step': ([P, D, I32, I64, P, C.POINTER(StepDiag), P], C.c_int),
        'gm_phase_timing': ([P, P], C.c_int),
        'gm_solver_info': ([P, C.POINTER(I32), C.POINTER(D)], C.c_int),
        'gm_tg_create': ([I32, D, I32, pp], C.c_int),
        'gm_tg_destroy': ([P], C.c_int),
        'gm_tg_last_error': ([P], C.c_char_p),
        'gm_tg_set_state': ([P, P, P], C.c_int),
        'gm_tg_get_state': ([P, P, P, P], C.c_int),
        'gm_tg_step': ([P, D, I32, C.POINTER(D)], C.c_int),
        'gm_unet_layers': ([P, P, P], C.c_int),
        'gm_unet_create': ([I32, I32, I32, pp], C.c_int),
        'gm_unet_destroy': ([P], C.c_int),
        'gm_unet_last_error': ([P], C.c_char_p),
        'gm_unet_input': ([P, P], C.c_int),
        'gm_unet_forward': ([P, P, P, P, P, P], C.c_int),
        'gm_unet_backward': ([P, P, P, P, P, P], C.c_int),
        'gm_set_learned_preconditioner': ([P, P, P, P], C.c_int),
        'gm_set_pressure_recorder': ([P, P, P, I32], C.c_int),
        'gm_pressure_recorded': ([P], I32),
        'gm_host_alloc': ([C.c_size_t, pp], C.c_int),
        'gm_host_free': ([P], C.c_int),
        'gm_cc_create': ([C.POINTER(CcConfig), pp], C.c_int),
        'gm_cc_destroy': ([P], C.c_int),
        'gm_cc_last_error': ([P], C.c_char_p),
        'gm_cc_get_sizes': ([P, C.POINTER(Sizes)], C.c_int),
        'gm_cc_get_indices': ([P, P, P, P], C.c_int),
        'gm_cc_get_surface_points': ([P, P], C.c_int),
        'gm_cc_set_state': ([P, P, P, P], C.c_int),
        'gm_cc_get_state': ([P, P, P, P], C.c_int),
        'gm_cc_set_inlet': ([P, P], C.c_int),
        'gm_cc_set_history': ([P, I32, P, P, D], C.c_int),
        'gm_cc_get_history': ([P, C.POINTER(I32), P, P, C.POINTER(D)], C.c_int),
        'gm_cc_step': ([P, D, I32, D, C.POINTER(CcStepDiag)], C.c_int),
        'gm_cc_apply': ([P, I32, D, P, P, P], C.c_int),
        'gm_cc_surface_forces': ([P, P, P, P, D, P], C.c_int),
        'gm_cc_divergence_stats': ([P, P, P, P], C.c_int),
        'gm_cc_phase_timing': ([P, P], C.c_int),
        'gm_mac_ab2_rhs': ([P, P, P, P, P, P, P, P, I32, I32, D, D, D, D, D, I32, I32, P], C.c_int),
        'gm_cc_legacy_step': ([P, D, I32, D, I32, C.POINTER(CcStepDiag)], C.c_int),
        'gm_cc_set_legacy_history': ([P, I32, P, D], C.c_int),
        'gm_cc_get_legacy_history': ([P, C.POINTER(I32), P, C.POINTER(D)], C.c_int),
        'gm_poisson_legacy_step': ([P, C.POINTER(LegacyState), D, I32, C.POINTER(LegacyStepDiag), P], C.c_int),
        'gm_mac_ghost_apply': ([P, I64, I64, P, P, P, P, P, P, I32, D, P], C.c_int),
        'gm_mac_ghost_correct': ([P, P, P, P, P, P, P, I32, I32, D, D, D, D, I32, P], C.c_int),
        'gm_mac_ghost_forces': ([P, P, P, I32, I32, D, D, D, D, D, I32, D, P, P], C.c_int),
        'gm_poisson_create': ([I32, I32, D, D, D, D, D, P, P, P, P, pp], C.c_int),
        'gm_poisson_destroy': ([P], C.c_int),
        'gm_poisson_last_error': ([P], C.c_char_p),
        'gm_poisson_solve': ([P, P, P, C.POINTER(D)], C.c_int),
    }
    for name, (args, res) in sig.items():
        f = getattr(lib, name)
        f.argtypes = args
        f.restype = res
    return lib


lib = _load()


class GhostError(Exception):
    pass


def error_for(rc: int, msg: str) -> Exception:
    """The reference's exception class for a GM_E* status."""
    return {GM_EVALUE: ValueError, GM_ERUNTIME: RuntimeError, GM_EFLOAT: FloatingPointError,
            GM_ENOTIMPL: NotImplementedError}.get(rc, GhostError)(msg)


def check(rc: int, handle=None):
    """Map a GM_E* status to the reference's exception classes."""
    if rc == GM_OK:
        return
    raise error_for(rc, lib.gm_last_error(handle).decode(errors='replace'))


def ptr(a):
    """Data pointer of a C-contiguous float64/int64 numpy array or a CUDA torch tensor."""
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        if not a.flags['C_CONTIGUOUS']:
            raise ValueError('arrays must be C-contiguous')
        return a.ctypes.data
    if hasattr(a, 'data_ptr'):
        if not a.is_contiguous():
            raise ValueError('tensors must be contiguous')
        return a.data_ptr()
    raise TypeError(f'unsupported array type {type(a)!r}')
