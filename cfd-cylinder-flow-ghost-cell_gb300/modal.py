"""Snapshot POD of wake fields on the GPU (postprocessing/modal_analysis.py).

``SnapshotPOD(n_modes).fit(snapshots)`` has the reference's attributes and conventions: the
mean field, the fluctuation Gram matrix C = X' X'^T / M (formed on the device by
gm_pod_gram), its eigen-decomposition on the host (M x M, numpy.linalg.eigh, sorted by
descending energy, negative eigenvalues clipped to zero), singular values sqrt(M lambda), energy
ratios and their cumulative sum, and the first n_modes spatial modes X'^T v_i / sigma_i and
temporal coefficients X' phi_i (formed on the device by gm_pod_modes).  Snapshots are (M, ny, nx)
or (M, n_points) arrays, numpy or CUDA torch; results are numpy.
``compute_phase_portrait_metrics(a1, a2)`` is the reference's limit-cycle measure of the first
two coefficients (host numpy).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import lib, ptr


class SnapshotPOD:
    def __init__(self, n_modes=10):
        self.n_modes = n_modes
        self.mean_field = None
        self.spatial_modes = None
        self.temporal_coeffs = None
        self.singular_values = None
        self.modal_energies = None
        self.energy_ratios = None
        self.cumulative_energy = None

    def fit(self, snapshots):
        shape = tuple(snapshots.shape)
        m = shape[0]
        grid = shape[1:]
        npts = int(np.prod(grid))
        if hasattr(snapshots, 'data_ptr'):
            import torch
            x = snapshots.reshape(m, npts).to(torch.float64).contiguous()
        else:
            x = np.ascontiguousarray(np.asarray(snapshots, dtype=np.float64).reshape(m, npts))
        h = C.c_void_p()
        rc = lib.gm_pod_create(int(m), int(npts), C.byref(h))
        if rc != _lib.GM_OK:
            raise _lib.error_for(rc, 'snapshot POD set-up failed (sizes or device memory)')
        try:
            mean = np.empty(npts)
            gram = np.empty((m, m))
            self._check(lib.gm_pod_gram(h, ptr(x), ptr(mean), ptr(gram), None), h)
            eigvals, eigvecs = np.linalg.eigh(gram)
            order = np.argsort(eigvals)[::-1]
            eigvals = np.maximum(eigvals[order], 0.0)
            eigvecs = eigvecs[:, order]
            self.singular_values = np.sqrt(eigvals * float(m))
            self.modal_energies = eigvals
            total = np.sum(eigvals)
            if total > 1e-15:
                self.energy_ratios = eigvals / total
                self.cumulative_energy = np.cumsum(self.energy_ratios)
            else:
                self.energy_ratios = np.zeros_like(eigvals)
                self.cumulative_energy = np.zeros_like(eigvals)
            k = min(self.n_modes, m)
            v = np.ascontiguousarray(eigvecs[:, :k])
            sig = np.ascontiguousarray(self.singular_values[:k])
            modes = np.empty((k, npts))
            coeffs = np.empty((k, m))
            self._check(lib.gm_pod_modes(h, ptr(v), ptr(sig), int(k), ptr(modes), ptr(coeffs), None), h)
        finally:
            lib.gm_pod_destroy(h)
        self.spatial_modes = modes
        self.temporal_coeffs = coeffs
        self.mean_field = mean
        if len(grid) == 2:
            self.spatial_modes = modes.reshape(k, grid[0], grid[1])
            self.mean_field = mean.reshape(grid[0], grid[1])
        return self

    @staticmethod
    def _check(rc, h):
        if rc != _lib.GM_OK:
            raise _lib.error_for(rc, (lib.gm_pod_last_error(h) or b'').decode(errors='replace'))


def compute_phase_portrait_metrics(a1, a2):
    """Mean radius of the (a1, a2) orbit and its circularity error std(r) / mean(r)
    (postprocessing/modal_analysis.py:101-114)."""
    a1, a2 = np.asarray(a1), np.asarray(a2)
    radius = np.hypot(a1, a2)
    mean_radius = float(np.mean(radius))
    return dict(mean_amplitude=mean_radius,
                circularity_error=float(np.std(radius) / np.maximum(mean_radius, 1e-14)))
