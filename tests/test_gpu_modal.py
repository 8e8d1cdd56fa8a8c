"""Snapshot POD on the GPU (modal.SnapshotPOD, csrc/modal.cu) against the reference's own
SnapshotPOD (postprocessing/modal_analysis.py) on a seeded synthetic wake
(tests/golden/modal.npz): the mean field bit-identical (same summation order), energies and
singular values to 1e-10 relative to the largest, the leading modes and coefficients to 1e-8
up to the sign of each mode (an eigenvector's sign is arbitrary), and the phase-portrait
metrics of the first two coefficients."""
import sys

import numpy as np
import pytest

from conftest import GOLDEN, load_package


@pytest.fixture(scope='module')
def modal():
    pkg = load_package()
    __import__(pkg.__name__ + '.modal')
    return sys.modules[pkg.__name__ + '.modal']


@pytest.fixture(scope='module')
def G():
    return np.load(GOLDEN / 'modal.npz')


@pytest.mark.gpu
def test_snapshot_pod_matches_reference(modal, G):
    pod = modal.SnapshotPOD(n_modes=6).fit(G['snapshots'])
    assert np.array_equal(pod.mean_field, G['mean_field'])
    top = G['modal_energies'][0]
    assert np.max(np.abs(pod.modal_energies - G['modal_energies'])) < 1e-10 * top
    assert np.max(np.abs(pod.singular_values - G['singular_values'])) < 1e-10 * G['singular_values'][0]
    assert np.max(np.abs(pod.cumulative_energy - G['cumulative_energy'])) < 1e-10
    # the well-separated leading modes (the noise modes beyond them are not unique)
    for i in range(4):
        a, b = pod.spatial_modes[i], G['spatial_modes'][i]
        sgn = np.sign(np.sum(a * b))
        assert np.max(np.abs(sgn * a - b)) < 1e-8 * np.max(np.abs(b)), i
        c, d = pod.temporal_coeffs[i], G['temporal_coeffs'][i]
        assert np.max(np.abs(sgn * c - d)) < 1e-8 * np.max(np.abs(d)), i
    pp = modal.compute_phase_portrait_metrics(pod.temporal_coeffs[0], pod.temporal_coeffs[1])
    assert abs(pp['mean_amplitude'] - G['phase'][0]) < 1e-8 * G['phase'][0]
    assert abs(pp['circularity_error'] - G['phase'][1]) < 1e-6


@pytest.mark.gpu
def test_snapshot_pod_device_snapshots(modal, G):
    """CUDA tensors in, same answer as numpy in (the snapshots are read on the device)."""
    torch = pytest.importorskip('torch')
    a = modal.SnapshotPOD(n_modes=3).fit(G['snapshots'])
    b = modal.SnapshotPOD(n_modes=3).fit(torch.from_numpy(G['snapshots']).cuda())
    assert np.array_equal(a.mean_field, b.mean_field)
    assert np.array_equal(a.modal_energies, b.modal_energies)
    assert np.array_equal(a.spatial_modes, b.spatial_modes)


def test_phase_portrait_metrics_host(modal):
    th = np.linspace(0, 2 * np.pi, 50, endpoint=False)
    pp = modal.compute_phase_portrait_metrics(2 * np.cos(th), 2 * np.sin(th))
    assert abs(pp['mean_amplitude'] - 2.0) < 1e-12 and pp['circularity_error'] < 1e-12
