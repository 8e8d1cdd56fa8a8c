"""The legacy ghost-cell loop on the GPU (MAC_CylinderFlow(boundary='ghost_cell',
time_scheme='legacy')) against the reference's own loop on the same grid
(tests/golden/legacy_ghost_48x24.npz, written by tests/golden/make_golden.py with mac_engine
built from solver/src/bindings.cpp, the reference's GhostCellBoundary and its sparse-LU
pressure solve): centred transport with the loop's AB2 step, and upwind transport with the
transient inlet perturbation.  The predictor, ghost velocities and corrector are bit-identical
to the reference's arithmetic and the pressure solve agrees with the LU to rounding, so the
fields agree to 1e-11; the forces on the true circle interpolate the same fields with the same
formulas, summed in another order, and agree to 1e-10 relative."""
from pathlib import Path

import numpy as np
import pytest

from conftest import load_package

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).parent / 'golden'
CASE = dict(nx=48, ny=24, Lx=4.8, Ly=2.4, D=1.0, xc=1.3, yc=1.15, nu=0.02, boundary='ghost_cell',
            time_scheme='legacy', pressure_solver='direct', verbose=False)


def rel(a, b):
    a, b = np.asarray(a, float), np.asarray(b, float)
    return float(np.max(np.abs(a - b))) / max(1.0, float(np.max(np.abs(b))))


@pytest.mark.parametrize('tag,transport,perturb', [('centered', 'centered', False), ('upwind', 'upwind', True)])
def test_legacy_ghost_loop_matches_reference(tag, transport, perturb):
    pkg = load_package()
    d = np.load(GOLDEN / 'legacy_ghost_48x24.npz')
    s = pkg.MAC_CylinderFlow(transport=transport, **CASE)
    assert isinstance(s, pkg.LegacyGhostFlow)
    assert s.ghost_counts()['u'][0] == len(d['ghost_u_faces'])
    assert np.array_equal(s.u, d[f'{tag}_init_u']) and np.array_equal(s.v, d[f'{tag}_init_v'])
    coef = []
    for k in range(20):
        _, cd, cl = s.solve(n_steps=1, dt=0.002, perturb_transient=perturb, perturb_duration=0.03,
                            save_artifacts=False, verbose=False)
        coef.append([cd[0], cl[0]])
        if k + 1 in (1, 5, 20):
            for key in ('u', 'v', 'p'):
                err = rel(getattr(s, key), d[f'{tag}_{key}{k + 1}'])
                assert err < 1e-11, (k + 1, key, err)
    ref = d[f'{tag}_coef']
    assert np.max(np.abs(np.array(coef) - ref) / np.maximum(1.0, np.abs(ref))) < 1e-10
    assert abs(s.time - float(d[f'{tag}_time'])) < 1e-14


def test_legacy_ghost_multistep_solve_matches_stepwise():
    """One solve(n_steps=20) call against the reference's twenty one-step calls."""
    pkg = load_package()
    d = np.load(GOLDEN / 'legacy_ghost_48x24.npz')
    s = pkg.MAC_CylinderFlow(transport='centered', **CASE)
    t, cd, cl = s.solve(n_steps=20, dt=0.002, perturb_transient=False, save_artifacts=False, verbose=False)
    assert t.shape == (20,)
    for key in ('u', 'v', 'p'):
        assert rel(getattr(s, key), d[f'centered_{key}20']) < 1e-11, key
    ref = d['centered_coef']
    assert np.max(np.abs(np.stack([cd, cl], 1) - ref) / np.maximum(1.0, np.abs(ref))) < 1e-10


def test_legacy_ghost_apply_matches_host_tables():
    """gm_mac_ghost_apply on host arrays against the sequential pass over the same tables."""
    pkg = load_package()
    st = pkg.staircase
    lib, ptr = pkg._lib.lib, pkg._lib.ptr
    nx, ny, dx, dy = 800, 820, 20.5 / 800, 21.0 / 820
    xs, ys = np.arange(nx + 1) * dx, (np.arange(ny) + 0.5) * dy
    t = st.ghost_face_tables(xs, ys, dx, dy, 5.0, 10.5, 0.5, True)
    assert t['n_levels'] > 1
    f = np.random.default_rng(3).standard_normal(ny * (nx + 1))
    ref = f.copy()
    for g in range(t['target'].size):
        w, c = t['weights'][g], t['src'][g]
        ip = w[0] * ref[c[0]] + w[1] * ref[c[1]] + w[2] * ref[c[2]] + w[3] * ref[c[3]]
        ref[t['target'][g]] = 0.25 - t['gamma'][g] * (ip - 0.25)
    out = f.copy()
    tabs = {k: np.ascontiguousarray(t[k]) for k in ('target', 'src', 'snap_of', 'weights', 'gamma', 'level')}
    rc = lib.gm_mac_ghost_apply(ptr(out), out.size, t['target'].size, ptr(tabs['target']), ptr(tabs['src']),
                                tabs['snap_of'].ctypes.data, ptr(tabs['weights']), ptr(tabs['gamma']),
                                tabs['level'].ctypes.data, t['n_levels'], 0.25, None)
    assert rc == pkg._lib.GM_OK
    assert np.array_equal(out, ref)


def test_legacy_ghost_rejects_reconstruction_options():
    pkg = load_package()
    with pytest.raises(ValueError, match='Ghost reconstruction options require Ghost AB2/CN'):
        pkg.MAC_CylinderFlow(ghost_velocity_interpolation='biquadratic', **CASE)
