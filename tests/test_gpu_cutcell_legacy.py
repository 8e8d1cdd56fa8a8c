"""The legacy cut-cell loop on the GPU (MAC_CylinderFlow(boundary='cut_cell') with the reference's
default time_scheme='legacy') against the reference's own loop on the same grids
(tests/golden/cutcell_legacy.npz, written by tests/golden/make_golden.py, group cutcell_legacy):
centred transport with AB2 after an Euler first step, and upwind transport with forward Euler and
the transient inlet perturbation, on the 40x20 grid and on the 48x30 grid with rho = 1.3.

The reference adds the advective and viscous fluxes before differencing them; this library
evaluates the two forms separately and adds the accelerations, and solves the pressure system to
rounding with the boundary-corrected inverse instead of a sparse LU.  Both differences are at
rounding level, so after 20 steps the fields agree to 1e-10 and the force coefficients to 1e-9
relative."""
from pathlib import Path

import numpy as np
import pytest

from conftest import load_package

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).parent / 'golden' / 'cutcell_legacy.npz'
CASES = {
    'cc40x20': dict(nx=40, ny=20, Lx=4., Ly=2., D=1., xc=1., yc=1., nu=0.02, rho=1.),
    'cc48x30': dict(nx=48, ny=30, Lx=4.8, Ly=2.4, D=1., xc=1.3, yc=1.15, nu=0.01, rho=1.3),
}
RUNS = [('centered', 'centered', False), ('upwind', 'upwind', True)]


def rel(a, b):
    a, b = np.asarray(a, float), np.asarray(b, float)
    return float(np.max(np.abs(a - b))) / max(1.0, float(np.max(np.abs(b))))


def make(pkg, case, transport):
    return pkg.MAC_CylinderFlow(boundary='cut_cell', transport=transport, pressure_solver='direct', verbose=False,
                                **CASES[case])


@pytest.fixture(scope='module')
def gold():
    return np.load(GOLDEN)


@pytest.mark.parametrize('case', list(CASES))
@pytest.mark.parametrize('tag,transport,perturb', RUNS)
def test_legacy_loop_matches_reference(gold, case, tag, transport, perturb):
    pkg = load_package()
    s = make(pkg, case, transport)
    assert isinstance(s, pkg.CutCellFlow) and s.time_scheme == 'legacy'
    key = f'{case}_{tag}'
    assert np.array_equal(s.u, gold[f'{key}_init_u']) and np.array_equal(s.v, gold[f'{key}_init_v'])
    coef = []
    for k in range(20):
        _, cd, cl = s.solve(n_steps=1, dt=0.002, perturb_transient=perturb, perturb_duration=0.03,
                            save_artifacts=False, verbose=False)
        coef.append([cd[0], cl[0]])
        d = s.last_step_diagnostics
        ref = gold[f'{key}_record'][k]
        assert d['predicted_divergence'] < 1e-10 and ref[2] < 1e-10
        assert d['residual_linf'] < 1e-8 and d['max_divergence'] < 1e-9
        assert abs(d['cfl'] - ref[4]) <= 1e-10 * max(1.0, ref[4])
        if k + 1 in (1, 5, 20):
            for name in ('u', 'v', 'p'):
                err = rel(getattr(s, name), gold[f'{key}_{name}{k + 1}'])
                assert err < 1e-10, (k + 1, name, err)
            assert np.array_equal(s.phi, s.p)
    ref = gold[f'{key}_coef']
    assert np.max(np.abs(np.array(coef) - ref) / np.maximum(1.0, np.abs(ref))) < 1e-9
    assert abs(s.time - float(gold[f'{key}_time'])) < 1e-14
    au, av, prev_dt = s.legacy_history()
    assert rel(au, gold[f'{key}_prev_au']) < 1e-9 and rel(av, gold[f'{key}_prev_av']) < 1e-9
    assert prev_dt == float(gold[f'{key}_prev_dt'])


@pytest.mark.parametrize('case', list(CASES))
def test_upwind_momentum_rhs(gold, case):
    """compute_momentum_rhs(..., transport='upwind') with advection and viscosity together."""
    pkg = load_package()
    s = make(pkg, case, 'upwind')
    out = s.cc.compute_momentum_rhs(gold[f'{case}_probe_u'], gold[f'{case}_probe_v'], s.nu, s.rho,
                                    transport='upwind')
    for got, name in zip(out, ('au', 'av', 'ru', 'rv')):
        assert rel(got, gold[f'{case}_upwind_{name}']) < 1e-12, name


def test_multistep_solve_matches_stepwise(gold):
    """One solve(n_steps=20) call (the device steps without host reads in between) against the
    reference's twenty one-step calls."""
    pkg = load_package()
    s = make(pkg, 'cc40x20', 'centered')
    t, cd, cl = s.solve(n_steps=20, dt=0.002, perturb_transient=False, save_artifacts=False, verbose=False)
    assert t.shape == (20,)
    for name in ('u', 'v', 'p'):
        assert rel(getattr(s, name), gold[f'cc40x20_centered_{name}20']) < 1e-10, name
    ref = gold['cc40x20_centered_coef']
    assert np.max(np.abs(np.stack([cd, cl], 1) - ref) / np.maximum(1.0, np.abs(ref))) < 1e-9


def test_checkpoint_restart_keeps_predictor_history(gold, tmp_path):
    """Ten steps, a schema-1 checkpoint with prev_au / prev_av / prev_dt, a restart, ten more: the
    reference's twenty-step fields (the AB2 history crosses the restart)."""
    pkg = load_package()
    s = make(pkg, 'cc48x30', 'centered')
    s.solve(n_steps=10, dt=0.002, perturb_transient=False, save_artifacts=False, verbose=False)
    path = tmp_path / 'legacy.npz'
    s.save_checkpoint(path)
    with np.load(path) as data:
        assert 'prev_au' in data and 'cn_advection' not in data
    r = pkg.MAC_CylinderFlow.from_checkpoint(path)
    assert isinstance(r, pkg.CutCellFlow) and r.time_scheme == 'legacy'
    r.solve(n_steps=10, dt=0.002, perturb_transient=False, save_artifacts=False, verbose=False)
    for name in ('u', 'v', 'p'):
        assert rel(getattr(r, name), gold[f'cc48x30_centered_{name}20']) < 1e-10, name


def test_reference_defaults():
    """The reference's constructor defaults: boundary='immersed' (not built here) and
    time_scheme='legacy'."""
    pkg = load_package()
    with pytest.raises(NotImplementedError, match='immersed'):
        pkg.MAC_CylinderFlow(nx=40, ny=20, Lx=4., Ly=2., xc=1., yc=1., verbose=False)
    with pytest.raises(ValueError, match='ab2_cn requires'):
        pkg.MAC_CylinderFlow(nx=40, ny=20, Lx=4., Ly=2., xc=1., yc=1., boundary='staircase', time_scheme='ab2_cn',
                             verbose=False)
    with pytest.raises(ValueError, match='cg_dct is supported only for cut_cell'):
        pkg.MAC_CylinderFlow(nx=40, ny=20, Lx=4., Ly=2., xc=1., yc=1., boundary='ghost_cell',
                             pressure_solver='cg_dct', verbose=False)
