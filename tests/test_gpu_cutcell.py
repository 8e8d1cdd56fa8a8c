"""Cut-cell AB2/CN path on the GPU (MAC_CylinderFlow(boundary='cut_cell', time_scheme='ab2_cn'))
against the reference's own outputs on the same grids (tests/golden/cutcell_*.npz, written by
tests/golden/make_golden.py from solver/cut_cell_solver.py run with numba replaced by plain
Python).  The reference solves its pressure system with a sparse LU and its CN system with
GMRES to rtol 1e-12; the GPU uses the boundary-corrected separable inverse and a device GMRES
to the same tolerance, so the operators agree to rounding (1e-12 relative), a pressure solve to
the system's conditioning (1e-9) and stepped fields to the GMRES tolerance carried through the
projections (velocity 1e-9, pressure 1e-7 relative to the field's magnitude)."""
from pathlib import Path

import numpy as np
import pytest

from conftest import load_package

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).parent / 'golden'
CASES = ('cc40x20', 'cc48x30')


def rel(a, b):
    a, b = np.asarray(a, float), np.asarray(b, float)
    return float(np.max(np.abs(a - b))) / max(1.0, float(np.max(np.abs(b))))


def make(pkg, d, **extra):
    nx, ny, Lx, Ly, D, xc, yc, nu, rho = d['config']
    return pkg.MAC_CylinderFlow(nx=int(nx), ny=int(ny), Lx=Lx, Ly=Ly, D=D, xc=xc, yc=yc, nu=nu, rho=rho,
                                boundary='cut_cell', time_scheme='ab2_cn', pressure_solver='direct',
                                verbose=False, **extra)


@pytest.fixture(scope='module', params=CASES)
def case(request):
    pkg = load_package()
    d = np.load(GOLDEN / f'cutcell_{request.param}.npz')
    return pkg, d, make(pkg, d)


def test_dispatch_and_initial_projection(case):
    pkg, d, s = case
    assert isinstance(s, pkg.CutCellFlow)
    assert rel(s.u, d['init_u']) < 1e-10 and rel(s.v, d['init_v']) < 1e-10
    assert np.array_equal(s.cut_geom.cell_type, d['geom_cell_type'])
    assert np.allclose(s.cc.pressure_points, d['surface_points'], rtol=0, atol=1e-14)


def test_momentum_rhs_both_forms(case):
    """compute_momentum_rhs on seeded fields: the advective form (nu = 0) and the viscous form."""
    _, d, s = case
    u, v = d['rand_u'], d['rand_v']
    for mode, nu, adv in (('adv', 0.0, True), ('dif', s.nu, False)):
        au, av, ru, rv = s.cc.compute_momentum_rhs(u, v, nu, s.rho, transport='centered', include_advection=adv)
        for got, key in ((au, 'au'), (av, 'av'), (ru, 'ru'), (rv, 'rv')):
            assert rel(got, d[f'{mode}_{key}']) < 1e-12, (mode, key, rel(got, d[f'{mode}_{key}']))


def test_pressure_solve(case):
    _, d, s = case
    phi = s.cc.solve_pressure(d['prhs'], 0.01, s.rho)
    ref = d['psol']
    assert np.max(np.abs(phi - ref)) < 1e-9 * max(1.0, np.max(np.abs(ref)))
    assert np.all(phi[s.cut_geom.cell_type == -1] == 0.0)


def test_forces_and_divergence_on_seeded_fields(case):
    _, d, s = case
    f = s.cc.extract_true_surface_forces(d['rand_u'], d['rand_v'], d['rand_p'], s.nu * s.rho)
    ref = d['forces_rand']
    assert np.max(np.abs(np.array(f) - ref)) < 1e-11 * max(1.0, np.max(np.abs(ref)))
    md, rd, mf = s.cc.divergence_stats(d['rand_u'], d['rand_v'])
    assert np.allclose([md, rd, mf], d['divergence_rand'], rtol=1e-12, atol=0)


def test_steps_from_perturbed_state(case):
    """Six AB2/CN steps (the projected midpoint start-up, then AB2) from the reference's seeded
    perturbation of the initial state: fields, force coefficients and gates per step, and the
    restart history afterwards."""
    pkg, d, _ = case
    s = make(pkg, d)
    s.u[:], s.v[:] = d['start_u'], d['start_v']
    keys = list(d['step_keys'])
    for k in range(6):
        s.solve(n_steps=1, dt=.002, perturb_transient=False, save_artifacts=False, verbose=False)
        ref = dict(zip(keys, d['step_scalars'][k]))
        diag = s.last_step_diagnostics
        ru, rv, rp = rel(s.u, d['step_u'][k]), rel(s.v, d['step_v'][k]), rel(s.p, d['step_p'][k])
        assert ru < 1e-9 and rv < 1e-9 and rp < 1e-7, (k, ru, rv, rp)
        for key in ('cd', 'cl', 'cd_pressure', 'cd_viscous', 'cl_pressure', 'cl_viscous'):
            assert abs(diag[key] - ref[key]) < 1e-7 * max(1.0, abs(ref[key])), (k, key, diag[key], ref[key])
        assert diag['max_divergence'] < 1e-10 and diag['cfl'] < 0.5
        assert abs(diag['cfl'] - ref['cfl']) < 1e-9
        assert diag['pressure_solves'] == int(ref['pressure_solves'])
        assert abs(diag['momentum_iterations'] - ref['momentum_iterations']) <= 2
    adv, half, dtp = s.cc.history()
    assert dtp == 0.002
    assert rel(half, d['history_half_p']) < 1e-7
    assert rel(adv, d['history_adv']) < 1e-8


def test_long_run_with_inlet_perturbation():
    """cc40x20: the six steps, then 60 more with the transient inlet perturbation of
    solver/main.py:281-286 (duration 0.3): final fields and coefficients."""
    pkg = load_package()
    d = np.load(GOLDEN / 'cutcell_cc40x20.npz')
    s = make(pkg, d)
    s.u[:], s.v[:] = d['start_u'], d['start_v']
    s.solve(n_steps=6, dt=.002, perturb_transient=False, save_artifacts=False, verbose=False)
    s.solve(n_steps=60, dt=.002, perturb_transient=True, perturb_duration=0.3, save_artifacts=False, verbose=False)
    keys = list(d['step_keys'])
    ref = dict(zip(keys + ['time'], d['long_scalars']))
    assert abs(s.time - ref['time']) < 1e-12
    assert rel(s.u, d['long_u']) < 1e-8 and rel(s.v, d['long_v']) < 1e-8 and rel(s.p, d['long_p']) < 1e-6
    diag = s.last_step_diagnostics
    for key in ('cd', 'cl'):
        assert abs(diag[key] - ref[key]) < 1e-6 * max(1.0, abs(ref[key])), (key, diag[key], ref[key])


def test_packed_operators_and_projection(case):
    """advance_ab2_cn's closures on a packed vector: the CN operator is linear in q (H(0) = 0,
    H(a q) = a H(q)), the projection leaves a field whose aperture divergence vanishes on the
    fluid cells, and projecting twice changes nothing."""
    _, d, s = case
    rng = np.random.default_rng(3)
    q = rng.standard_normal(s.cc.qsize)
    h1 = s.cc.H_matvec(q, 0.002)
    assert np.max(np.abs(s.cc.H_matvec(np.zeros_like(q), 0.002))) == 0.0
    assert rel(s.cc.H_matvec(2.5 * q, 0.002), 2.5 * h1) < 1e-13
    p1, phi = s.cc.project(q, 0.002)
    u, v = s.cc.unpack(p1)
    md, _, _ = s.cc.divergence_stats(u, v)
    assert md < 1e-9
    p2, _ = s.cc.project(p1, 0.002)
    assert rel(p2, p1) < 1e-12


def test_invalid_configurations():
    pkg = load_package()
    with pytest.raises(ValueError, match='centered'):
        pkg.MAC_CylinderFlow(nx=40, ny=20, Lx=4., Ly=2., xc=1., yc=1., boundary='cut_cell', transport='upwind',
                             time_scheme='ab2_cn', verbose=False)
    with pytest.raises(ValueError, match='strictly inside'):
        pkg.MAC_CylinderFlow(nx=40, ny=20, Lx=4., Ly=2., xc=.4, yc=1., boundary='cut_cell', time_scheme='ab2_cn',
                             verbose=False)


def test_checkpoint_round_trip(tmp_path):
    """save_checkpoint / from_checkpoint of a cut-cell case (solver/main.py:503-567): the resumed
    solver continues exactly as the original."""
    pkg = load_package()
    d = np.load(GOLDEN / 'cutcell_cc40x20.npz')
    s = make(pkg, d)
    s.u[:], s.v[:] = d['start_u'], d['start_v']
    s.solve(n_steps=4, dt=.002, perturb_transient=False, save_artifacts=False, verbose=False)
    ck = tmp_path / 'cc.npz'
    s.save_checkpoint(ck)
    with pytest.raises(FileExistsError):
        s.save_checkpoint(ck)
    r = pkg.MAC_CylinderFlow.from_checkpoint(ck)
    assert isinstance(r, pkg.CutCellFlow) and r.time == s.time
    for x in (s, r):
        x.solve(n_steps=3, dt=.002, perturb_transient=False, save_artifacts=False, verbose=False)
    assert np.max(np.abs(r.u - s.u)) < 1e-14 and np.max(np.abs(r.v - s.v)) < 1e-14
    assert np.max(np.abs(r.p - s.p)) < 1e-12 * max(1.0, np.max(np.abs(s.p)))


def test_reference_checkpoint_resume():
    """A checkpoint the reference's own save_checkpoint wrote after six cut-cell steps: rejected as
    a source mismatch by default, imported with accept_reference, and three resumed steps match
    the reference's own resumed fields."""
    pkg = load_package()
    d = np.load(GOLDEN / 'cutcell_cc40x20.npz')
    ck = GOLDEN / 'reference_checkpoint_cutcell_cc40x20.npz'
    with pytest.raises(ValueError, match='source mismatch'):
        pkg.MAC_CylinderFlow.from_checkpoint(ck)
    r = pkg.MAC_CylinderFlow.from_checkpoint(ck, accept_reference=True)
    assert r.restored_from == 'reference'
    r.solve(n_steps=3, dt=.002, perturb_transient=False, save_artifacts=False, verbose=False)
    t, cd, cl = d['resume_scalars']
    assert abs(r.time - t) < 1e-12
    assert rel(r.u, d['resume_u']) < 1e-9 and rel(r.v, d['resume_v']) < 1e-9 and rel(r.p, d['resume_p']) < 1e-7
    assert abs(r.last_step_diagnostics['cd'] - cd) < 1e-7 * abs(cd)


def test_benched_grid_against_reference():
    """The benched grid (800x820, 40D x 41D, Re 100) from bench.py's seeded 1e-2 v perturbation:
    three steps against the reference's own three steps (tests/golden/cutcell_wide_800x820.npz:
    4000 seeded samples per field and step, the field norms and the force coefficients)."""
    import sys
    pkg = load_package()
    d = np.load(GOLDEN / 'cutcell_wide_800x820.npz')
    sys.path.insert(0, str(GOLDEN.parents[1]))
    import bench
    w = bench.CUTCELL_WORKLOADS['cutcell_800x820_re100']
    kw = {k: w[k] for k in ('nx', 'ny', 'Lx', 'Ly', 'D', 'xc', 'yc', 'nu')}
    s = pkg.MAC_CylinderFlow(boundary='cut_cell', time_scheme='ab2_cn', verbose=False, **kw)
    bench.seeded_state(s, w)
    for k in range(3):
        s.solve(n_steps=1, dt=w['dt'], perturb_transient=False, save_artifacts=False, verbose=False)
        diag = s.last_step_diagnostics
        cd, cl, mdiv, cfl, its = d['scalars'][k]
        for got, ref, scale in ((s.u.ravel()[d['sample_u']], d['u_samples'][k], d['norms'][k][0]),
                                (s.v.ravel()[d['sample_v']], d['v_samples'][k], d['norms'][k][1])):
            assert np.max(np.abs(got - ref)) < 1e-9 * max(1.0, scale), k
        assert np.max(np.abs(s.p.ravel()[d['sample_p']] - d['p_samples'][k])) < 1e-7 * max(1.0, d['norms'][k][2]), k
        assert abs(float(np.sqrt(np.mean(s.u ** 2))) - d['norms'][k][3]) < 1e-10
        assert abs(diag['cd'] - cd) < 1e-7 * abs(cd) and abs(diag['cl'] - cl) < 1e-7 * max(1.0, abs(cl))
        assert diag['max_divergence'] < 1e-10 and abs(diag['cfl'] - cfl) < 1e-9
        assert abs(diag['momentum_iterations'] - its) <= 2


def test_options_parabolic_slip_cg_dct():
    """Parabolic inflow (U_m = 1.2), slip channel walls and pressure_solver='cg_dct' on the 40x20
    grid: the initial projection and four steps against the reference run with the same options
    (the reference's CG / boundary-Schur-DCT solve and this library's direct inverse meet the same
    1e-10 divergence budget, so the fields agree to it)."""
    pkg = load_package()
    d = np.load(GOLDEN / 'cutcell_options_40x20.npz')
    s = pkg.MAC_CylinderFlow(nx=40, ny=20, Lx=4., Ly=2., D=1., xc=1.1, yc=0.95, nu=0.02, inflow='parabolic',
                             U_m=1.2, slip_walls=True, pressure_solver='cg_dct', boundary='cut_cell',
                             time_scheme='ab2_cn', verbose=False)
    assert np.array_equal(s.u_inlet, d['u_inlet'])
    assert rel(s.u, d['init_u']) < 1e-9 and rel(s.v, d['init_v']) < 1e-9
    for k in range(4):
        s.solve(n_steps=1, dt=.002, perturb_transient=False, save_artifacts=False, verbose=False)
        cd, cl, mdiv, cfl = d['scalars'][k]
        assert rel(s.u, d['step_u'][k]) < 1e-8 and rel(s.v, d['step_v'][k]) < 1e-8, k
        assert rel(s.p, d['step_p'][k]) < 1e-6, k
        diag = s.last_step_diagnostics
        assert abs(diag['cd'] - cd) < 1e-6 * abs(cd) and abs(diag['cl'] - cl) < 1e-6 * max(1.0, abs(cl))
        assert diag['max_divergence'] < 1e-10


def test_benched_grid_momentum_gate_like_reference():
    """The benched workload stepped until the CN momentum gate (solver/time_integration.py:100-104)
    raises: the reference's own loop raises at step 71 (tests/golden/cutcell_gate_800x820.npz,
    group cutcell_gate of tests/golden/make_golden.py).  Here the gate raises at the same step with
    the same message, and every earlier step's momentum residual (about 2e-12 to 2e-11) agrees
    with the reference's to 1e-2 relative, its GMRES iteration count to 2."""
    import sys
    pkg = load_package()
    d = np.load(GOLDEN / 'cutcell_gate_800x820.npz')
    sys.path.insert(0, str(GOLDEN.parents[1]))
    import bench
    w = bench.CUTCELL_WORKLOADS['cutcell_800x820_re100']
    kw = {k: w[k] for k in ('nx', 'ny', 'Lx', 'Ly', 'D', 'xc', 'yc', 'nu')}
    s = pkg.MAC_CylinderFlow(boundary='cut_cell', time_scheme='ab2_cn', verbose=False, **kw)
    bench.seeded_state(s, w)
    raised = int(d['raised'])
    assert raised > 0
    for k in range(raised - 1):
        s.solve(n_steps=1, dt=w['dt'], perturb_transient=False, save_artifacts=False, verbose=False)
        diag = s.last_step_diagnostics
        ref = float(d['residuals'][k])
        assert abs(diag['momentum_residual_linf'] - ref) <= 1e-2 * ref, (k + 1, diag['momentum_residual_linf'], ref)
        assert abs(diag['momentum_iterations'] - int(d['iterations'][k])) <= 2
    with pytest.raises(RuntimeError) as e:
        s.solve(n_steps=1, dt=w['dt'], perturb_transient=False, save_artifacts=False, verbose=False)
    head = 'CN momentum solve failed: info=0, residual='
    ref_msg = str(d['message'])
    assert ref_msg.startswith(head) and str(e.value).startswith(head), (str(e.value), ref_msg)
    ref_res, got_res = float(ref_msg[len(head):]), float(str(e.value)[len(head):])
    assert ref_res > 1e-10 and abs(got_res - ref_res) <= 1e-2 * ref_res
