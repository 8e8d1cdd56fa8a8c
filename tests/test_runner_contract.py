"""The runner contract and checkpoint interop of the reference campaign tooling.

Fixtures (tests/golden/make_golden.py, group ``runner``) come from the reference's own code:
a checkpoint written by its save_checkpoint (solver/main.py:503-530) with the fields after it
resumes that checkpoint for three steps; its runner (validation/run_ghost_validation.py:19-102)
on a small steady case; its point-pressure reconstruction (solver/cut_cell_solver.py:25-55)
and recirculation lengths (postprocessing/cylinder_observables.py:8-27).

CPU tests: the reconstruction operator through a host-only handle, the recirculation rule and
the window means of the reference's own sample file.  GPU tests: resuming the reference's
checkpoint, and the runner's files against the reference runner's.
"""
import ctypes as C
import json
import sys

import numpy as np
import pytest

from conftest import GOLDEN, load_package


@pytest.fixture(scope='module')
def G():
    return np.load(GOLDEN / 'runner_88x16.npz')


@pytest.fixture(scope='module')
def pkg():
    return load_package()


def module(pkg, name):
    __import__(pkg.__name__ + '.' + name)
    return sys.modules[pkg.__name__ + '.' + name]


def host_handle(L, solver):
    cfg = L.Config(nx=solver['nx'], ny=solver['ny'], Lx=solver['Lx'], Ly=solver['Ly'], D=solver['D'],
                   xc=solver['xc'], yc=solver['yc'], nu=solver['nu'], rho=1., U_inf=1., inflow=0, U_m=0.,
                   pressure_solver=0, pressure_extension=0, velocity_interpolation=0, precision=0)
    h = C.c_void_p()
    L.check(L.lib.gm_create_host(C.byref(cfg), C.byref(h)))
    return h


def test_pressure_reconstruction_matches_reference(pkg, G):
    """The quadratic point-pressure operator at the stagnation points and three other points:
    the same neighbours (bit-exact columns) and weights to 1e-12 (one least-squares solve)."""
    L = pkg._lib
    ghost = module(pkg, 'ghost')
    solver = json.loads(str(G['case']))['solver']
    h = host_handle(L, solver)
    try:
        op = ghost.pressure_reconstruction(h, G['rec_points'], solver['nx'] * solver['ny'])
    finally:
        L.lib.gm_destroy(h)
    assert np.array_equal(op.indptr, G['rec_indptr'])
    for k in range(len(op.indptr) - 1):
        a, b = slice(op.indptr[k], op.indptr[k + 1]), slice(G['rec_indptr'][k], G['rec_indptr'][k + 1])
        oa, ob = np.argsort(op.indices[a]), np.argsort(G['rec_indices'][b])
        assert np.array_equal(op.indices[a][oa], G['rec_indices'][b][ob])
        assert np.max(np.abs(op.data[a][oa] - G['rec_data'][b][ob])) < 1e-12


@pytest.mark.parametrize('points, message', [([[2.0, 2.0]], 'inside the solid'), ([[5.0, 1.0]], 'inside the domain'),
                                             ([[np.nan, 1.0]], 'finite')])
def test_pressure_reconstruction_rejects_points(pkg, G, points, message):
    L = pkg._lib
    ghost = module(pkg, 'ghost')
    solver = json.loads(str(G['case']))['solver']
    h = host_handle(L, solver)
    try:
        with pytest.raises(ValueError, match=message):
            ghost.pressure_reconstruction(h, np.array(points), solver['nx'] * solver['ny'])
    finally:
        L.lib.gm_destroy(h)


def test_recirculation_length_rule(pkg, G):
    obs = module(pkg, 'observables')
    x = G['recirc_x']
    cases = (np.linspace(-1, 1, 10), np.linspace(0.1, 1, 10), np.r_[0.2, 0.3, -0.1, -0.2, np.linspace(.1, 1, 6)],
             -np.ones(10))
    for vel, length, status in zip(cases, G['recirc_lengths'].ravel(), G['recirc_status']):
        r = obs.recirculation_length(x, vel, 1.5, 1.0)
        assert r['status'] == str(status)
        if np.isnan(length):
            assert r['length_D'] is None
        else:
            assert abs(r['length_D'] - length) < 1e-14
    with pytest.raises(ValueError, match='Invalid wake centerline'):
        obs.recirculation_length(x[::-1], cases[0], 1.5, 1.0)


def test_mean_observables_of_reference_samples(pkg, G, tmp_path):
    """mean_observables over the reference runner's own centre-line file gives its
    mean_observables.json (same trapezoids, same window)."""
    obs = module(pkg, 'observables')
    path = tmp_path / 'centerline.bin'
    G['centerline'].astype('<f8').tofile(path)
    path.with_suffix('.json').write_text(str(G['centerline_meta']))
    ref = json.loads(str(G['mean_observables']))
    got = obs.mean_observables(path, *ref['window'])
    for key in ('p_front_mean', 'p_back_mean', 'delta_p_mean', 'sample_max_dt'):
        assert abs(got[key] - ref[key]) <= 1e-14 * max(1.0, abs(ref[key])), key
    assert np.max(np.abs(np.array(got['u_centerline_mean']) - ref['u_centerline_mean'])) < 1e-14
    assert got['recirculation'] == ref['recirculation']
    with pytest.raises(ValueError, match='cover'):
        obs.mean_observables(path, ref['window'][0] - 1.0, ref['window'][1])


@pytest.mark.gpu
def test_resume_reference_checkpoint(pkg):
    """A checkpoint written by the reference is rejected by default and imported with
    accept_reference=True; three more steps then match the reference resuming it (fields
    1e-10, C_D 1e-8 relative)."""
    ck = GOLDEN / 'reference_checkpoint_88x16.npz'
    R = np.load(GOLDEN / 'reference_resume_88x16.npz')
    with pytest.raises(ValueError, match='reference'):
        pkg.MAC_CylinderFlow.from_checkpoint(ck)
    s = pkg.MAC_CylinderFlow.from_checkpoint(ck, accept_reference=True)
    assert s.restored_from == 'reference'
    for k in range(3):
        s.solve(n_steps=1, dt=.002, perturb_transient=False, save_artifacts=False, verbose=False)
        t, cd, cl, div = R['scalars'][k]
        d = s.last_step_diagnostics
        assert abs(s.time - t) < 1e-12
        assert abs(d['cd'] - cd) < 1e-8 * abs(cd)
        assert d['max_divergence'] < 1e-10
    for key in ('u', 'v', 'p'):
        ref = R[key]
        assert np.max(np.abs(getattr(s, key) - ref)) < 1e-10 * max(1.0, np.max(np.abs(ref))), key


@pytest.mark.gpu
def test_runner_matches_reference_runner(pkg, G, tmp_path):
    """runner.run on the reference runner's case writes the same files; the history rows,
    window statistics and mean observables agree with the reference's (C_D, C_L, delta_p to
    1e-8 relative; times exactly)."""
    runner = module(pkg, 'runner')
    cfg = tmp_path / 'case.json'
    cfg.write_text(str(G['case']))
    out = tmp_path / 'run'
    runner.run(cfg, out)
    for name in ('manifest.json', 'history.jsonl', 'summary.json', 'mean_observables.json', 'centerline.bin',
                 'centerline.json', 'checkpoint.npz'):
        assert (out / name).exists(), name
    rows = [json.loads(line) for line in (out / 'history.jsonl').read_text().splitlines()]
    keys = [str(k) for k in G['history_keys']]
    assert set(keys) <= set(rows[0]), set(keys) - set(rows[0])
    got = np.array([[float(r[k]) for k in keys] for r in rows])
    ref = G['history']
    assert got.shape == ref.shape
    col = {k: i for i, k in enumerate(keys)}
    assert np.array_equal(got[:, col['step']], ref[:, col['step']])
    assert np.max(np.abs(got[:, col['time']] - ref[:, col['time']])) < 1e-12
    for k in ('cd', 'cl', 'delta_p', 'cd_pressure', 'cd_viscous'):
        assert np.max(np.abs(got[:, col[k]] - ref[:, col[k]])) < 1e-8 * max(1.0, np.max(np.abs(ref[:, col[k]]))), k
    assert np.max(got[:, col['max_divergence']]) < 1e-10
    s_got = json.loads((out / 'summary.json').read_text())
    s_ref = json.loads(str(G['summary']))
    assert s_got['completed'] and s_got['steps'] == s_ref['steps']
    assert s_got['sample_window'] == s_ref['sample_window']
    for stat in ('mean', 'rms', 'minimum', 'maximum', 'amplitude'):
        a, b = np.array(s_got['statistics'][stat]), np.array(s_ref['statistics'][stat])
        assert np.max(np.abs(a - b)) < 1e-8 * max(1.0, np.max(np.abs(b))), stat
    m_got = json.loads((out / 'mean_observables.json').read_text())
    m_ref = json.loads(str(G['mean_observables']))
    for key in ('p_front_mean', 'p_back_mean', 'delta_p_mean'):
        assert abs(m_got[key] - m_ref[key]) < 1e-8 * max(1.0, abs(m_ref[key])), key
    assert np.max(np.abs(np.array(m_got['u_centerline_mean']) - m_ref['u_centerline_mean'])) < 1e-9
    assert m_got['recirculation']['status'] == m_ref['recirculation']['status']
    # a restart from the run's own checkpoint cannot cover the sample window again
    with pytest.raises(ValueError, match='Window'):
        runner.run(cfg, tmp_path / 'again', restart=out / 'checkpoint.npz')
