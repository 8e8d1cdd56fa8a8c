"""Pin the CPU oracle to golden vectors produced by the reference's own code.

The fixtures in tests/golden were written by tests/golden/make_golden.py, which
runs the reference solver (numba replaced by plain Python).  Indices and
stencils must match exactly; fields are compared at 1e-12 relative.
"""
import numpy as np
import pytest

import ghost_oracle as go
from conftest import GOLDEN

REL = 1e-12


def close(a, b, rel=REL):
    scale = max(1.0, float(np.max(np.abs(b)))) if np.size(b) else 1.0
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b)))) <= rel * scale


def ghost_part(E, ids):
    E = E.tocsr()
    ident = np.zeros(E.shape[0], bool)
    ident[ids] = True
    rows = np.flatnonzero(~ident & (np.diff(E.indptr) > 0))
    sub = E[rows]
    sub.sort_indices()
    return rows, sub


@pytest.fixture(scope='module')
def small():
    return np.load(GOLDEN / 'small_88x16.npz')


def test_small_geometry_bit_exact(small):
    c = go.CylinderCase(nx=88, ny=16, Lx=22., Ly=4.1, xc=2., yc=2.)
    o = c.ops
    for name in ('ui', 'vi', 'pi'):
        assert np.array_equal(getattr(o, name), small[name]), name
    for key, E, ids in (('Eu', o.Eu, o.ui), ('Ev', o.Ev, o.vi), ('P', o.P, o.pi)):
        rows, sub = ghost_part(E, ids)
        assert np.array_equal(rows, small[f'{key}__rows'])
        assert np.array_equal(sub.indptr, small[f'{key}__indptr'])
        assert np.array_equal(sub.indices, small[f'{key}__cols'])
        assert close(sub.data, small[f'{key}__vals'], 1e-15)
    rect = go.rectangle(c.nx, c.ny, c.dx, c.dy, 'pressure', rho=c.rho)[0]
    assert np.array_equal(go.schur_rows(o.A, o.pi, rect)[0], small['schur_rows_p'])


def test_small_operators(small):
    c = go.CylinderCase(nx=88, ny=16, Lx=22., Ly=4.1, xc=2., yc=2.)
    o = c.ops
    q = small['q']
    assert close(o.advection(q), small['advection'])
    assert close(o.diffusion(q), small['diffusion'])
    assert close(o.gradient(small['p_rand']), small['gradient'])
    assert close(o.divergence(q), small['divergence'])
    assert close(o.H_matvec(q, 0.003), small['H_q'])
    u, v = o.unpack(q)
    assert close(u, small['unpack_u']) and close(v, small['unpack_v'])
    pq, phi = o.project(q, .003)
    assert close(pq, small['project_q']) and close(phi, small['project_phi'])
    assert close(o.pressure_solve(small['rhs_p']), small['sol_p'])
    assert close(c.u, small['init_u']) and close(c.v, small['init_v'])


def test_small_steps_and_forces(small):
    c = go.CylinderCase(nx=88, ny=16, Lx=22., Ly=4.1, xc=2., yc=2.)
    for k in range(5):
        c.solve(1, .001)
        d = c.last_step_diagnostics
        assert close(c.u, small['step_u'][k]) and close(c.v, small['step_v'][k])
        assert close(c.p, small['step_p'][k])
        sc = small['step_scalars'][k]
        assert abs(d['cd'] - sc[0]) <= 1e-12 and abs(d['cl'] - sc[1]) <= 1e-12
        assert d['max_divergence'] < 1e-10
    assert close(c.ops.surface_forces(c.u, c.v, c.p, c.nu * c.rho), small['forces'])
    stats = go.mac_divergence_stats(c.u, c.v, c.dx, c.dy, c.mask)
    assert close([stats[0], stats[1], stats[3]], small['mac_divergence'], 1e-10)
    assert [stats[2], stats[4]] == list(small['mac_divergence_counts'])


@pytest.mark.parametrize('tag,opts', [('bq', dict(ghost_velocity_interpolation='biquadratic')),
                                      ('qp', dict(ghost_pressure_extension='quadratic')),
                                      ('iter', dict(pressure_solver='iterative'))])
def test_option_paths(tag, opts):
    G = np.load(GOLDEN / f'opt40x30_{tag}.npz')
    c = go.CylinderCase(nx=40, ny=30, Lx=4., Ly=3., xc=1.5, yc=1.5, **opts)
    for key, E, ids in (('Eu', c.ops.Eu, c.ops.ui), ('P', c.ops.P, c.ops.pi)):
        rows, sub = ghost_part(E, ids)
        assert np.array_equal(rows, G[f'{key}__rows']) and np.array_equal(sub.indices, G[f'{key}__cols'])
    c.solve(3, .001)
    assert close(c.u, G['u'], 1e-10) and close(c.p, G['p'], 1e-9)
    assert abs(c.last_step_diagnostics['cd'] - G['scalars'][0]) < 1e-10


def test_traction_known_answer():
    G = np.load(GOLDEN / 'traction.npz')
    for k, (nx, ny) in enumerate(((40, 30), (80, 60), (120, 90))):
        c = go.CylinderCase(nx=nx, ny=ny, Lx=4., Ly=3., xc=1.5, yc=1.5)
        xu, yu = c.ops.coords['u']
        xv, yv = c.ops.coords['v']
        xx, yy = np.meshgrid(xu, yu)
        rr = np.hypot(xx - c.xc, yy - c.yc)
        u = -(rr - c.D / 2) * (yy - c.yc) / rr
        xx, yy = np.meshgrid(xv, yv)
        rr = np.hypot(xx - c.xc, yy - c.yc)
        v = (rr - c.D / 2) * (xx - c.xc) / rr
        p = np.broadcast_to(c.ops.coords['p'][0], c.p.shape)
        f = c.ops.surface_forces(u, v, p, c.nu * c.rho)
        assert close(f, G['forces'][k])
        assert abs(f[2] + np.pi * (c.D / 2) ** 2) < 1e-10 and abs(f[3]) < 1e-10


def test_rectangle_transforms():
    G = np.load(GOLDEN / 'rectangle_24x10.npz')
    for kind in ('pressure', 'u', 'v'):
        _, solve, _ = go.rectangle(24, 10, 0.3, 0.25, kind, 0.02, 0.004, 1.3)
        assert close(solve(G[f'{kind}_in'].copy()), G[f'{kind}_out'])


def test_config1_two_steps():
    G = np.load(GOLDEN / 'config1_400x200.npz')
    c = go.CylinderCase(nx=400, ny=200, Lx=20., Ly=10., D=1., xc=5., yc=5., nu=1 / 40)
    assert len(c.ops.ui) == G['ui_count'] and len(c.ops.pi) == G['pi_count']
    assert np.array_equal(np.packbits(np.isin(np.arange(c.u.size), c.ops.ui)), G['ui'])
    assert np.array_equal(np.packbits(np.isin(np.arange(c.p.size), c.ops.pi)), G['pi'])
    q = c.ops.pack(c.u, c.v)
    q += 1e-3 * np.random.default_rng(0).standard_normal(q.size)
    c.u, c.v = c.ops.unpack(q)
    for k in range(2):
        c.solve(1, .002)
        assert close(c.u.ravel()[G['sample_u']], G['u_samples'][k])
        assert close(c.p.ravel()[G['sample_p']], G['p_samples'][k])
        assert abs(c.last_step_diagnostics['cd'] - G['scalars'][k][0]) < 1e-12
    assert c.ops.pressure_info['rank'] == G['pressure_rank']
    assert [i['rank'] for i in c.ops.helmholtz_info] == list(G['helmholtz_ranks'])


def test_taylor_green_oracle_matches_reference():
    """The oracle's periodic Taylor-Green run against the reference's own
    verification/taylor_green.run (tests/golden/taylor_green.npz; the reference solves the
    CN system with GMRES to rtol 1e-12, the oracle exactly in Fourier space)."""
    G = np.load(GOLDEN / 'taylor_green.npz')
    for tag in ('n16', 'n32'):
        n, dt, end, nu = G[f'{tag}_params']
        info, q, p = go.taylor_green_run(int(n), dt, end, nu)
        assert np.max(np.abs(q - G[f'{tag}_q'])) < 1e-12 * np.max(np.abs(G[f'{tag}_q']))
        assert np.max(np.abs(p - G[f'{tag}_p'])) < 1e-11 * np.max(np.abs(G[f'{tag}_p']))
        norms = np.array([info['velocity'][k] for k in ('l1', 'l2', 'linf')] +
                         [info['pressure'][k] for k in ('l1', 'l2', 'linf')])
        np.testing.assert_allclose(norms, G[f'{tag}_norms'][:6], rtol=1e-9)
        assert info['max_divergence'] < 1e-10


def test_periodic_metrics_matches_reference():
    """The host-side force-history analysis against the reference's periodic_metrics on seeded
    synthetic series (tests/golden/analysis.npz)."""
    import importlib.util
    from pathlib import Path
    spec = importlib.util.spec_from_file_location(
        'gm_analysis', Path(__file__).resolve().parents[1] / 'cfd-cylinder-flow-ghost-cell_gb300' / 'analysis.py')
    an = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(an)
    G = np.load(GOLDEN / 'analysis.npz')
    t, cd, cl = G['t'], G['cd'], G['cl']
    cases = ((t, cd, cl, 5.0), (t[:200], cd[:200], cl[:200] * 0 + 1e-3 * t[:200], 0.0))
    for (tt, a, b, ts), want in zip(cases, G['values']):
        m = an.periodic_metrics(tt, a, b, ts, D=1.0, U_ref=1.0)
        got = np.array([float(m[str(k)]) for k in G['keys']])
        np.testing.assert_allclose(got, want, rtol=1e-12, atol=1e-14, equal_nan=True)
    with pytest.raises(ValueError):
        an.periodic_metrics([0, 1], [1, 1], [0, 0], 0.0)


def test_grid_convergence_index_matches_reference():
    """calculate_gci against the reference's own results (tests/golden/analysis.npz): equal and
    unequal refinement ratios and the non-estimable branches."""
    import importlib.util
    import json
    from pathlib import Path
    spec = importlib.util.spec_from_file_location(
        'gm_analysis', Path(__file__).resolve().parents[1] / 'cfd-cylinder-flow-ghost-cell_gb300' / 'analysis.py')
    an = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(an)
    G = np.load(GOLDEN / 'analysis.npz')
    for case, want in zip(json.loads(str(G['gci_cases'])), json.loads(str(G['gci']))):
        got = an.calculate_gci(*case[:3], r=case[3], Fs=case[4], r32=case[5])
        assert set(got) == set(want), case
        for k, v in want.items():
            if isinstance(v, float):
                assert abs(got[k] - v) <= 1e-12 * max(1.0, abs(v)), (case, k)
            else:
                assert got[k] == v, (case, k)
    with pytest.raises(ValueError, match='GCI requires'):
        an.calculate_gci(1.0, 1.1, 1.2, r=1.0)
    with pytest.raises(ValueError, match='coarser spacing'):
        an.calculate_gci(1.0, 1.1, 1.2, r32=0.5)
