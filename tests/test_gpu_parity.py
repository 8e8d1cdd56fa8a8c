"""GPU parity of libghostmac.so against the oracle and the reference's golden vectors.

Every comparison goes through the C ABI (ctypes) on a GB300.  Tolerances
(max-norm, relative to max(1, |reference|)):
  single operators, Helmholtz transforms ...... 1e-12
  pressure rectangle inverse ................... 1e-10 (condition number up to 1e6)
  projected fields, pressure solves ........... 1e-11
  fields after a few AB2/CN steps ............. 1e-10
  force coefficients .......................... 1e-8 (relative)
  discrete divergence ......................... < 1e-10 absolute
Indices and stencils are compared bit-exactly by tests/test_geometry_host.py.
"""
import numpy as np
import pytest

import ghost_oracle as go
from conftest import GOLDEN, load_package

pytestmark = pytest.mark.gpu


# The pressure rectangle (Neumann walls, Dirichlet outlet) has condition ~(L/h)^2 up to 1e6:
# two backward-stable inverses agree to ~cond * eps, not to eps.  Helmholtz rectangles are
# well conditioned.
RECT_TOL = dict(pressure=1e-10, u=1e-12, v=1e-12)


def rel(a, b):
    a, b = np.asarray(a, float), np.asarray(b, float)
    return float(np.max(np.abs(a - b))) / max(1.0, float(np.max(np.abs(b))))


@pytest.fixture(scope='module')
def pkg():
    return load_package()


def small(pkg, **kw):
    return pkg.MAC_CylinderFlow(boundary='ghost_cell', time_scheme='ab2_cn', nx=88, ny=16, Lx=22., Ly=4.1, xc=2., yc=2., verbose=False, **kw)


@pytest.fixture(scope='module')
def G():
    return np.load(GOLDEN / 'small_88x16.npz')


def test_rectangle_transforms(pkg):
    G = np.load(GOLDEN / 'rectangle_24x10.npz')
    s = pkg.MAC_CylinderFlow(boundary='ghost_cell', time_scheme='ab2_cn', nx=24, ny=10, Lx=7.2, Ly=2.5, D=0.4, xc=3.6, yc=1.25, nu=0.02, rho=1.3, verbose=False)
    for kind in ('pressure', 'u', 'v'):
        x = s.gg.rectangle_solve(kind, G[f'{kind}_in'], dt=0.004)
        assert rel(x, G[f'{kind}_out']) < RECT_TOL[kind], kind


@pytest.mark.parametrize('n', [(40, 30, 0.5), (88, 16, 0.3), (400, 200, 1.0), (256, 128, 1.0), (820, 410, 1.0)])
def test_rectangle_transforms_sizes(pkg, n):
    nx, ny, D = n
    h = 0.05
    s = pkg.MAC_CylinderFlow(boundary='ghost_cell', time_scheme='ab2_cn', nx=nx, ny=ny, Lx=nx * h, Ly=ny * h, D=D, xc=nx * h / 4, yc=ny * h / 2, nu=0.01,
                             verbose=False)
    rng = np.random.default_rng(nx)
    for kind in ('pressure', 'u', 'v'):
        _, solve, shape = go.rectangle(nx, ny, s.dx, s.dy, kind, 0.01, 0.002, 1.0, self_check=False)
        b = rng.normal(size=shape)
        assert rel(s.gg.rectangle_solve(kind, b, dt=0.002), solve(b.copy())) < RECT_TOL[kind], kind


def test_operators_match_golden(pkg, G):
    s = small(pkg)
    g = s.gg
    assert np.array_equal(g.ui, G['ui']) and np.array_equal(g.pi, G['pi'])
    q = G['q']
    assert rel(g.advection(q), G['advection']) < 1e-12
    assert rel(g.diffusion(q), G['diffusion']) < 1e-12
    assert rel(g.gradient(G['p_rand']), G['gradient']) < 1e-12
    assert rel(g.divergence(q), G['divergence']) < 1e-12
    assert rel(g.H_matvec(q, 0.003), G['H_q']) < 1e-12
    u, v = g.unpack(q)
    assert rel(u, G['unpack_u']) < 1e-14 and rel(v, G['unpack_v']) < 1e-14
    assert rel(g.pack(u, v), q) == 0.0
    assert rel(g.pressure_solve(G['rhs_p']), G['sol_p']) < 1e-11
    pq, phi = g.project(q, .003)
    assert rel(pq, G['project_q']) < 1e-11 and rel(phi, G['project_phi']) < 1e-11
    assert np.max(np.abs(g.divergence(pq))) < 1e-10
    assert rel(s.u, G['init_u']) < 1e-12 and rel(s.v, G['init_v']) < 1e-12


def test_steps_match_golden(pkg, G):
    s = small(pkg)
    for k in range(5):
        s.solve(n_steps=1, dt=.001, perturb_transient=False, save_artifacts=False, verbose=False)
        d = s.last_step_diagnostics
        sc = G['step_scalars'][k]
        assert rel(s.u, G['step_u'][k]) < 1e-10, k
        assert rel(s.v, G['step_v'][k]) < 1e-10, k
        assert rel(s.p, G['step_p'][k]) < 1e-10, k
        assert abs(d['cd'] - sc[0]) <= 1e-8 * abs(sc[0]) and abs(d['cl'] - sc[1]) <= 1e-8 * max(abs(sc[1]), 1e-3)
        assert d['max_divergence'] < 1e-10
    assert rel(s.gg.surface_forces(s.u, s.v, s.p, s.nu * s.rho), G['forces']) < 1e-10
    stats = s.divergence_stats()
    assert abs(stats[0] - G['mac_divergence'][0]) < 1e-12
    assert [stats[2], stats[4]] == list(G['mac_divergence_counts'])


def test_state_arrays_page_locked(pkg):
    """The facade's u, v, p live in page-locked memory (gm_host_alloc), and the state copies
    through them are exact: a state written in place comes back unchanged, and a case stepped
    from ordinary (pageable) copies of it gives bitwise the same fields."""
    import ctypes
    a = small(pkg)
    for key in ('u', 'v', 'p'):
        base = getattr(a, key)
        while isinstance(base, np.ndarray):
            base = base.base
        assert isinstance(base, ctypes.Array), key
    rng = np.random.default_rng(3)
    a.v[1:-1] += 1e-3 * rng.standard_normal(a.v[1:-1].shape)
    a._push()  # the device keeps the active entries and rebuilds ghosts and inlet
    a._pull()
    ref = {k: getattr(a, k).copy() for k in ('u', 'v', 'p')}
    a._push()
    a._pull()
    for key in ('u', 'v', 'p'):
        assert np.array_equal(getattr(a, key), ref[key]), key
    b = small(pkg)
    b.u, b.v, b.p = (ref[k].copy() for k in ('u', 'v', 'p'))
    assert b.u.flags.owndata
    a.solve(n_steps=3, dt=.001, perturb_transient=False, save_artifacts=False, verbose=False)
    b.solve(n_steps=3, dt=.001, perturb_transient=False, save_artifacts=False, verbose=False)
    for key in ('u', 'v', 'p'):
        assert np.array_equal(getattr(a, key), getattr(b, key)), key


def test_multi_step_call_equals_single_steps(pkg):
    a, b = small(pkg), small(pkg)
    a.solve(n_steps=6, dt=.001, perturb_transient=False, save_artifacts=False, verbose=False)
    for _ in range(6):
        b.solve(n_steps=1, dt=.001, perturb_transient=False, save_artifacts=False, verbose=False)
    for key in ('u', 'v', 'p'):
        assert np.array_equal(getattr(a, key), getattr(b, key)), key


@pytest.mark.parametrize('tag,opts', [('bq', dict(ghost_velocity_interpolation='biquadratic')),
                                      ('qp', dict(ghost_pressure_extension='quadratic'))])
def test_option_paths(pkg, tag, opts):
    G = np.load(GOLDEN / f'opt40x30_{tag}.npz')
    s = pkg.MAC_CylinderFlow(boundary='ghost_cell', time_scheme='ab2_cn', nx=40, ny=30, Lx=4., Ly=3., xc=1.5, yc=1.5, verbose=False, **opts)
    s.solve(n_steps=3, dt=.001, perturb_transient=False, save_artifacts=False, verbose=False)
    assert rel(s.u, G['u']) < 1e-10 and rel(s.p, G['p']) < 1e-9
    assert abs(s.last_step_diagnostics['cd'] - G['scalars'][0]) < 1e-8 * abs(G['scalars'][0])
    assert s.last_step_diagnostics['max_divergence'] < 1e-10


def test_traction_known_answers(pkg):
    G = np.load(GOLDEN / 'traction.npz')
    for k, (nx, ny) in enumerate(((40, 30), (80, 60), (120, 90))):
        s = pkg.MAC_CylinderFlow(boundary='ghost_cell', time_scheme='ab2_cn', nx=nx, ny=ny, Lx=4., Ly=3., xc=1.5, yc=1.5, verbose=False)
        xu, yu = np.arange(nx + 1) * s.dx, (np.arange(ny) + .5) * s.dy
        xv, yv = (np.arange(nx) + .5) * s.dx, np.arange(ny + 1) * s.dy
        xx, yy = np.meshgrid(xu, yu)
        rr = np.hypot(xx - s.xc, yy - s.yc)
        u = -(rr - s.D / 2) * (yy - s.yc) / rr
        xx, yy = np.meshgrid(xv, yv)
        rr = np.hypot(xx - s.xc, yy - s.yc)
        v = (rr - s.D / 2) * (xx - s.xc) / rr
        p = np.ascontiguousarray(np.broadcast_to(xv, s.p.shape))
        f = s.gg.surface_forces(u, v, p, s.nu * s.rho)
        assert rel(f, G['forces'][k]) < 1e-12
        assert abs(f[2] + np.pi * (s.D / 2) ** 2) < 1e-10 and abs(f[3]) < 1e-10


def test_config1_two_steps(pkg):
    G = np.load(GOLDEN / 'config1_400x200.npz')
    s = pkg.MAC_CylinderFlow(boundary='ghost_cell', time_scheme='ab2_cn', nx=400, ny=200, Lx=20., Ly=10., D=1., xc=5., yc=5., nu=1 / 40, verbose=False)
    q = s.gg.pack(s.u, s.v)
    q += 1e-3 * np.random.default_rng(0).standard_normal(q.size)
    s.u[:], s.v[:] = s.gg.unpack(q)
    for k in range(2):
        s.solve(n_steps=1, dt=.002, perturb_transient=False, save_artifacts=False, verbose=False)
        assert rel(s.u.ravel()[G['sample_u']], G['u_samples'][k]) < 1e-10
        assert rel(s.v.ravel()[G['sample_v']], G['v_samples'][k]) < 1e-10
        assert rel(s.p.ravel()[G['sample_p']], G['p_samples'][k]) < 1e-10
        d = s.last_step_diagnostics
        assert abs(d['cd'] - G['scalars'][k][0]) < 1e-8 * abs(G['scalars'][k][0])
        assert d['max_divergence'] < 1e-10


def test_oracle_parity_with_noise_20_steps(pkg):
    """Same seeded inputs through the oracle and the GPU for 20 steps (tolerance 1e-10)."""
    kw = dict(nx=88, ny=16, Lx=22., Ly=4.1, xc=2., yc=2., nu=0.02)
    s = pkg.MAC_CylinderFlow(boundary='ghost_cell', time_scheme='ab2_cn', verbose=False, **kw)
    c = go.CylinderCase(**kw)
    q = c.ops.pack(c.u, c.v)
    q += 1e-2 * np.random.default_rng(5).standard_normal(q.size)
    c.u, c.v = c.ops.unpack(q)
    s.u[:], s.v[:] = c.u, c.v
    s.solve(n_steps=20, dt=.002, perturb_transient=False, save_artifacts=False, verbose=False)
    c.solve(20, .002)
    for key in ('u', 'v', 'p'):
        assert rel(getattr(s, key), getattr(c, key)) < 1e-10, key
    assert abs(s.last_step_diagnostics['cd'] / c.last_step_diagnostics['cd'] - 1) < 1e-8


def test_checkpoint_restart(pkg, tmp_path):
    cont, div = small(pkg), small(pkg)
    cont.solve(n_steps=20, dt=.001, perturb_transient=False, save_artifacts=False, verbose=False)
    div.solve(n_steps=7, dt=.001, perturb_transient=False, save_artifacts=False, verbose=False)
    path = tmp_path / 'ck.npz'
    div.save_checkpoint(path)
    res = pkg.MAC_CylinderFlow.from_checkpoint(path)
    res.solve(n_steps=13, dt=.001, perturb_transient=False, save_artifacts=False, verbose=False)
    for key in ('u', 'v', 'p'):
        assert np.max(np.abs(getattr(cont, key) - getattr(res, key))) < 1e-11, key
    with np.load(path, allow_pickle=False) as data:
        arrays = {k: data[k].copy() for k in data.files if k != 'half_pressure'}
    np.savez(path, **arrays)
    with pytest.raises(ValueError):
        pkg.MAC_CylinderFlow.from_checkpoint(path)


def test_gates_raise(pkg):
    s = small(pkg)
    with pytest.raises(RuntimeError):
        s.solve(n_steps=1, dt=1.0, perturb_transient=False, save_artifacts=False, verbose=False)
    s = small(pkg)
    s.u[3, 5] = np.nan
    with pytest.raises((ValueError, RuntimeError)):
        s.solve(n_steps=1, dt=.001, perturb_transient=False, save_artifacts=False, verbose=False)
    s = small(pkg)
    s.solve(n_steps=2, dt=.001, perturb_transient=False, save_artifacts=False, verbose=False)
    assert s.last_step_diagnostics['max_divergence'] < 1e-10


# ---------------------------------------------------------------------------
# FP32 separable inverses with FP64 refinement
# ---------------------------------------------------------------------------
def test_fp32_mode_matches_fp64_oracle(pkg):
    """FP32 inverses and stencils refined against the FP64 operators: same gates, divergence
    < 1e-10; after 20 noisy steps velocity within 1e-7, pressure within 1e-5 and the drag
    coefficient within 1e-6 (relative) of the FP64 oracle."""
    kw = dict(nx=88, ny=16, Lx=22., Ly=4.1, xc=2., yc=2., nu=0.02)
    s = pkg.MAC_CylinderFlow(boundary='ghost_cell', time_scheme='ab2_cn', verbose=False, precision='fp32', **kw)
    c = go.CylinderCase(**kw)
    q = c.ops.pack(c.u, c.v)
    q += 1e-2 * np.random.default_rng(5).standard_normal(q.size)
    c.u, c.v = c.ops.unpack(q)
    s.u[:], s.v[:] = c.u, c.v
    s.solve(n_steps=20, dt=.002, perturb_transient=False, save_artifacts=False, verbose=False)
    c.solve(20, .002)
    d = s.last_step_diagnostics
    assert d['max_divergence'] < 1e-10
    for key in ('u', 'v'):
        assert rel(getattr(s, key), getattr(c, key)) < 1e-7, key
    assert rel(s.p, c.p) < 1e-5
    assert abs(d['cd'] / c.last_step_diagnostics['cd'] - 1) < 1e-6
    assert d['pressure_refinement_iterations'] >= 1


def test_fp32_mode_config1(pkg):
    G = np.load(GOLDEN / 'config1_400x200.npz')
    s = pkg.MAC_CylinderFlow(boundary='ghost_cell', time_scheme='ab2_cn', nx=400, ny=200, Lx=20., Ly=10., D=1., xc=5., yc=5., nu=1 / 40, verbose=False,
                             precision='fp32')
    q = s.gg.pack(s.u, s.v)
    q += 1e-3 * np.random.default_rng(0).standard_normal(q.size)
    s.u[:], s.v[:] = s.gg.unpack(q)
    for k in range(2):
        s.solve(n_steps=1, dt=.002, perturb_transient=False, save_artifacts=False, verbose=False)
        assert rel(s.u.ravel()[G['sample_u']], G['u_samples'][k]) < 1e-7
        assert rel(s.p.ravel()[G['sample_p']], G['p_samples'][k]) < 1e-5
        d = s.last_step_diagnostics
        assert abs(d['cd'] - G['scalars'][k][0]) < 1e-6 * abs(G['scalars'][k][0])
        assert d['max_divergence'] < 1e-10


def test_iterative_pressure_path_golden(pkg):
    """pressure_solver='iterative' (GMRES with the rectangle preconditioner) against the
    reference's own three steps (tests/golden/opt40x30_iter.npz).  GMRES stops at
    rtol = 1e-12 plus refinement, so the fields agree to the solver tolerance."""
    G = np.load(GOLDEN / 'opt40x30_iter.npz')
    s = pkg.MAC_CylinderFlow(boundary='ghost_cell', time_scheme='ab2_cn', nx=40, ny=30, Lx=4., Ly=3., xc=1.5, yc=1.5, verbose=False, pressure_solver='iterative')
    s.solve(n_steps=3, dt=.001, perturb_transient=False, save_artifacts=False, verbose=False)
    assert rel(s.u, G['u']) < 1e-9 and rel(s.v, G['v']) < 1e-9 and rel(s.p, G['p']) < 1e-8
    assert abs(s.last_step_diagnostics['cd'] - G['scalars'][0]) < 1e-8 * abs(G['scalars'][0])
    d = s.last_step_diagnostics
    assert d['max_divergence'] < 1e-10 and d['pressure_backend'] == 'gmres_rectangle'
    assert d['pressure_iterations'] > 0


def test_iterative_matches_direct_solve(pkg):
    """GMRES and the FFT + boundary Schur direct solve agree (the reference asserts 1e-9 /
    1e-8 between its two backends)."""
    kw = dict(nx=88, ny=16, Lx=22., Ly=4.1, xc=2., yc=2., verbose=False)
    sd = pkg.MAC_CylinderFlow(boundary='ghost_cell', time_scheme='ab2_cn', **kw)
    si = pkg.MAC_CylinderFlow(boundary='ghost_cell', time_scheme='ab2_cn', pressure_solver='iterative', **kw)
    rng = np.random.default_rng(3)
    b = rng.standard_normal(len(sd.gg.pi))
    xd = sd.gg.pressure_solve(b)
    xi = si.gg.pressure_solve(b)
    assert np.max(np.abs(xd - xi)) < 1e-9 * max(1.0, np.max(np.abs(xd)))
    for prec in ('fp32',):
        sf = pkg.MAC_CylinderFlow(boundary='ghost_cell', time_scheme='ab2_cn', pressure_solver='iterative', precision=prec, **kw)
        xf = sf.gg.pressure_solve(b)
        assert np.max(np.abs(xf - xd)) < 1e-8 * max(1.0, np.max(np.abs(xd)))


def test_fp32_helmholtz_jacobi_and_fft_inverse(pkg, monkeypatch):
    """The FP32 mode applies its CN Helmholtz inverse by FP32 Jacobi iterations when the row-sum
    norm of the Jacobi iteration matrix is below 1/4 (about 4 dt nu / 2 / h^2); the FFT and
    boundary-Schur inverse (GHOSTMAC_HELM_JACOBI=0) gives the same fields to the mode's
    tolerances.  Both against the FP64 oracle after 20 noisy steps: velocity 1e-7, pressure
    1e-5, drag 1e-6 relative, divergence < 1e-10."""
    kw = dict(nx=88, ny=16, Lx=22., Ly=4.1, xc=2., yc=2., nu=0.02)
    c = go.CylinderCase(**kw)
    q = c.ops.pack(c.u, c.v)
    q += 1e-2 * np.random.default_rng(5).standard_normal(q.size)
    c.u, c.v = c.ops.unpack(q)
    u0, v0 = c.u.copy(), c.v.copy()
    c.solve(20, .002)
    for env, expect_jacobi in ((None, True), ('0', False)):
        if env is None:
            monkeypatch.delenv('GHOSTMAC_HELM_JACOBI', raising=False)
        else:
            monkeypatch.setenv('GHOSTMAC_HELM_JACOBI', env)
        s = pkg.MAC_CylinderFlow(boundary='ghost_cell', time_scheme='ab2_cn', verbose=False, precision='fp32', **kw)
        s.u[:], s.v[:] = u0, v0
        s.solve(n_steps=20, dt=.002, perturb_transient=False, save_artifacts=False, verbose=False)
        info = s.helmholtz_solver_info()
        assert (info['jacobi_iters'] > 0) == expect_jacobi, info
        if expect_jacobi:
            assert 0 < info['jacobi_rho'] < 0.25
        d = s.last_step_diagnostics
        assert d['max_divergence'] < 1e-10
        assert rel(s.u, c.u) < 1e-7 and rel(s.v, c.v) < 1e-7 and rel(s.p, c.p) < 1e-5
        assert abs(d['cd'] / c.last_step_diagnostics['cd'] - 1) < 1e-6


@pytest.mark.parametrize('kw', [dict(nx=88, ny=16, Lx=22., Ly=4.1, xc=2., yc=2., nu=0.02),
                                dict(nx=400, ny=200, Lx=20., Ly=10., D=1., xc=5., yc=5., nu=1 / 40)])
def test_fp32_helmholtz_jacobi_tiled_equals_launches(pkg, monkeypatch, kw):
    """The temporally blocked Jacobi application (one launch, iterations in shared memory) gives
    bitwise the fields of one launch per iteration over the whole grid."""
    out = []
    for tiled in ('1', '0'):
        monkeypatch.setenv('GHOSTMAC_HELM_JACOBI_TILED', tiled)
        s = pkg.MAC_CylinderFlow(boundary='ghost_cell', time_scheme='ab2_cn', verbose=False, precision='fp32', **kw)
        q = s.gg.pack(s.u, s.v)
        q += 1e-2 * np.random.default_rng(11).standard_normal(q.size)
        s.u[:], s.v[:] = s.gg.unpack(q)
        s.solve(n_steps=8, dt=.002, perturb_transient=False, save_artifacts=False, verbose=False)
        assert s.helmholtz_solver_info()['jacobi_iters'] > 0
        out.append((s.u.copy(), s.v.copy(), s.p.copy()))
    for a, b in zip(*out):
        assert np.array_equal(a, b)
