"""FGMRES(50) with its control on the device (restart cycles as a graph WHILE node, Arnoldi
steps as IF nodes, rotations and the least-squares update in one-thread kernels) against the
host-controlled loop it replaces (GHOSTMAC_GMRES_HOST=1): the same kernels and scalar
arithmetic in the same order, so the iteration counts are identical and the solutions agree to
rounding (the rotations' hypot and the contraction of their products into FMAs differ between
the device and the host compiler, last bits only); and both
against the direct FFT + boundary Schur solve (the reference asserts 1e-9 between its two
backends, tests/test_gemini_followup.py:60-61)."""
import numpy as np
import pytest

from conftest import load_package

pytestmark = pytest.mark.gpu

CASES = [dict(nx=88, ny=16, Lx=22., Ly=4.1, xc=2., yc=2.),
         dict(nx=400, ny=200, Lx=20., Ly=10., D=1., xc=5., yc=5., nu=1 / 40)]


@pytest.fixture(scope='module')
def pkg():
    return load_package()


@pytest.mark.parametrize('precision', ['fp64', 'fp32'])
@pytest.mark.parametrize('kw', CASES, ids=['88x16', '400x200'])
def test_device_control_equals_host_control(pkg, monkeypatch, kw, precision):
    b = None
    out = {}
    for tag, env in (('device', None), ('host', '1')):
        if env is None:
            monkeypatch.delenv('GHOSTMAC_GMRES_HOST', raising=False)
        else:
            monkeypatch.setenv('GHOSTMAC_GMRES_HOST', env)
        s = pkg.MAC_CylinderFlow(boundary='ghost_cell', time_scheme='ab2_cn', verbose=False, pressure_solver='iterative', precision=precision, **kw)
        if b is None:
            b = np.random.default_rng(11).standard_normal(len(s.gg.pi))
        x1 = s.gg.pressure_solve(b)
        info1 = dict(s.gg.pressure_inverse_info['last_solve'])
        x2 = s.gg.pressure_solve(2.0 * b)  # a second right-hand side through the same graph
        out[tag] = (x1, info1, x2)
    assert out['device'][1]['iterations'] == out['host'][1]['iterations'] > 0
    for k in (0, 2):
        ref = out['host'][k]
        assert np.max(np.abs(out['device'][k] - ref)) < 1e-12 * max(1.0, np.max(np.abs(ref)))
    d = pkg.MAC_CylinderFlow(boundary='ghost_cell', time_scheme='ab2_cn', verbose=False, **kw)
    xd = d.gg.pressure_solve(b)
    assert np.max(np.abs(out['device'][0] - xd)) < 1e-9 * max(1.0, np.max(np.abs(xd)))


def test_device_control_steps(pkg, monkeypatch):
    """Ten AB2/CN steps with the iterative pressure path: device and host control give the same
    GMRES iteration counts and the same fields to rounding."""
    res = []
    for env in (None, '1'):
        if env is None:
            monkeypatch.delenv('GHOSTMAC_GMRES_HOST', raising=False)
        else:
            monkeypatch.setenv('GHOSTMAC_GMRES_HOST', env)
        s = pkg.MAC_CylinderFlow(boundary='ghost_cell', time_scheme='ab2_cn', verbose=False, pressure_solver='iterative', **CASES[0])
        s.solve(n_steps=10, dt=.002, perturb_transient=False, save_artifacts=False, verbose=False)
        assert s.last_step_diagnostics['max_divergence'] < 1e-10
        res.append((s.u.copy(), s.v.copy(), s.p.copy(), s.last_step_diagnostics['pressure_iterations']))
    for a, c in zip(res[0][:3], res[1][:3]):
        assert np.max(np.abs(a - c)) < 1e-11 * max(1.0, np.max(np.abs(c)))
    assert res[0][3] == res[1][3]
