"""The AB2 momentum right-hand side from shared-memory tiles (k_momentum_tiled: each corner and
centre flux formed once and shared by the faces that use it) against the one-thread-per-face
kernel (GHOSTMAC_MOMENTUM_TILED=0), both through whole AB2/CN steps.  The flux formulas are
those of solver/numba_kernels.py:17-142; only the rounding of the shared products may differ
(an FMA contracted in one kernel and not the other), so the fields agree to 1e-13 in FP64 and
to the FP32 mode's own tolerance (1e-7) there; both stay within the golden tolerances of
test_gpu_parity.py, which run the tiled kernel."""
import numpy as np
import pytest

from conftest import load_package

pytestmark = pytest.mark.gpu

CASES = [dict(nx=88, ny=16, Lx=22., Ly=4.1, xc=2., yc=2., nu=0.02),
         dict(nx=400, ny=200, Lx=20., Ly=10., D=1., xc=5., yc=5., nu=1 / 40),
         dict(nx=800, ny=820, Lx=40., Ly=41., D=1., xc=10., yc=20.5, nu=1 / 100)]


def rel(a, b):
    return float(np.max(np.abs(a - b))) / max(1.0, float(np.max(np.abs(b))))


@pytest.fixture(scope='module')
def pkg():
    return load_package()


@pytest.mark.parametrize('precision', ['fp64', 'fp32'])
@pytest.mark.parametrize('kw', CASES, ids=['88x16', '400x200', '800x820'])
def test_tiled_momentum_equals_per_face(pkg, monkeypatch, kw, precision):
    out = []
    for tiled in ('1', '0'):
        monkeypatch.setenv('GHOSTMAC_MOMENTUM_TILED', tiled)
        s = pkg.MAC_CylinderFlow(boundary='ghost_cell', time_scheme='ab2_cn', verbose=False, precision=precision, **kw)
        q = s.gg.pack(s.u, s.v)
        q += 1e-2 * np.random.default_rng(17).standard_normal(q.size)
        s.u[:], s.v[:] = s.gg.unpack(q)
        s.solve(n_steps=6, dt=.002, perturb_transient=False, save_artifacts=False, verbose=False)
        assert s.last_step_diagnostics['max_divergence'] < 1e-10
        out.append((s.u.copy(), s.v.copy(), s.p.copy(), s.last_step_diagnostics['cd']))
    tol = 1e-13 if precision == 'fp64' else 1e-7
    for a, b in zip(out[0][:2], out[1][:2]):
        assert rel(a, b) < tol
    assert rel(out[0][2], out[1][2]) < (1e-11 if precision == 'fp64' else 1e-5)
    assert abs(out[0][3] / out[1][3] - 1) < (1e-11 if precision == 'fp64' else 1e-6)
