"""Many cases per GPU (gm_batch_step): a batch gives every case the same state as stepping
it alone, including the start-up step, graph-replayed steady steps and a dt change."""
import numpy as np
import pytest

from conftest import load_package

pytestmark = pytest.mark.gpu

CASES = [
    dict(nx=88, ny=16, Lx=22., Ly=4.1, xc=2., yc=2., nu=0.02),
    dict(nx=64, ny=32, Lx=6.4, Ly=3.2, D=0.9, xc=1.7, yc=1.55, nu=0.009),
    dict(nx=96, ny=40, Lx=4.8, Ly=2.0, D=0.5, xc=1.2, yc=1.0, nu=0.005, precision='fp32'),
]


def _make(pkg, seed):
    out = []
    for i, kw in enumerate(CASES):
        s = pkg.MAC_CylinderFlow(boundary='ghost_cell', time_scheme='ab2_cn', verbose=False, **kw)
        rng = np.random.default_rng(seed + i)
        q = s.gg.pack(s.u, s.v)
        q += 1e-3 * rng.standard_normal(q.size)
        s.u, s.v = s.gg.unpack(q)
        out.append(s)
    return out


def test_batch_matches_cases_stepped_alone():
    pkg = load_package()
    alone = _make(pkg, 5)
    together = _make(pkg, 5)
    for s in alone:
        s.solve(n_steps=9, dt=0.002, perturb_transient=False, save_artifacts=False, verbose=False)
        s.solve(n_steps=4, dt=0.0015, perturb_transient=False, save_artifacts=False, verbose=False)
    b = pkg.CylinderBatch(together)
    r1 = b.solve(9, dt=0.002)
    r2 = b.solve(4, dt=0.0015)
    for s, t, (ts, cd, cl) in zip(alone, together, r1):
        assert len(ts) == 9 and np.all(np.isfinite(cd))
        np.testing.assert_array_equal(t.u, s.u)
        np.testing.assert_array_equal(t.v, s.v)
        np.testing.assert_array_equal(t.p, s.p)
        assert t.time == pytest.approx(s.time, abs=1e-15)
        assert t.last_step_diagnostics['cd'] == s.last_step_diagnostics['cd']
        assert t.last_step_diagnostics['max_divergence'] < 1e-10
        adv_s, half_s, dt_s = s.gg.history()
        adv_t, half_t, dt_t = t.gg.history()
        np.testing.assert_array_equal(adv_t, adv_s)
        np.testing.assert_array_equal(half_t, half_s)
        assert dt_t == dt_s
    assert all(len(r[0]) == 4 for r in r2)
    b.close()


def test_batch_rejects_duplicates_and_empty():
    pkg = load_package()
    s = pkg.MAC_CylinderFlow(boundary='ghost_cell', time_scheme='ab2_cn', nx=88, ny=16, Lx=22., Ly=4.1, xc=2., yc=2., verbose=False)
    with pytest.raises(ValueError):
        pkg.CylinderBatch([s, s])
    with pytest.raises(ValueError):
        pkg.CylinderBatch([])


GROUPED = [
    dict(nx=64, ny=32, Lx=6.4, Ly=3.2, D=0.9, xc=1.7, yc=1.55, nu=0.009),
    dict(nx=64, ny=32, Lx=6.4, Ly=3.2, D=1.0, xc=1.9, yc=1.65, nu=0.012),
    dict(nx=64, ny=32, Lx=6.4, Ly=3.2, D=0.8, xc=1.6, yc=1.5, nu=0.02),
    dict(nx=96, ny=40, Lx=4.8, Ly=2.0, D=0.5, xc=1.2, yc=1.0, nu=0.005, precision='fp32'),
    dict(nx=96, ny=40, Lx=4.8, Ly=2.0, D=0.55, xc=1.3, yc=0.95, nu=0.004, precision='fp32'),
]


def test_grouped_batch_matches_cases_stepped_alone(monkeypatch):
    """With GHOSTMAC_BATCH_GROUPED=1 the cases of one grid shape and precision share
    case-indexed solve launches (blockIdx.y is the case); every case must still end bitwise
    where it ends when stepped alone."""
    monkeypatch.setenv('GHOSTMAC_BATCH_GROUPED', '1')
    pkg = load_package()

    def make():
        out = []
        for i, kw in enumerate(GROUPED):
            s = pkg.MAC_CylinderFlow(boundary='ghost_cell', time_scheme='ab2_cn', verbose=False, **kw)
            q = s.gg.pack(s.u, s.v)
            q += 1e-3 * np.random.default_rng(40 + i).standard_normal(q.size)
            s.u, s.v = s.gg.unpack(q)
            out.append(s)
        return out

    alone, together = make(), make()
    for s in alone:
        s.solve(n_steps=12, dt=0.002, perturb_transient=False, save_artifacts=False, verbose=False)
    b = pkg.CylinderBatch(together)
    r = b.solve(12, dt=0.002)
    for s, t, (ts, cd, cl) in zip(alone, together, r):
        assert len(ts) == 12
        np.testing.assert_array_equal(t.u, s.u)
        np.testing.assert_array_equal(t.v, s.v)
        np.testing.assert_array_equal(t.p, s.p)
        assert t.last_step_diagnostics['cd'] == s.last_step_diagnostics['cd']
        assert t.last_step_diagnostics['max_divergence'] < 1e-10
    b.close()
