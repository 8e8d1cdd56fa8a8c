"""GPU step parity against the oracle on the workload shapes the benchmark and the sweep use.

Each test steps libghostmac.so (through the C ABI) and the FP64 oracle from the same seeded
state and compares the fields after the steps.  Tolerances (max-norm, relative to
max(1, |oracle|)):
  plain FP64 fields ............................ 1e-10   (config 1 also after 200 steps)
  plain FP64 drag / lift ....................... 1e-8 relative (lift: of max(|C_L|, 1e-3))
  FP32 mode: velocity 1e-7, pressure 1e-5, drag 1e-6 relative
  GMRES pressure path against the oracle's GMRES: fields 1e-9, pressure 1e-8 (two Krylov
  runs stopped at rtol 1e-12 agree to the solver tolerance, not to roundoff)
  discrete divergence .......................... < 1e-10 after every step
Workloads:
  wide 800x820 (40D x 41D, cylinder at (10D, 20.5D), Re 100, dt 0.002, 1e-2 v noise): 5 steps
  channel 400x200 (20D x 10D, (5D, 5D), Re 40, dt 0.002, 1e-3 u and v noise): 200 steps
  one 800x410 case drawn like the 64-case sweep (Re in [40, 200], D in [0.8, 1.2], centre
  (Lx/4, Ly/2) jittered by up to 0.5 D, 1e-3 noise): 5 steps in FP64 and in the FP32 mode
  1024x512 at h = 0.04 (Re 150, cylinder at (8D, 10.24D), dt 0.0015, 1e-2 v noise): 3 steps
  with the direct pressure path and 3 with GMRES
  the inlet perturbation of solver/main.py:281-286 (perturb_transient=True) for 35 steps
"""
import numpy as np
import pytest

import ghost_oracle as go
from conftest import load_package

pytestmark = pytest.mark.gpu

WIDE = dict(nx=800, ny=820, Lx=40.0, Ly=41.0, D=1.0, xc=10.0, yc=20.5, nu=0.01)
CHANNEL = dict(nx=400, ny=200, Lx=20.0, Ly=10.0, D=1.0, xc=5.0, yc=5.0, nu=1 / 40)
GMRES_CASE = dict(nx=1024, ny=512, Lx=40.96, Ly=20.48, D=1.0, xc=8.0, yc=10.24, nu=1 / 150)


def rel(a, b):
    a, b = np.asarray(a, float), np.asarray(b, float)
    return float(np.max(np.abs(a - b))) / max(1.0, float(np.max(np.abs(b))))


@pytest.fixture(scope='module')
def pkg():
    return load_package()


def sweep_800x410_draw(seed=4):
    """One case of the sweep's distribution with the 800x410 grid (h = 0.05)."""
    rng = np.random.default_rng(seed)
    nx, ny, h = 800, 410, 0.05
    re, d = rng.uniform(40.0, 200.0), rng.uniform(0.8, 1.2)
    lx, ly = nx * h, ny * h
    xc = lx / 4 + rng.uniform(-0.5, 0.5) * d
    yc = ly / 2 + rng.uniform(-0.5, 0.5) * d
    return dict(nx=nx, ny=ny, Lx=lx, Ly=ly, D=d, xc=xc, yc=yc, nu=d / re)


def seeded_pair(pkg, kw, noise, amp, seed, precision='fp64', pressure_solver='direct'):
    """The oracle case and the GPU case from the same seeded perturbation of the active faces."""
    c = go.CylinderCase(pressure_solver=pressure_solver, **kw)
    q = c.ops.pack(c.u, c.v)
    rng = np.random.default_rng(seed)
    nu = len(c.ops.ui)
    if noise == 'uv':
        q += amp * rng.standard_normal(q.size)
    else:
        q[nu:] += amp * rng.standard_normal(q.size - nu)
    c.u, c.v = c.ops.unpack(q)
    s = pkg.MAC_CylinderFlow(boundary='ghost_cell', time_scheme='ab2_cn', verbose=False, precision=precision, pressure_solver=pressure_solver, **kw)
    s.u[:], s.v[:] = c.u, c.v
    return c, s


def step_both(c, s, n, dt, per_step=True, **opts):
    """Step both cases; returns the GPU's diagnostics of every step (divergence gate)."""
    out = []
    if per_step:
        for _ in range(n):
            s.solve(n_steps=1, dt=dt, save_artifacts=False, verbose=False, **opts)
            c.solve(1, dt, **opts)
            out.append(dict(s.last_step_diagnostics))
    else:
        s.solve(n_steps=n, dt=dt, save_artifacts=False, verbose=False, **opts)
        c.solve(n, dt, **opts)
        out.append(dict(s.last_step_diagnostics))
    return out


def assert_fields(c, s, tol_uv, tol_p, tol_cd, tol_cl=None):
    assert rel(s.u, c.u) < tol_uv, ('u', rel(s.u, c.u))
    assert rel(s.v, c.v) < tol_uv, ('v', rel(s.v, c.v))
    assert rel(s.p, c.p) < tol_p, ('p', rel(s.p, c.p))
    d, e = s.last_step_diagnostics, c.last_step_diagnostics
    assert abs(d['cd'] - e['cd']) <= tol_cd * abs(e['cd']), (d['cd'], e['cd'])
    if tol_cl is not None:
        assert abs(d['cl'] - e['cl']) <= tol_cl * max(abs(e['cl']), 1e-3), (d['cl'], e['cl'])


@pytest.fixture(scope='module')
def wide_oracle():
    """The oracle's 5 steps of the wide 800x820 workload (the benchmark's default)."""
    c = go.CylinderCase(**WIDE)
    q = c.ops.pack(c.u, c.v)
    nu = len(c.ops.ui)
    q[nu:] += 1e-2 * np.random.default_rng(0).standard_normal(q.size - nu)
    c.u, c.v = c.ops.unpack(q)
    u0, v0 = c.u.copy(), c.v.copy()
    c.solve(5, 0.002)
    return u0, v0, c


@pytest.mark.parametrize('precision', ['fp64', 'fp32'])
def test_wide_800x820_five_steps(pkg, wide_oracle, precision):
    u0, v0, c = wide_oracle
    s = pkg.MAC_CylinderFlow(boundary='ghost_cell', time_scheme='ab2_cn', verbose=False, precision=precision, **WIDE)
    s.u[:], s.v[:] = u0, v0
    for _ in range(5):
        s.solve(n_steps=1, dt=0.002, perturb_transient=False, save_artifacts=False, verbose=False)
        assert s.last_step_diagnostics['max_divergence'] < 1e-10
    if precision == 'fp64':
        assert_fields(c, s, 1e-10, 1e-10, 1e-8, 1e-8)
    else:
        assert_fields(c, s, 1e-7, 1e-5, 1e-6)


def test_channel_400x200_two_hundred_steps(pkg):
    """Config 1 for its full 200 steps: fields within 1e-10 at steps 50, 100, 150 and 200."""
    c, s = seeded_pair(pkg, CHANNEL, 'uv', 1e-3, 0)
    for _ in range(4):
        s.solve(n_steps=50, dt=0.002, perturb_transient=False, save_artifacts=False, verbose=False)
        c.solve(50, 0.002)
        assert s.last_step_diagnostics['max_divergence'] < 1e-10
        assert_fields(c, s, 1e-10, 1e-10, 1e-8, 1e-8)


@pytest.mark.parametrize('precision', ['fp64', 'fp32'])
def test_sweep_800x410_draw(pkg, precision):
    kw = sweep_800x410_draw()
    c, s = seeded_pair(pkg, kw, 'uv', 1e-3, 7, precision=precision)
    for d in step_both(c, s, 5, 0.002, perturb_transient=False):
        assert d['max_divergence'] < 1e-10
    if precision == 'fp64':
        assert_fields(c, s, 1e-10, 1e-10, 1e-8, 1e-8)
    else:
        assert_fields(c, s, 1e-7, 1e-5, 1e-6)


def test_gmres_case_1024x512_direct(pkg):
    c, s = seeded_pair(pkg, GMRES_CASE, 'v', 1e-2, 0)
    for d in step_both(c, s, 3, 0.0015, perturb_transient=False):
        assert d['max_divergence'] < 1e-10
    assert_fields(c, s, 1e-10, 1e-10, 1e-8, 1e-8)


def test_gmres_case_1024x512_iterative(pkg):
    c, s = seeded_pair(pkg, GMRES_CASE, 'v', 1e-2, 0, pressure_solver='iterative')
    for d in step_both(c, s, 3, 0.0015, perturb_transient=False):
        assert d['max_divergence'] < 1e-10
        assert d['pressure_backend'] == 'gmres_rectangle' and d['pressure_iterations'] > 0
    assert_fields(c, s, 1e-9, 1e-8, 1e-8)


@pytest.mark.parametrize('precision', ['fp64', 'fp32'])
def test_inlet_perturbation(pkg, precision):
    """perturb_transient=True: the inlet profile u_base (1 + a sin(2 pi y / Ly)(1 - t / T))
    of solver/main.py:281-286 on every step inside the perturbation window T = 0.06: 25 steps
    inside it, then 10 more that cross its end and run on the base profile again."""
    kw = dict(nx=88, ny=16, Lx=22., Ly=4.1, xc=2., yc=2., nu=0.02)
    c, s = seeded_pair(pkg, kw, 'uv', 1e-2, 5, precision=precision)
    opts = dict(perturb_transient=True, perturb_duration=0.06, perturb_amp=0.15)
    tol = (1e-10, 1e-10, 1e-8, 1e-8) if precision == 'fp64' else (1e-7, 1e-5, 1e-6)
    step_both(c, s, 25, 0.002, per_step=False, **opts)
    assert_fields(c, s, *tol)
    # the inlet column of the state carries the perturbed profile of the last step
    prof = c.u_inlet_base * (1.0 + 0.15 * np.sin(2.0 * np.pi * c.y_centers / c.Ly) * (1.0 - s.time / 0.06))
    assert np.max(np.abs(s.u[:, 0] - prof)) < 1e-14
    assert np.max(np.abs(prof - c.u_inlet_base)) > 1e-3
    step_both(c, s, 10, 0.002, per_step=False, **opts)
    assert np.max(np.abs(s.u[:, 0] - c.u_inlet_base)) < 1e-14
    assert_fields(c, s, *tol)


def test_verbose_line(pkg, capsys):
    """The verbose step line of solver/main.py:436-454: Div_RMS is sqrt(sum div^2 / count)
    over the fluid cells, Div_Max their maximum, printed at step 0 and at the last step."""
    kw = dict(nx=88, ny=16, Lx=22., Ly=4.1, xc=2., yc=2., nu=0.02)
    c, s = seeded_pair(pkg, kw, 'uv', 1e-2, 5)
    s.solve(n_steps=3, dt=0.002, perturb_transient=False, save_artifacts=False, verbose=True)
    lines = [ln for ln in capsys.readouterr().out.splitlines() if ln.startswith('Step')]
    assert [int(ln.split('|')[0].split()[1]) for ln in lines] == [0, 2]
    fields = dict(f.split(':') for f in lines[-1].split('|')[1:])
    mx, s2, n, _, _ = go.mac_divergence_stats(s.u, s.v, s.dx, s.dy, s.mask)
    rms = float(fields[' Div_RMS'])
    assert abs(rms - np.sqrt(s2 / n)) <= 0.01 * np.sqrt(s2 / n) + 1e-300
    assert abs(float(fields[' Div_Max']) - mx) <= 0.01 * mx + 1e-300
    assert abs(float(fields[' Cd']) - s.last_step_diagnostics['cd']) < 1e-4
