"""The three legacy loops on the benched grid (800x820, Re 100; bench.py workloads
staircase_800x820_re100, legacy_ghost_800x820_re100, cutcell_legacy_800x820_re100) against three
steps of the reference's own loops (tests/golden/legacy_wide_800x820.npz, written by
tests/golden/make_golden.py, group legacy_wide: 2000 seeded samples per field and step, the field
maxima and the force coefficients).  The predictors and correctors are the reference's
arithmetic and the pressure solves agree with its sparse LU to rounding; at this grid size the
pressure system's conditioning (about 1e6) lifts that rounding to about 2e-10 of max |p| (1.9e-10
measured on the staircase loop's second step).  So the velocity samples agree to 1e-10 of the
field maxima, the pressure samples to 2e-9, and the force coefficients, which carry the
pressure force, to 5e-9 relative."""
from pathlib import Path

import numpy as np
import pytest

from conftest import load_package

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).parent / 'golden' / 'legacy_wide_800x820.npz'
KW = dict(nx=800, ny=820, Lx=40.0, Ly=41.0, D=1.0, xc=10.0, yc=20.5, nu=0.01)


@pytest.mark.parametrize('tag,boundary', [('staircase', 'staircase'), ('ghost', 'ghost_cell'),
                                          ('cutcell', 'cut_cell')])
def test_legacy_loop_on_the_benched_grid(tag, boundary):
    pkg = load_package()
    d = np.load(GOLDEN)
    s = pkg.MAC_CylinderFlow(boundary=boundary, time_scheme='legacy', transport='centered', pressure_solver='direct',
                             verbose=False, **KW)
    for k in range(3):
        _, cd, cl = s.solve(n_steps=1, dt=0.002, perturb_transient=False, save_artifacts=False, verbose=False)
        ref = d[f'{tag}_coef'][k]
        assert abs(cd[0] - ref[0]) <= 5e-9 * max(1.0, abs(ref[0])), (k, cd[0], ref[0])
        assert abs(cl[0] - ref[1]) <= 5e-9 * max(1.0, abs(ref[0])), (k, cl[0], ref[1])
        for q, (name, field) in enumerate((('u', s.u), ('v', s.v), ('p', s.p))):
            tol = 2e-9 if name == 'p' else 1e-10
            scale = max(1.0, float(d[f'{tag}_maxima'][k][q]))
            got = field.ravel()[d[f'sample_{name}']]
            err = float(np.max(np.abs(got - d[f'{tag}_{name}'][k]))) / scale
            assert err < tol, (k, name, err)
            assert abs(np.abs(field).max() - d[f'{tag}_maxima'][k][q]) <= tol * scale
