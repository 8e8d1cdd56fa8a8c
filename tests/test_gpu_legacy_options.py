"""The legacy loop's options on the GPU against the reference's own loop
(tests/golden/legacy_options.npz, written by tests/golden/make_golden.py, group legacy_options):
slip channel walls with parabolic inflow and upwind transport on the staircase branch,
rho = 1.3 with parabolic inflow on the ghost-cell branch, and slip walls, parabolic inflow,
upwind transport and the cg_dct pressure solver on the cut-cell branch; 12 steps each.  This
library solves every pressure_solver name to rounding: against the reference's sparse LU the
fields agree to 1e-10, against its CG-DCT solve (rtol 1e-12, refined to the 1e-10 divergence
budget) to 1e-9."""
from pathlib import Path

import numpy as np
import pytest

from conftest import load_package

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).parent / 'golden' / 'legacy_options.npz'
CASES = {
    'staircase_slip_parabolic_upwind': (dict(nx=48, ny=24, Lx=4.8, Ly=2.4, D=1.0, xc=1.3, yc=1.15, nu=0.02,
                                             boundary='staircase', transport='upwind', slip_walls=True,
                                             inflow='parabolic', U_m=1.2, pressure_solver='direct'), 1e-10, 1e-9),
    'ghost_parabolic_rho': (dict(nx=48, ny=24, Lx=4.8, Ly=2.4, D=1.0, xc=1.3, yc=1.15, nu=0.02, rho=1.3,
                                 boundary='ghost_cell', transport='centered', inflow='parabolic',
                                 pressure_solver='direct'), 1e-10, 1e-9),
    'cutcell_slip_parabolic_cgdct': (dict(nx=40, ny=20, Lx=4., Ly=2., D=1., xc=1.1, yc=0.95, nu=0.02,
                                          boundary='cut_cell', transport='upwind', slip_walls=True,
                                          inflow='parabolic', U_m=1.2, pressure_solver='cg_dct'), 1e-9, 1e-8),
}


def rel(a, b):
    a, b = np.asarray(a, float), np.asarray(b, float)
    return float(np.max(np.abs(a - b))) / max(1.0, float(np.max(np.abs(b))))


@pytest.mark.parametrize('tag', list(CASES))
def test_legacy_options_match_reference(tag):
    kw, ftol, ctol = CASES[tag]
    pkg = load_package()
    d = np.load(GOLDEN)
    s = pkg.MAC_CylinderFlow(time_scheme='legacy', verbose=False, **kw)
    assert np.array_equal(s.u_inlet, d[f'{tag}_inlet'])
    assert np.array_equal(s.u, d[f'{tag}_init_u']) and np.array_equal(s.v, d[f'{tag}_init_v'])
    coef = []
    for _ in range(12):
        _, cd, cl = s.solve(n_steps=1, dt=0.002, perturb_transient=True, perturb_duration=0.03,
                            save_artifacts=False, verbose=False)
        coef.append([cd[0], cl[0]])
    for name in ('u', 'v', 'p'):
        err = rel(getattr(s, name), d[f'{tag}_{name}'])
        assert err < ftol, (name, err)
    ref = d[f'{tag}_coef']
    assert np.max(np.abs(np.array(coef) - ref) / np.maximum(1.0, np.abs(ref))) < ctol
