"""The legacy staircase loop on the GPU (MAC_CylinderFlow(boundary='staircase', time_scheme='legacy'))
against the reference's own loop on the same grid (tests/golden/staircase_48x24.npz, written by
tests/golden/make_golden.py with mac_engine built from solver/src/bindings.cpp and the sparse-LU
pressure solve): centred transport with the loop's AB2 step, and upwind transport with the
transient inlet perturbation.  The native kernels are bit-identical to the reference's and the
pressure solve agrees with the LU to rounding, so the fields agree to 1e-11 and the force
coefficients to 1e-10 relative."""
from pathlib import Path

import numpy as np
import pytest

from conftest import load_package

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).parent / 'golden'


def rel(a, b):
    a, b = np.asarray(a, float), np.asarray(b, float)
    return float(np.max(np.abs(a - b))) / max(1.0, float(np.max(np.abs(b))))


@pytest.mark.parametrize('tag,transport,perturb', [('centered', 'centered', False), ('upwind', 'upwind', True)])
def test_staircase_loop_matches_reference(tag, transport, perturb):
    pkg = load_package()
    d = np.load(GOLDEN / 'staircase_48x24.npz')
    s = pkg.MAC_CylinderFlow(nx=48, ny=24, Lx=4.8, Ly=2.4, D=1.0, xc=1.3, yc=1.15, nu=0.02, boundary='staircase',
                             time_scheme='legacy', transport=transport, pressure_solver='direct', verbose=False)
    assert isinstance(s, pkg.StaircaseFlow)
    assert np.array_equal(s.u, d[f'{tag}_init_u']) and np.array_equal(s.v, d[f'{tag}_init_v'])
    coef = []
    for k in range(20):
        _, cd, cl = s.solve(n_steps=1, dt=0.002, perturb_transient=perturb, perturb_duration=0.03,
                            save_artifacts=False, verbose=False)
        coef.append([cd[0], cl[0]])
        if k + 1 in (1, 5, 20):
            for key in ('u', 'v', 'p'):
                err = rel(getattr(s, key), d[f'{tag}_{key}{k + 1}'])
                assert err < 1e-11, (k + 1, key, err)
    ref = d[f'{tag}_coef']
    assert np.max(np.abs(np.array(coef) - ref) / np.maximum(1.0, np.abs(ref))) < 1e-10
    assert abs(s.time - float(d[f'{tag}_time'])) < 1e-14
    max_div, _, _, _, _ = s.divergence_stats()
    assert max_div < 1e-9


def test_staircase_rejects_ab2_cn():
    pkg = load_package()
    with pytest.raises(ValueError, match='ab2_cn requires'):
        pkg.MAC_CylinderFlow(nx=48, ny=24, Lx=4.8, Ly=2.4, xc=1.3, yc=1.15, boundary='staircase',
                             time_scheme='ab2_cn', verbose=False)


def test_staircase_metadata_and_no_checkpoint(tmp_path):
    """metadata() records the run like the reference's; the legacy loop keeps no checkpoint
    (the reference raises the same ValueError)."""
    pkg = load_package()
    s = pkg.MAC_CylinderFlow(nx=48, ny=24, Lx=4.8, Ly=2.4, D=1.0, xc=1.3, yc=1.15, nu=0.02, boundary='staircase',
                             time_scheme='legacy', transport='upwind', verbose=False)
    m = s.metadata(0.002, 10)
    assert m['time_integrator'] == 'Euler' and m['boundary'] == 'staircase' and m['time_scheme'] == 'legacy'
    assert set(m['source_sha256']) and all(len(v) == 64 for v in m['source_sha256'].values())
    with pytest.raises(ValueError, match='Checkpoints require'):
        s.save_checkpoint(tmp_path / 'x.npz')
