"""The cut-cell host setup (cutcell_geometry.py) against the reference's own setup, run on the
same grids by tests/golden/make_golden.py (group cutcell): fractions and cell classes
bit-exact, merge tables and owned-volume maps exact, stencil operators by their action on a
seeded field to rounding."""
import numpy as np
import pytest

from conftest import load_module

CASES = ('cc40x20', 'cc48x30')


@pytest.fixture(scope='module', params=CASES)
def case(request):
    from pathlib import Path
    d = np.load(Path(__file__).parent / 'golden' / f'cutcell_{request.param}.npz')
    cg = load_module('cutcell_geometry')
    nx, ny, Lx, Ly, D, xc, yc, nu, rho = d['config']
    setup = cg.CutCellSetup(int(nx), int(ny), Lx, Ly, xc, yc, D / 2)
    return d, setup


def rel(a, b):
    a, b = np.asarray(a, float), np.asarray(b, float)
    return float(np.max(np.abs(a - b))) / max(1.0, float(np.max(np.abs(b))))


def test_fractions_and_classes_bit_exact(case):
    d, st = case
    g = st.geom
    for name in ('ax', 'ay', 'volume_fraction', 'u_volume_fraction', 'v_volume_fraction', 'ax_mid', 'ay_mid',
                 'ay_u', 'ax_v'):
        assert np.array_equal(getattr(g, name), d['geom_' + name]), name
    assert np.array_equal(g.cell_type, d['geom_cell_type'])
    assert np.array_equal(np.array(g.u_merge_list, dtype=np.int64).reshape(-1, 4), d['u_merge'])
    assert np.array_equal(np.array(g.v_merge_list, dtype=np.int64).reshape(-1, 4), d['v_merge'])


def test_owned_volumes(case):
    d, st = case
    for c in ('u', 'v'):
        assert np.array_equal(getattr(st, f'{c}_covered'), d[f'{c}_covered'])
        assert np.array_equal(getattr(st, f'{c}_owner'), d[f'{c}_owner'])
        assert np.array_equal(getattr(st, f'{c}_vol'), d[f'{c}_vol'])
        assert np.array_equal(getattr(st, f'{c}_vol_eff'), d[f'{c}_vol_eff'])


def test_wall_and_face_stencils(case):
    d, st = case
    f = d['probe_field']
    w = st.wall
    for name in ('tx', 'ty', 'ds', 'u_indices', 'v_indices'):
        assert np.array_equal(getattr(w, name), d['wall_' + name]), name
    assert w.rate.nnz == int(d['wall_rate_nnz'])
    assert rel(w.rate @ f, d['wall_rate_action']) < 1e-12
    for (c, a), mf in st.momentum_faces.items():
        key = f'mf_{c}{a}'
        assert np.array_equal(mf.indices, d[key + '_indices'])
        assert np.array_equal(mf.patch, d[key + '_patch'])
        assert np.array_equal(mf.lengths, d[key + '_lengths'])
        assert [mf.u.nnz, mf.v.nnz, mf.gradient.nnz] == list(d[key + '_nnz'])
        assert rel(mf.u @ f, d[key + '_u_action']) < 1e-12
        assert rel(mf.v @ f, d[key + '_v_action']) < 1e-12
        assert rel(mf.gradient @ f, d[key + '_gradient_action']) < 1e-12
        df = st.diffusion_faces[c, a]
        assert np.array_equal(df.indices, d[f'df_{c}{a}_indices'])
        assert rel(df.gradient @ f, d[f'df_{c}{a}_gradient_action']) < 1e-12


def test_geometry_rejects_invalid_cases():
    cg = load_module('cutcell_geometry')
    with pytest.raises(ValueError, match='nx and ny'):
        cg.CutCellGeometry(3, 10, 4., 2., 1., 1., .5)
    with pytest.raises(ValueError, match='strictly inside'):
        cg.CutCellGeometry(40, 20, 4., 2., .4, 1., .5)
