"""Host tables of the legacy ghost-cell branch (staircase.ghost_face_tables) against the
reference's GhostCellBoundary on the same grid (tests/golden/legacy_ghost_48x24.npz, written by
tests/golden/make_golden.py, group legacy_ghost): ghost faces in the reference's order, image
cells, bilinear weights and gammas bit-exact.  The level schedule the GPU runs (one launch per
level, corners that are later ghost faces read from a copy taken before the pass) is checked
against the reference's sequential pass on a seeded field, in numpy."""
from pathlib import Path

import numpy as np
import pytest

from conftest import load_module

GOLDEN = Path(__file__).parent / 'golden' / 'legacy_ghost_48x24.npz'
NX, NY, LX, LY, D, XC, YC = 48, 24, 4.8, 2.4, 1.0, 1.3, 1.15


def grids():
    dx, dy = LX / NX, LY / NY
    return dx, dy, {'u': (np.arange(NX + 1) * dx, (np.arange(NY) + 0.5) * dy, True),
                    'v': ((np.arange(NX) + 0.5) * dx, np.arange(NY + 1) * dy, False)}


@pytest.fixture(scope='module')
def tables():
    st = load_module('staircase')
    dx, dy, g = grids()
    return {k: (st.ghost_face_tables(xs, ys, dx, dy, XC, YC, D / 2, is_u), xs.size)
            for k, (xs, ys, is_u) in g.items()}


@pytest.mark.parametrize('face', ['u', 'v'])
def test_tables_bit_exact(tables, face):
    d = np.load(GOLDEN)
    t, nxf = tables[face]
    faces = d[f'ghost_{face}_faces']
    assert t['target'].size == len(faces) > 0
    assert np.array_equal(t['target'], faces[:, 0] * nxf + faces[:, 1])
    cells = d[f'ghost_{face}_cells']
    assert np.array_equal(t['src'][:, 0], cells[:, 0] * nxf + cells[:, 1])
    assert np.array_equal(t['src'][:, 3], (cells[:, 0] + 1) * nxf + cells[:, 1] + 1)
    assert np.array_equal(t['weights'], d[f'ghost_{face}_weights'])
    assert np.array_equal(t['gamma'], d[f'ghost_{face}_gammas'])


def sequential(f, t, wall=0.0):
    """apply_velocity_ghost_cells of solver/ghost_cell.py:159-184 on a flat field, in order."""
    f = f.copy()
    for g in range(t['target'].size):
        w, c = t['weights'][g], t['src'][g]
        ip = w[0] * f[c[0]] + w[1] * f[c[1]] + w[2] * f[c[2]] + w[3] * f[c[3]]
        f[t['target'][g]] = wall - t['gamma'][g] * (ip - wall)
    return f


def levelled(f, t, wall=0.0):
    """The GPU schedule: a copy of the ghost faces first, then one vectorised update per level."""
    f = f.copy()
    snap = f[t['target']].copy()
    for lv in range(t['n_levels']):
        g = np.flatnonzero(t['level'] == lv)
        vals = np.where(t['snap_of'][g] >= 0, snap[np.maximum(t['snap_of'][g], 0)], f[t['src'][g]])
        w = t['weights'][g]
        ip = w[:, 0] * vals[:, 0] + w[:, 1] * vals[:, 1] + w[:, 2] * vals[:, 2] + w[:, 3] * vals[:, 3]
        f[t['target'][g]] = wall - t['gamma'][g] * (ip - wall)
    return f


@pytest.mark.parametrize('face', ['u', 'v'])
def test_level_schedule_matches_sequential_pass(tables, face):
    t, nxf = tables[face]
    rng = np.random.default_rng(12)
    size = nxf * (NY if face == 'u' else NY + 1)
    f = rng.standard_normal(size)
    assert np.array_equal(levelled(f, t), sequential(f, t))
    # a planted error in the schedule shows: every face read with its value before the pass
    flat = dict(t, level=np.zeros_like(t['level']), n_levels=1,
                snap_of=np.where(t['snap_of'] >= 0, t['snap_of'], -1))
    if t['n_levels'] > 1:
        assert not np.array_equal(levelled(f, flat), sequential(f, t))


def test_levels_respect_the_order(tables):
    for t, nxf in tables.values():
        order = np.full(t['src'].max() + nxf + 2, -1)
        order[t['target']] = np.arange(t['target'].size)
        for g in range(t['target'].size):
            for q in range(4):
                k = order[t['src'][g, q]]
                if 0 <= k < g:
                    assert t['level'][g] > t['level'][k] and t['snap_of'][g, q] == -1
                elif k >= g:
                    assert t['snap_of'][g, q] == k


@pytest.mark.parametrize('is_u', [True, False])
def test_level_schedule_on_the_benched_grid(is_u):
    """800x820, 40D x 41D (the legacy ghost-cell bench workload): more launch levels than the
    small grid, the same sequential result."""
    st = load_module('staircase')
    nx, ny, lx, ly = 800, 820, 40.0, 41.0
    dx, dy = lx / nx, ly / ny
    xs = np.arange(nx + 1) * dx if is_u else (np.arange(nx) + 0.5) * dx
    ys = (np.arange(ny) + 0.5) * dy if is_u else np.arange(ny + 1) * dy
    t = st.ghost_face_tables(xs, ys, dx, dy, 10.0, 20.5, 0.5, is_u)
    assert t['n_levels'] >= 2 and t['target'].size > 0
    f = np.random.default_rng(5).standard_normal(xs.size * ys.size)
    assert np.array_equal(levelled(f, t, wall=0.1), sequential(f, t, wall=0.1))
