"""The legacy staircase path's native kernels (module mac_engine, solver/src/bindings.cpp) on
the GPU against the reference's own compiled module (tests/golden/legacy_kernels.npz, made by
make_golden.py from bindings.cpp built here).

predictor_rhs_cpp and corrector_cpp repeat the reference's per-point arithmetic without FMA
contraction: their outputs must be bit-identical.  The force and divergence sums are reduced in
a different (fixed) order: 1e-13 relative.  The argument checks run on the host and are tested
without a GPU.
"""
import sys

import numpy as np
import pytest

from conftest import GOLDEN, load_package


@pytest.fixture(scope='module')
def M():
    pkg = load_package()
    __import__(pkg.__name__ + '.mac_engine')
    return sys.modules[pkg.__name__ + '.mac_engine']


@pytest.fixture(scope='module')
def G():
    return np.load(GOLDEN / 'legacy_kernels.npz')


def case(G, tag):
    nx, ny, dx, dy, dt, nu, rho = G[f'{tag}_in']
    arrays = {k: np.ascontiguousarray(G[f'{tag}_{k}']) for k in ('u', 'v', 'p', 'phi', 'inlet', 'mask')}
    return int(nx), int(ny), dx, dy, dt, nu, rho, arrays


@pytest.mark.gpu
@pytest.mark.parametrize('tag', ['a', 'b'])
def test_predictor_rhs_bit_identical(M, G, tag):
    nx, ny, dx, dy, dt, nu, rho, a = case(G, tag)
    for slip in (0, 1):
        for centered in (0, 1):
            us, vs, rhs = np.full_like(a['u'], 7.0), np.full_like(a['v'], 7.0), np.full_like(a['p'], 7.0)
            M.predictor_rhs_cpp(a['u'], a['v'], us, vs, rhs, a['p'], a['mask'], a['inlet'], dx, dy, dt, nu, rho,
                                bool(slip), bool(centered))
            key = f'{tag}_pred_s{slip}c{centered}'
            assert np.array_equal(us, G[key + '_us']), key
            assert np.array_equal(vs, G[key + '_vs']), key
            assert np.array_equal(rhs, G[key + '_rhs']), key


@pytest.mark.gpu
@pytest.mark.parametrize('tag', ['a', 'b'])
def test_corrector_bit_identical(M, G, tag):
    nx, ny, dx, dy, dt, nu, rho, a = case(G, tag)
    u, v = a['u'].copy(), a['v'].copy()
    M.corrector_cpp(u, v, np.ascontiguousarray(G[f'{tag}_corr_us']), np.ascontiguousarray(G[f'{tag}_corr_vs']),
                    a['phi'], a['mask'], a['inlet'], dx, dy, dt, rho, False)
    assert np.array_equal(u, G[f'{tag}_corr_u'])
    assert np.array_equal(v, G[f'{tag}_corr_v'])


@pytest.mark.gpu
@pytest.mark.parametrize('tag', ['a', 'b'])
def test_forces_and_divergence(M, G, tag):
    nx, ny, dx, dy, dt, nu, rho, a = case(G, tag)
    f = np.array(M.calculate_mac_forces_cpp(a['u'], a['v'], a['p'], a['mask'], dx, dy, nu * rho))
    ref = G[f'{tag}_forces']
    assert np.max(np.abs(f - ref)) <= 1e-13 * max(1.0, np.max(np.abs(ref)))
    d = M.calculate_mac_divergence_cpp(a['u'], a['v'], a['mask'], dx, dy)
    r = G[f'{tag}_div']
    assert d[0] == r[0]                                  # a maximum is order-independent
    assert d[2] == int(r[2]) and d[4] == int(r[4])
    assert abs(d[1] - r[1]) <= 1e-13 * r[1] and abs(d[3] - r[3]) <= 1e-13 * r[3]


@pytest.mark.gpu
def test_device_tensors_in_place(M, G):
    """The same call with CUDA tensors runs on them in place (no staging)."""
    torch = pytest.importorskip('torch')
    nx, ny, dx, dy, dt, nu, rho, a = case(G, 'a')
    dev = {k: torch.from_numpy(v).cuda() for k, v in a.items()}
    us, vs = torch.zeros_like(dev['u']), torch.zeros_like(dev['v'])
    rhs = torch.zeros_like(dev['p'])
    M.predictor_rhs_cpp(dev['u'], dev['v'], us, vs, rhs, dev['p'], dev['mask'], dev['inlet'], dx, dy, dt, nu, rho,
                        False, True)
    assert np.array_equal(us.cpu().numpy(), G['a_pred_s0c1_us'])
    assert np.array_equal(rhs.cpu().numpy(), G['a_pred_s0c1_rhs'])


def test_argument_checks(M, G):
    nx, ny, dx, dy, dt, nu, rho, a = case(G, 'b')
    us, vs, rhs = np.zeros_like(a['u']), np.zeros_like(a['v']), np.zeros_like(a['p'])
    args = [a['u'], a['v'], us, vs, rhs, a['p'], a['mask'], a['inlet'], dx, dy, dt, nu, rho, False]
    bad = list(args)
    bad[0] = a['u'][:, :-1].copy()
    with pytest.raises(ValueError, match='matching staggered shapes'):
        M.predictor_rhs_cpp(*bad)
    bad = list(args)
    bad[6] = a['mask'].astype(np.uint8)
    with pytest.raises(ValueError, match='matching staggered shapes'):
        M.predictor_rhs_cpp(*bad)
    bad = list(args)
    bad[7] = a['inlet'][:-1].copy()
    with pytest.raises(ValueError, match='inlet must be'):
        M.predictor_rhs_cpp(*bad)
    bad = list(args)
    bad[10] = 0.0
    with pytest.raises(ValueError, match='dt and rho'):
        M.predictor_rhs_cpp(*bad)
    bad = list(args)
    bad[11] = -1.0
    with pytest.raises(ValueError, match='nu must be'):
        M.predictor_rhs_cpp(*bad)
    with pytest.raises(ValueError, match='dx and dy'):
        M.calculate_mac_divergence_cpp(a['u'], a['v'], a['mask'], 0.0, dy)
    with pytest.raises(ValueError, match='mu must be'):
        M.calculate_mac_forces_cpp(a['u'], a['v'], a['p'], a['mask'], dx, dy, np.nan)
    with pytest.raises(ValueError, match='at least 2 cells'):
        M.calculate_mac_divergence_cpp(a['u'][:1, :2], a['v'][:2, :1], a['mask'][:1, :1], dx, dy)
