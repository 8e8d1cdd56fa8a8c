"""The allocation-free divergence statistics entry point against the allocating one.

gm_divergence_stats_noalloc exists for callers that cannot call cudaMalloc (code
living inside another runtime's fixed device arena, or tools that only borrow
device arrays): it keeps its scratch in a static device array instead.  This
file is named to be collected last, so that a failure here leaves every other
test already run.  It builds its own state and also passes alone in a fresh
process.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import load_package

pytestmark = pytest.mark.gpu


def _noalloc(L, u, v, mask, nx, ny, dx, dy, stream=None):
    out = np.zeros(3)
    counts = np.zeros(2, np.int64)
    rc = L.lib.gm_divergence_stats_noalloc(L.ptr(u), L.ptr(v), L.ptr(mask), nx, ny, dx, dy, L.ptr(out),
                                           L.ptr(counts), stream)
    L.check(rc)
    return out, counts


def test_noalloc_divergence_stats_matches_allocating_entry_point():
    torch = pytest.importorskip('torch')
    pkg = load_package()
    L = pkg._lib
    s = pkg.MAC_CylinderFlow(boundary='ghost_cell', time_scheme='ab2_cn', nx=88, ny=16, Lx=22., Ly=4.1, xc=2., yc=2., nu=0.02, verbose=False)
    mask = torch.from_numpy(s.mask.astype(np.uint8)).cuda()
    rng = np.random.default_rng(11)
    for call in range(2):  # two calls in a row: the shared scratch keeps the previous call's contents
        s.solve(n_steps=2 + call, dt=0.002, perturb_transient=False, save_artifacts=False, verbose=False)
        # perturb so that the divergence is far from round-off and differs between calls
        u = s.u + 1e-3 * rng.standard_normal(s.u.shape)
        v = s.v + 1e-3 * rng.standard_normal(s.v.shape)
        s.u[:], s.v[:] = u, v
        expected = s.divergence_stats()
        out, counts = _noalloc(L, torch.from_numpy(u).cuda(), torch.from_numpy(v).cuda(), mask, s.nx, s.ny, s.dx, s.dy)
        assert out[0] == pytest.approx(expected[0], rel=1e-15, abs=0)
        assert out[1] == pytest.approx(expected[1], rel=1e-12)
        assert out[2] == pytest.approx(expected[3], rel=1e-12)
        assert (int(counts[0]), int(counts[1])) == (expected[2], expected[4])
        s.u[:], s.v[:] = s.gg.unpack(s.gg.pack(s.u, s.v))


def test_noalloc_rejects_oversized_grid_and_host_arrays():
    torch = pytest.importorskip('torch')
    L = load_package()._lib
    u = torch.zeros(16, 17, dtype=torch.float64, device='cuda')
    v = torch.zeros(17, 16, dtype=torch.float64, device='cuda')
    mask = torch.zeros(16, 16, dtype=torch.uint8, device='cuda')
    side = int(np.sqrt(L.NOALLOC_MAX_CELLS)) + 1
    with pytest.raises(ValueError, match='GM_NOALLOC_MAX_CELLS'):
        _noalloc(L, u, v, mask, side, side, 0.1, 0.1)
    with pytest.raises(ValueError, match='device arrays'):
        _noalloc(L, u.cpu().numpy(), v.cpu().numpy(), mask.cpu().numpy(), 16, 16, 0.1, 0.1)
