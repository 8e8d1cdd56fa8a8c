"""Periodic Taylor-Green path on the GPU (verification/taylor_green.py:14-59) against the
reference's own runs (tests/golden/taylor_green.npz).  The reference solves the CN system with
GMRES to rtol 1e-12, this library exactly in Fourier space: fields agree to 1e-11 relative,
error norms to 1e-8 relative.  FP32 mode: stencils and transforms in FP32 with both solves
refined against the FP64 operators; velocity within 1e-6 of the FP64 path, divergence < 1e-10."""
import numpy as np
import pytest

from conftest import GOLDEN, load_package

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize('tag', ['n16', 'n32'])
def test_taylor_green_matches_reference(tag):
    tg = load_package().taylor_green
    G = np.load(GOLDEN / 'taylor_green.npz')
    n, dt, end, nu = G[f'{tag}_params']
    info, q, p = tg.run(int(n), float(dt), float(end), float(nu))
    assert np.max(np.abs(q - G[f'{tag}_q'])) < 1e-11 * np.max(np.abs(G[f'{tag}_q']))
    assert np.max(np.abs(p - G[f'{tag}_p'])) < 1e-10 * np.max(np.abs(G[f'{tag}_p']))
    norms = np.array([info['velocity'][k] for k in ('l1', 'l2', 'linf')] +
                     [info['pressure'][k] for k in ('l1', 'l2', 'linf')])
    np.testing.assert_allclose(norms, G[f'{tag}_norms'][:6], rtol=1e-8)
    assert info['max_divergence'] < 1e-10


def test_taylor_green_fp32_refined():
    tg = load_package().taylor_green
    info64, q64, p64 = tg.run(64, .005, .1, .05)
    info32, q32, p32 = tg.run(64, .005, .1, .05, precision='fp32')
    assert info32['max_divergence'] < 1e-10
    assert np.max(np.abs(q32 - q64)) < 1e-6 * np.max(np.abs(q64))
    assert np.max(np.abs(p32 - p64)) < 1e-5 * np.max(np.abs(p64))
    assert abs(info32['velocity']['l2'] / info64['velocity']['l2'] - 1) < 1e-3


def test_taylor_green_rejects_bad_arguments():
    tg = load_package().taylor_green
    with pytest.raises(ValueError):
        tg.run(4, .01)
    with pytest.raises(ValueError):
        tg.run(16, .03, end_time=.1)
