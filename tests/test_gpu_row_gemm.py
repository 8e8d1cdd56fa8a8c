"""The FP32 mode's pressure row transforms as split-TF32 GEMMs on the tensor cores.

In the FP32 mode the two row passes of every pressure inverse (the DCT/DST rows of
solver/rectangular_inverse.py:8-58) run as tcgen05 GEMMs against the explicit transform
matrices, with the boundary Schur correction applied as the inverse pass loads its tiles.
The path is opt-in (GHOSTMAC_ROW_GEMM=1; the FFT passes are the default, being faster and more
accurate on the benched case).  Both sit inside the FP64 refinement, so both must
reach the FP64 solution: the tests compare them with each other and with the FP64 oracle, and
check through the kernel-class timers that the tensor-core kernels actually ran.
"""
import ctypes as C

import numpy as np
import pytest

import ghost_oracle as go
from conftest import load_package

pytestmark = pytest.mark.gpu

ROW_GEMM_CLASS = 12


def rel(a, b):
    a, b = np.asarray(a, float), np.asarray(b, float)
    return float(np.max(np.abs(a - b))) / max(1.0, float(np.max(np.abs(b))))


@pytest.fixture(scope='module')
def pkg():
    return load_package()


def row_gemm_launches(pkg, fn):
    """Launches of the tensor-core row passes while fn() runs (kernel timing on)."""
    lib = pkg._lib.lib
    lib.gm_kernel_timing(0, 1, None, None, None)
    try:
        fn()
        tot, cnt, by = C.c_double(), C.c_int64(), C.c_double()
        lib.gm_kernel_timing(ROW_GEMM_CLASS, 0, C.byref(tot), C.byref(cnt), C.byref(by))
    finally:
        lib.gm_kernel_timing(0, 0, None, None, None)
    return cnt.value


CASES = [dict(nx=88, ny=16, Lx=22., Ly=4.1, xc=2., yc=2., nu=0.02),
         dict(nx=400, ny=200, Lx=20., Ly=10., D=1., xc=5., yc=5., nu=1 / 40),
         dict(nx=800, ny=820, Lx=40., Ly=41., D=1., xc=10., yc=20.5, nu=1 / 100)]


@pytest.mark.parametrize('kw', CASES, ids=['88x16', '400x200', '800x820'])
def test_pressure_solve_tensor_core_rows(pkg, monkeypatch, kw):
    """One pressure solve A phi = b (random b on the active cells) in the FP32 mode with the
    tensor-core row passes, with the FFT row passes, and in plain FP64: all three meet the
    residual target, so they agree to the conditioning of A (1e-9 relative)."""
    out, b = {}, None
    for tag, prec, env in (('gemm', 'fp32', '1'), ('fft', 'fp32', '0'), ('fp64', 'fp64', '1')):
        monkeypatch.setenv('GHOSTMAC_ROW_GEMM', env)
        s = pkg.MAC_CylinderFlow(boundary='ghost_cell', time_scheme='ab2_cn', verbose=False, precision=prec, **kw)
        if b is None:
            b = np.random.default_rng(7).standard_normal(len(s.gg.pi))
        n = row_gemm_launches(pkg, lambda: out.__setitem__(tag, s.gg.pressure_solve(b)))
        assert (n > 0) == (tag == 'gemm'), (tag, n)
        out[tag + '_info'] = dict(s.gg.pressure_inverse_info['last_solve'])
    scale = max(1.0, float(np.max(np.abs(out['fp64']))))
    assert np.max(np.abs(out['gemm'] - out['fp64'])) < 1e-9 * scale
    assert np.max(np.abs(out['fft'] - out['fp64'])) < 1e-9 * scale
    # the tensor cores' FP32 accumulation costs at most one extra refinement sweep
    assert out['gemm_info']['refinement_iterations'] <= out['fft_info']['refinement_iterations'] + 1, out


def test_fp32_steps_tensor_core_rows_match_oracle(pkg, monkeypatch):
    """20 noisy AB2/CN steps of the FP32 mode with the tensor-core row passes against the FP64
    oracle: velocity 1e-7, pressure 1e-5, drag 1e-6 relative, divergence < 1e-10, and the
    row passes ran as tensor-core GEMMs in every step."""
    monkeypatch.setenv('GHOSTMAC_ROW_GEMM', '1')
    kw = CASES[0]
    s = pkg.MAC_CylinderFlow(boundary='ghost_cell', time_scheme='ab2_cn', verbose=False, precision='fp32', **kw)
    c = go.CylinderCase(**kw)
    q = c.ops.pack(c.u, c.v)
    q += 1e-2 * np.random.default_rng(5).standard_normal(q.size)
    c.u, c.v = c.ops.unpack(q)
    s.u[:], s.v[:] = c.u, c.v
    n = row_gemm_launches(pkg, lambda: s.solve(n_steps=2, dt=.002, perturb_transient=False, save_artifacts=False,
                                                verbose=False))
    assert n >= 2 * 2 * 2  # two steps, two projections, forward and inverse pass
    s.solve(n_steps=18, dt=.002, perturb_transient=False, save_artifacts=False, verbose=False)
    c.solve(20, .002)
    d = s.last_step_diagnostics
    assert d['max_divergence'] < 1e-10
    assert rel(s.u, c.u) < 1e-7 and rel(s.v, c.v) < 1e-7
    assert rel(s.p, c.p) < 1e-5
    assert abs(d['cd'] / c.last_step_diagnostics['cd'] - 1) < 1e-6
