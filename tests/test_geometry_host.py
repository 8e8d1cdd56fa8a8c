"""Host-side setup of libghostmac.so against the oracle: bit-exact classification and stencils.

These run without a GPU: gm_create_host builds the geometry, ghost stencils,
operator rows and boundary Schur rows on the host.
"""
import ctypes as C

import numpy as np
import pytest

import ghost_oracle as go
from conftest import load_package

CASES = [
    ((88, 16, 22., 4.1, 1., 2., 2.), {}),
    ((40, 30, 4., 3., 1., 1.5, 1.5), dict(vi=1)),
    ((40, 30, 4., 3., 1., 1.5, 1.5), dict(pe=1)),
    ((80, 60, 4., 3., 1., 1.5, 1.5), {}),
    ((400, 200, 20., 10., 1., 5., 5.), dict(nu=1 / 40)),
]


@pytest.fixture(scope='module')
def L():
    return load_package()._lib


def host_handle(L, nx, ny, Lx, Ly, D, xc, yc, nu=0.01, pe=0, vi=0):
    cfg = L.Config(nx=nx, ny=ny, Lx=Lx, Ly=Ly, D=D, xc=xc, yc=yc, nu=nu, rho=1., U_inf=1., inflow=0, U_m=0.,
                   pressure_solver=0, pressure_extension=pe, velocity_interpolation=vi, precision=0)
    h = C.c_void_p()
    L.check(L.lib.gm_create_host(C.byref(cfg), C.byref(h)))
    return h


def stencils(L, h, which):
    n, nnz = C.c_int64(), C.c_int64()
    L.check(L.lib.gm_get_ghost_stencils(h, which, C.byref(n), C.byref(nnz), None, None, None, None), h)
    rows, p_ = np.empty(n.value, np.int64), np.empty(n.value + 1, np.int64)
    cols, vals = np.empty(nnz.value, np.int64), np.empty(nnz.value)
    L.check(L.lib.gm_get_ghost_stencils(h, which, None, None, L.ptr(rows), L.ptr(p_), L.ptr(cols), L.ptr(vals)), h)
    return rows, p_, cols, vals


def schur(L, h, which):
    n = C.c_int64()
    L.check(L.lib.gm_get_schur_rows(h, which, C.byref(n), None), h)
    r = np.empty(n.value, np.int64)
    L.check(L.lib.gm_get_schur_rows(h, which, None, L.ptr(r)), h)
    return r


def test_library_exports_every_declared_symbol(L):
    import re
    from conftest import ROOT
    header = (ROOT / 'include' / 'ghostmac.h').read_text()
    declared = set(re.findall(r'^\s*(?:int|int32_t|int64_t|const char\*)\s+(gm_\w+)\s*\(', header, re.M))
    assert declared and declared == set(L.SYMBOLS), declared ^ set(L.SYMBOLS)
    for name in declared:
        assert hasattr(L.lib, name), name


def test_host_alloc_with_or_without_a_device(L):
    """gm_host_alloc gives page-locked memory on a GPU machine and GM_ECUDA with a NULL
    pointer without one; the facade's pinned_empty then falls back to an ordinary array."""
    import sys
    p = C.c_void_p()
    rc = L.lib.gm_host_alloc(C.c_size_t(64), C.byref(p))
    if rc == L.GM_OK:
        assert p.value
        assert L.lib.gm_host_free(p) == L.GM_OK
    else:
        assert rc == L.GM_ECUDA and not p.value
    assert L.lib.gm_host_free(None) == L.GM_OK
    ghost = sys.modules[load_package().__name__ + '.ghost']
    a = ghost.pinned_empty((3, 5))
    assert a.shape == (3, 5) and a.dtype == np.float64 and a.flags.writeable and a.flags.c_contiguous
    a[:] = 1.5
    assert float(a.sum()) == 22.5


@pytest.mark.parametrize('args,kw', CASES)
def test_setup_matches_oracle(L, args, kw):
    h = host_handle(L, *args, **kw)
    try:
        c = go.CylinderCase(nx=args[0], ny=args[1], Lx=args[2], Ly=args[3], D=args[4], xc=args[5], yc=args[6],
                            nu=kw.get('nu', .01),
                            ghost_velocity_interpolation='biquadratic' if kw.get('vi') else 'bilinear',
                            ghost_pressure_extension='quadratic' if kw.get('pe') else 'neumann')
        o = c.ops
        s = L.Sizes()
        L.check(L.lib.gm_get_sizes(h, C.byref(s)), h)
        ui, vi, pi = (np.empty(n, np.int64) for n in (s.nu_active, s.nv_active, s.np_active))
        L.check(L.lib.gm_get_indices(h, L.ptr(ui), L.ptr(vi), L.ptr(pi)), h)
        assert np.array_equal(ui, o.ui) and np.array_equal(vi, o.vi) and np.array_equal(pi, o.pi)
        for which, E, ids in ((0, o.Eu, o.ui), (1, o.Ev, o.vi), (2, o.P, o.pi)):
            rows, p_, cols, vals = stencils(L, h, which)
            Ec = E.tocsr()
            ident = np.zeros(E.shape[0], bool)
            ident[ids] = True
            orows = np.flatnonzero(~ident & (np.diff(Ec.indptr) > 0))
            sub = Ec[orows]
            sub.sort_indices()
            assert np.array_equal(rows, orows)
            assert np.array_equal(p_, sub.indptr) and np.array_equal(cols, ids[sub.indices])
            # the rows read active points only, so applying them twice rewrites the same values
            # (the step relies on this when it extends a field once for two consumers)
            assert not np.isin(cols, rows).any()
            tol = 1e-12 if (which == 2 and kw.get('pe')) else 0.0
            assert np.max(np.abs(vals - sub.data)) <= tol
        rect = go.rectangle(c.nx, c.ny, c.dx, c.dy, 'pressure', rho=c.rho)[0]
        assert np.array_equal(schur(L, h, 0), go.schur_rows(o.A, o.pi, rect)[0])
        L.check(L.lib.gm_prepare_dt(h, 0.001), h)
        o.build_helmholtz(0.001)
        assert np.array_equal(schur(L, h, 1), o.helmholtz_parts[0].rows)
        assert np.array_equal(schur(L, h, 2), o.helmholtz_parts[1].rows)
        pts = np.empty((s.n_surface, 2))
        L.check(L.lib.gm_get_surface_points(h, L.ptr(pts)), h)
        assert np.max(np.abs(pts - o.surface_points)) <= 1e-14
    finally:
        L.lib.gm_destroy(h)


def test_setup_errors_map_to_value_error(L):
    with pytest.raises(ValueError, match='strictly inside'):
        host_handle(L, 40, 30, 4., 3., 1., 0.2, 1.5)
    with pytest.raises(ValueError, match='outer boundary'):
        host_handle(L, 8, 8, 1.0, 1.0, 0.9, 0.5, 0.5)
