"""CPU oracle for the ghost-cell MAC AB2/CN step: TEST INFRASTRUCTURE ONLY.

This module restates, in vectorised numpy/scipy, the reference algorithm of
invisce/cfd-cylinder-flow-ghost-cell for one path:
``MAC_CylinderFlow(boundary='ghost_cell', time_scheme='ab2_cn')``.
It is the checker for the CUDA library, the CPU baseline timed by ``bench.py``
and nothing else: product code never imports it.

Parity of this oracle with the reference itself is pinned by the golden
vectors under ``tests/golden`` (made by running the reference's own code with
``tests/golden/make_golden.py``) and checked by ``tests/test_oracle_golden.py``.

Every function names the reference file:line it follows.  Third-party
arithmetic used on the reference path is used here the same way:
scipy.fft (separable transforms), scipy.linalg LU (dense Schur factor),
scipy.sparse.linalg.gmres (iterative pressure path), scipy.spatial.cKDTree
(setup-time neighbour search).
"""
from __future__ import annotations

import time
import warnings
from types import SimpleNamespace

import numpy as np
import scipy.sparse as sp
from scipy.fft import dct, idct, dst, idst
from scipy.linalg import LinAlgWarning, lu_factor, lu_solve
from scipy.sparse.linalg import LinearOperator, gmres
from scipy.spatial import cKDTree

EPS = np.finfo(float).eps


# ---------------------------------------------------------------------------
# geometry  (solver/ghost_cell.py:12-63)
# ---------------------------------------------------------------------------
class Circle:
    """Signed distance and outward normal of a circle (solver/ghost_cell.py:12-30)."""

    def __init__(self, xc, yc, radius):
        self.xc, self.yc, self.radius = xc, yc, radius

    def distance(self, x, y):
        return np.sqrt((x - self.xc) ** 2 + (y - self.yc) ** 2) - self.radius

    def normal(self, x, y):
        r = np.maximum(np.sqrt((x - self.xc) ** 2 + (y - self.yc) ** 2), 1e-14)
        return (x - self.xc) / r, (y - self.yc) / r


def staggered_coordinates(nx, ny, dx, dy):
    """Face and centre coordinates of the MAC grid (solver/ghost_cell.py:48-53)."""
    xu = np.arange(nx + 1) * dx
    yu = (np.arange(ny) + 0.5) * dy
    xv = (np.arange(nx) + 0.5) * dx
    yv = np.arange(ny + 1) * dy
    return dict(u=(xu, yu), v=(xv, yv), p=(xv, yu))


# ---------------------------------------------------------------------------
# ghost extension  (solver/optimized_ghost_cell.py:14-58)
# ---------------------------------------------------------------------------
def ghost_extension(x, y, shape_sdf, active, *, neumann=False, interpolation='bilinear'):
    """Extension matrix E (grid <- active unknowns) with quadratic-normal ghost rows.

    Ghost rows are grid points with -2h <= distance <= 1e-13.  Each takes two
    probes at distances s and 2s along the normal (s = max(d, 1.5h), grown by
    1.25 up to eight times until every probe stencil is active) and the
    Dirichlet (or Neumann) quadratic weights of
    solver/optimized_ghost_cell.py:53-54.
    """
    if interpolation not in ('bilinear', 'biquadratic'):
        raise ValueError('Unknown ghost probe interpolation')
    X, Y = np.meshgrid(x, y)
    dist = shape_sdf.distance(X, Y)
    ids = np.flatnonzero(active)
    label = -np.ones(active.shape, dtype=np.int64)
    label.ravel()[ids] = np.arange(ids.size)
    step_x, step_y = x[1] - x[0], y[1] - y[0]
    h = max(step_x, step_y)
    quad = interpolation == 'biquadratic'
    width = 3 if quad else 2
    r_rows, r_cols, r_vals = [ids], [np.arange(ids.size)], [np.ones(ids.size)]
    gj, gi = np.nonzero((dist <= 1e-13) & (dist >= -2 * h))
    for j, i in zip(gj, gi):
        d = max(0.0, -dist[j, i])
        n_x, n_y = shape_sdf.normal(x[i], y[j])
        s = max(d, 1.5 * h)
        for _attempt in range(8):
            probes = []
            for ell in (s, 2 * s):
                fx = (x[i] + (d + ell) * n_x - x[0]) / step_x
                fy = (y[j] + (d + ell) * n_y - y[0]) / step_y
                if quad:
                    i0, j0 = int(np.floor(fx + 0.5)) - 1, int(np.floor(fy + 0.5)) - 1
                else:
                    i0, j0 = int(np.floor(fx)), int(np.floor(fy))
                if not (0 <= i0 <= len(x) - width and 0 <= j0 <= len(y) - width):
                    raise ValueError('Ghost probe reaches an outer boundary')
                cols = label[j0:j0 + width, i0:i0 + width].ravel()
                a, b = fx - i0, fy - j0
                if quad:
                    wx = np.array([0.5 * (a - 1) * (a - 2), -a * (a - 2), 0.5 * a * (a - 1)])
                    wy = np.array([0.5 * (b - 1) * (b - 2), -b * (b - 2), 0.5 * b * (b - 1)])
                    w = np.outer(wy, wx).ravel()
                else:
                    w = np.array([(1 - a) * (1 - b), a * (1 - b), (1 - a) * b, a * b])
                probes.append((cols, w))
            if all((c >= 0).all() for c, _ in probes):
                break
            s *= 1.25
        else:
            raise ValueError('No exterior ghost stencil')
        if neumann:
            f = ((4 * s * s - d * d) / (3 * s * s), (d * d - s * s) / (3 * s * s))
        else:
            f = (-d * (d + 2 * s) / (s * s), d * (d + s) / (2 * s * s))
        for fk, (cols, w) in zip(f, probes):
            r_rows.append(np.full(cols.size, j * len(x) + i))
            r_cols.append(cols)
            r_vals.append(fk * w)
    E = sp.csr_matrix((np.concatenate(r_vals), (np.concatenate(r_rows), np.concatenate(r_cols))),
                      shape=(active.size, ids.size))
    return E, ids


def quadratic_pressure_extension(x, y, shape_sdf, active):
    """Least-squares exterior pressure continuation (solver/ghost_reconstruction.py:7-45)."""
    X, Y = np.meshgrid(x, y)
    dist = shape_sdf.distance(X, Y)
    hx, hy = x[1] - x[0], y[1] - y[0]
    h = max(hx, hy)
    ids = np.flatnonzero(active)
    label = -np.ones(active.size, dtype=np.int64)
    label[ids] = np.arange(ids.size)
    pool = np.flatnonzero(active & (dist < 6 * h))
    if pool.size < 12:
        raise ValueError('Pressure continuation needs twelve exterior centers')
    ghosts = np.flatnonzero((dist <= 1e-13) & (dist >= -2 * h))
    pts = np.column_stack((Y.ravel()[pool], X.ravel()[pool]))
    tree = cKDTree(pts)
    rows, cols, vals = [ids], [np.arange(ids.size)], [np.ones(ids.size)]
    conds, errs, counts = [], [], []
    target = np.array([1.0, 0, 0, 0, 0, 0])
    for g in ghosts:
        at = np.array([Y.ravel()[g], X.ravel()[g]])
        for k in (12, 20, 32):
            rad, _ = tree.query(at, k=min(k, len(pts)))
            near = tree.query_ball_point(at, rad[-1] * (1 + 1e-12))
            oy, ox = ((pts[near] - at) / [hy, hx]).T
            basis = np.array([np.ones(len(near)), ox, oy, ox * ox, ox * oy, oy * oy])
            w, _, rank, _ = np.linalg.lstsq(basis, target, rcond=1e-12)
            cond = float(np.linalg.cond(basis))
            w[np.argmax(abs(w))] += 1 - w.sum()
            err = float(np.max(abs(basis @ w - target)))
            if rank == 6 and np.isfinite(cond) and cond <= 1e8 and err <= 1e-10:
                break
        else:
            raise ValueError('Unresolved exterior pressure polynomial')
        rows.append(np.full(len(near), g))
        cols.append(label[pool[near]])
        vals.append(w)
        conds.append(cond)
        errs.append(err)
        counts.append(len(near))
    P = sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))),
                      shape=(active.size, ids.size))
    return P, ids, dict(stencil_condition_max=max(conds, default=0.0),
                        polynomial_reproduction_linf=max(errs, default=0.0),
                        neighbor_count_max=max(counts, default=0))


# ---------------------------------------------------------------------------
# surface quadrature  (solver/cut_cell_solver.py:25-77,
#                      solver/optimized_ghost_cell.py:144-172)
# ---------------------------------------------------------------------------
def point_pressure_operator(g, points):
    """12-NN quadratic point-pressure weights (solver/cut_cell_solver.py:25-67)."""
    points = np.asarray(points, dtype=float)
    pad = 4 * max(g.dx, g.dy)
    lo = np.maximum(0, np.floor((points.min(axis=0) - pad) / [g.dy, g.dx]).astype(int))
    hi = np.minimum([g.ny, g.nx], np.ceil((points.max(axis=0) + pad) / [g.dy, g.dx]).astype(int) + 1)
    J, I = np.meshgrid(np.arange(lo[0], hi[0]), np.arange(lo[1], hi[1]), indexing='ij')
    yc, xc = (J + 0.5) * g.dy, (I + 0.5) * g.dx
    outside = (g.cell_type[J, I] != -1) & (np.hypot(xc - g.xc, yc - g.yc) >= g.R * (1 - 1e-12))
    flat = (J * g.nx + I)[outside]
    if flat.size < 12:
        raise ValueError('Pressure reconstruction needs at least 12 exterior centers')
    pts = np.column_stack((yc[outside], xc[outside]))
    tree = cKDTree(pts)
    dk, _ = tree.query(points, k=12)
    groups = tree.query_ball_point(points, dk[:, -1] * (1 + 1e-12))
    rows, cols, vals = [], [], []
    for k, near in enumerate(groups):
        oy, ox = ((pts[near] - points[k]) / [g.dy, g.dx]).T
        basis = np.array([np.ones(len(near)), ox, oy, ox * ox, ox * oy, oy * oy])
        w, _, rank, _ = np.linalg.lstsq(basis, [1.0, 0, 0, 0, 0, 0], rcond=1e-12)
        if rank != 6:
            raise ValueError('Pressure stencil cannot resolve a quadratic polynomial')
        rows.extend([k] * len(near))
        cols.extend(flat[near])
        vals.extend(w)
    return sp.csr_matrix((vals, (rows, cols)), shape=(len(points), g.nx * g.ny))


def surface_points(g):
    """Quadrature points, pressure operator and weighted normals (solver/cut_cell_solver.py:70-77)."""
    count = max(360, 4 * int(np.ceil(2 * np.pi * g.R / min(g.dx, g.dy))))
    theta = np.arange(count) * (2 * np.pi / count)
    normals = np.column_stack((np.cos(theta), np.sin(theta)))
    pts = np.column_stack((g.yc + g.R * normals[:, 1], g.xc + g.R * normals[:, 0]))
    return pts, point_pressure_operator(g, pts), normals * (2 * np.pi * g.R / count)


def wall_normal_derivative(g, x, y, active, pts):
    """14-NN LSQ d/dn at circle points (solver/optimized_ghost_cell.py:152-172)."""
    X, Y = np.meshgrid(x, y)
    h = max(g.dx, g.dy)
    rad = np.hypot(X - g.xc, Y - g.yc)
    ids = np.flatnonzero(active & (rad < g.R + 6 * h))
    xy = np.column_stack((Y.ravel()[ids], X.ravel()[ids]))
    tree = cKDTree(xy)
    dk, _ = tree.query(pts, k=14)
    groups = tree.query_ball_point(pts, dk[:, -1] * (1 + 1e-12))
    rows, cols, vals = [], [], []
    for k, near in enumerate(groups):
        ys, xs = xy[near].T
        theta = np.arctan2(pts[k, 0] - g.yc, pts[k, 1] - g.xc)
        ang = np.arctan2(ys - g.yc, xs - g.xc) - theta
        nn = (np.hypot(xs - g.xc, ys - g.yc) - g.R) / h
        tt = g.R * np.arctan2(np.sin(ang), np.cos(ang)) / h
        w, _, rank, _ = np.linalg.lstsq(np.array([nn, nn * nn, nn * tt]), [1 / h, 0.0, 0.0], rcond=1e-12)
        if rank != 3:
            raise ValueError('Unresolved wall-gradient stencil')
        rows.extend([k] * len(near))
        cols.extend(ids[near])
        vals.extend(w)
    return sp.csr_matrix((vals, (rows, cols)), shape=(len(pts), active.size))


# ---------------------------------------------------------------------------
# separable rectangle inverses  (solver/rectangular_inverse.py:8-58)
# ---------------------------------------------------------------------------
RECT_KINDS = {
    # kind: (rows-from-ny offset, diag ends x (left,right), diag ends y (lower,upper),
    #        x-frequency offset, y-frequency offset, x type, y type, transform family)
    'pressure': (0, (1.0, 3.0), (1.0, 1.0), 0.5, 0.0, 4, 2, 'cos'),
    'u': (0, (2.0, 2.0), (3.0, 3.0), 0.5, 1.0, 3, 2, 'sin'),
    'v': (1, (3.0, 1.0), (2.0, 2.0), 0.5, 1.0, 4, 1, 'sin'),
}


def rectangle(nx, ny, dx, dy, kind, nu=0.0, dt=0.0, rho=1.0, self_check=True):
    """Rectangle operator, its separable DCT/DST inverse and grid shape.

    Follows solver/rectangular_inverse.py:8-58: pressure uses DCT-IV (x) and
    DCT-II (y); u uses DST-III (x) and DST-II (y); v uses DST-IV (x) and DST-I
    (y) on ny-1 rows.  The inverse is checked against the assembled rectangle
    to 1e-10 (solver/rectangular_inverse.py:54-57).
    """
    if kind not in RECT_KINDS:
        raise ValueError('Unknown rectangular MAC field')
    drop, (left, right), (lower, upper), fx, fy, tx, ty, family = RECT_KINDS[kind]
    cols, rows = nx, ny - drop
    sx = (np.arange(cols) + fx) * np.pi / (2 * nx)
    sy = (np.arange(rows) + fy) * np.pi / (2 * ny)
    main_x = np.full(cols, -2.0)
    main_x[0], main_x[-1] = -left, -right
    main_y = np.full(rows, -2.0)
    main_y[0], main_y[-1] = -lower, -upper
    sub_x = np.ones(cols - 1)
    if kind == 'u':
        sub_x[-1] = 2.0
    lx = sp.diags((sub_x, main_x, np.ones(cols - 1)), (-1, 0, 1), format='csr') / dx ** 2
    ly = sp.diags((np.ones(rows - 1), main_y, np.ones(rows - 1)), (-1, 0, 1), format='csr') / dy ** 2
    lap = sp.kron(sp.eye(rows), lx) + sp.kron(ly, sp.eye(cols))
    rates = 4 * np.sin(sy[:, None]) ** 2 / dy ** 2 + 4 * np.sin(sx[None, :]) ** 2 / dx ** 2
    if kind == 'pressure':
        matrix = (lap / rho).tocsc()
        divisor = -rates / rho
    else:
        matrix = (sp.eye(cols * rows) - 0.5 * dt * nu * lap).tocsc()
        divisor = 1 + 0.5 * dt * nu * rates
    fwd, bwd = (dct, idct) if family == 'cos' else (dst, idst)

    def solve(b):
        t = fwd(fwd(b, type=tx, axis=1), type=ty, axis=0)
        t /= divisor
        return bwd(bwd(t, type=ty, axis=0), type=tx, axis=1)

    if self_check:
        probe = np.random.default_rng(17).normal(size=(rows, cols))
        err = np.max(abs(matrix @ solve(probe).ravel() - probe.ravel()))
        if err > 1e-10:
            raise RuntimeError(f'Rectangular transform mismatch: {kind}, {err:g}')
    return matrix, solve, (rows, cols)


# ---------------------------------------------------------------------------
# boundary Schur correction and monitored solver  (solver/pressure_schur.py)
# ---------------------------------------------------------------------------
def schur_rows(actual, indices, rect):
    """Rows where the extended operator differs from the rectangle
    (solver/pressure_schur.py:77-91): returns (rows, delta csr, tolerance)."""
    indices = np.asarray(indices)
    covered = np.ones(rect.shape[0], bool)
    covered[indices] = False
    a = actual.tocoo()
    ext = sp.csr_matrix((a.data, (indices[a.row], indices[a.col])), shape=rect.shape)
    r = rect.tocoo()
    keep = covered[r.row] & covered[r.col]
    ext += sp.csr_matrix((r.data[keep], (r.row[keep], r.col[keep])), shape=rect.shape)
    delta = (ext - rect).tocsr()
    tol = 8 * EPS * max(1.0, float(np.max(abs(rect.diagonal()))))
    delta.data[abs(delta.data) < tol] = 0.0
    delta.eliminate_zeros()
    rows = np.flatnonzero(np.diff(delta.indptr))
    return rows, delta, tol


def boundary_schur_inverse(actual, indices, rect, inverse, shape):
    """Exact low-rank correction of the separable inverse
    (solver/pressure_schur.py:75-124), with two refinement sweeps."""
    indices = np.asarray(indices)
    rows, delta, tol = schur_rows(actual, indices, rect)
    if len(rows) > 2048:
        raise ValueError('Ghost inverse exceeds the bounded boundary-row rank')
    C = delta[rows]
    S = np.eye(len(rows))
    unit = np.zeros(shape)
    for c, r in enumerate(rows):
        unit.ravel()[r] = 1.0
        S[:, c] += C @ inverse(unit).ravel()
        unit.ravel()[r] = 0.0
    with warnings.catch_warnings():
        warnings.simplefilter('error', LinAlgWarning)
        lu = lu_factor(S)
    grid = np.zeros(shape)

    def apply(values):
        grid.fill(0.0)
        grid.ravel()[indices] = values
        first = inverse(grid)
        grid.fill(0.0)
        grid.ravel()[rows] = lu_solve(lu, C @ first.ravel())
        return (first - inverse(grid)).ravel()[indices]

    info = dict(rank=len(rows), dense_bytes=int(S.nbytes), roundoff_drop_tolerance=tol)

    def solve(values):
        x = apply(values)
        target = max(1e-10, 32 * EPS * max(1.0, float(np.max(abs(values)))))
        sweeps = 0
        for _ in range(2):
            res = values - actual @ x
            if np.max(abs(res)) <= target:
                break
            x += apply(res)
            sweeps += 1
        info['last_refinement_iterations'] = sweeps
        return x

    solve.rows, solve.schur = rows, S
    return solve, info


def monitored_solver(actual, indices, rect, inverse, shape, *, iterative=False):
    """Direct (Schur) or GMRES pressure solve with the true-residual and
    roundoff gate (solver/pressure_schur.py:16-72)."""
    indices = np.asarray(indices)
    absA = abs(actual).tocsr()
    weights = (2 * np.diff(absA.indptr) + 2) * EPS
    if iterative:
        def precondition(vals):
            g = np.zeros(shape)
            g.ravel()[indices] = vals
            return inverse(g).ravel()[indices]
        M = LinearOperator(actual.shape, matvec=precondition, dtype=float)
        info = dict(backend='gmres_rectangle', preconditioner='separable_rectangle',
                    krylov_rtol=1e-12, krylov_atol=1e-12)
        direct = None
    else:
        direct, info = boundary_schur_inverse(actual, indices, rect, inverse, shape)
        info['backend'] = 'fft_boundary_schur'

    def solve(values):
        t0 = time.perf_counter()
        if not np.isfinite(values).all():
            raise ValueError('Pressure RHS must be finite')
        its = [0]

        def count(_):
            its[0] += 1

        def krylov(b):
            return gmres(actual, b, M=M, rtol=info['krylov_rtol'], atol=info['krylov_atol'],
                         restart=50, maxiter=100, callback=count, callback_type='pr_norm')

        if iterative:
            x, status = krylov(values)
        else:
            x, status = direct(values), 0
        res = values - actual @ x
        target = max(1e-10, 64 * EPS * max(1.0, float(np.max(abs(values)))))
        sweeps = info.get('last_refinement_iterations', 0)
        if iterative:
            sweeps = 0
            for _ in range(2):
                if status or np.max(abs(res)) <= target:
                    break
                dx_, status = krylov(res)
                x += dx_
                res = values - actual @ x
                sweeps += 1
        linf = float(np.max(abs(res)))
        rel = float(np.linalg.norm(res) / max(np.linalg.norm(values), np.finfo(float).tiny))
        scale = absA @ abs(x) + abs(values)
        bound = float(np.max(weights * scale))
        target = max(target, bound)
        info['last_solve'] = dict(iterations=its[0], residual_linf=linf, residual_relative_l2=rel,
                                  refinement_iterations=sweeps, residual_target_linf=target,
                                  roundoff_bound_linf=bound,
                                  backward_error_linf=linf / max(float(np.max(scale)), np.finfo(float).tiny),
                                  status=int(status), seconds=time.perf_counter() - t0)
        if status or not np.isfinite(x).all() or linf > target:
            raise RuntimeError(f'Pressure solve failed: {info["last_solve"]}')
        return x

    return solve, info


# ---------------------------------------------------------------------------
# flux-form centred advection  (solver/numba_kernels.py:17-142 with nu=0,
# unit apertures, rho=1; packing/scaling solver/optimized_ghost_cell.py:186-199)
# ---------------------------------------------------------------------------
def advective_acceleration(u, v, dx, dy):
    """Return (ru, rv): -N(u), -N(v) flux sums on the full staggered grids (not yet /dxdy)."""
    ny, nx1 = u.shape
    nx = nx1 - 1
    uf = 0.5 * (u[:, :-1] + u[:, 1:])                     # u at centres
    fxx = -((uf * uf) * dy)                                # (ny, nx)
    fxy = np.zeros((ny + 1, nx + 1))
    vface = np.empty((ny - 1, nx + 1))
    vface[:, 0] = v[1:ny, 0]
    vface[:, nx] = v[1:ny, nx - 1]
    vface[:, 1:nx] = 0.5 * (v[1:ny, :-1] + v[1:ny, 1:])
    uadv = 0.5 * (u[:-1, :] + u[1:, :])
    fxy[1:ny] = -((vface * uadv) * dx)
    ru = np.zeros_like(u)
    ru[:, 1:nx] = (fxx[:, 1:] - fxx[:, :-1]) + (fxy[1:, 1:nx] - fxy[:-1, 1:nx])
    ru[:, nx] = (-u[:, nx] * u[:, nx]) * dy - fxx[:, nx - 1] + 0.5 * (fxy[1:, nx] - fxy[:-1, nx])

    vf = 0.5 * (v[:-1, :] + v[1:, :])
    fyy = -((vf * vf) * dx)                                # (ny, nx)
    fyx = np.zeros((ny + 1, nx + 1))
    uface = np.empty((ny + 1, nx - 1))
    uface[0] = u[0, 1:nx]
    uface[ny] = u[ny - 1, 1:nx]
    uface[1:ny] = 0.5 * (u[:-1, 1:nx] + u[1:, 1:nx])
    vadv = 0.5 * (v[:, :-1] + v[:, 1:])
    fyx[:, 1:nx] = -((uface * vadv) * dy)
    uout = np.empty(ny + 1)
    uout[0], uout[ny] = u[0, nx], u[ny - 1, nx]
    uout[1:ny] = 0.5 * (u[:-1, nx] + u[1:, nx])
    fyx[:, nx] = (-uout * v[:, nx - 1]) * dy
    rv = np.zeros_like(v)
    rv[1:ny] = (fyx[1:ny, 1:] - fyx[1:ny, :-1]) + (fyy[1:] - fyy[:-1])
    return ru, rv


# ---------------------------------------------------------------------------
# operators  (solver/optimized_ghost_cell.py:61-150)
# ---------------------------------------------------------------------------
class GhostOperators:
    """Discrete operators of the ghost-cell AB2/CN path
    (solver/optimized_ghost_cell.py:61-234)."""

    def __init__(self, nx, ny, Lx, Ly, D, xc, yc, nu, rho, u_inlet, *,
                 pressure_extension='neumann', velocity_interpolation='bilinear',
                 pressure_solver='direct'):
        self.nx, self.ny = nx, ny
        self.dx, self.dy = Lx / nx, Ly / ny
        dx, dy = self.dx, self.dy
        self.nu, self.rho, self.diameter = nu, rho, D
        self.shape_sdf = Circle(xc, yc, D / 2.0)
        coords = staggered_coordinates(nx, ny, dx, dy)
        self.coords = coords
        dist = {k: self.shape_sdf.distance(*np.meshgrid(*coords[k])) for k in coords}
        self.dist = dist
        act_u = dist['u'] > 1e-13
        act_v = dist['v'] > 1e-13
        act_u[:, 0] = False
        act_v[[0, -1]] = False
        act_p = dist['p'] > 1e-13
        self.active = dict(u=act_u, v=act_v, p=act_p)
        eu, self.ui = ghost_extension(*coords['u'], self.shape_sdf, act_u, interpolation=velocity_interpolation)
        ev, self.vi = ghost_extension(*coords['v'], self.shape_sdf, act_v, interpolation=velocity_interpolation)
        self.Eu, self.Ev = eu, ev
        self.reconstruction_info = dict(velocity=velocity_interpolation, pressure=pressure_extension)
        if pressure_extension == 'quadratic':
            self.P, self.pi, fit = quadratic_pressure_extension(*coords['p'], self.shape_sdf, act_p)
            self.reconstruction_info.update(fit)
        else:
            self.P, self.pi = ghost_extension(*coords['p'], self.shape_sdf, act_p, neumann=True)
        self.ushape, self.vshape, self.pshape = (ny, nx + 1), (ny + 1, nx), (ny, nx)
        self.usize = (nx + 1) * ny
        self.E = sp.block_diag((eu, ev), format='csr')
        self.nu_act = len(self.ui)
        self.qsize = len(self.ui) + len(self.vi)
        self.offset = np.zeros(self.E.shape[0])
        self.offset[:self.usize].reshape(self.ushape)[:, 0] = u_inlet
        # divergence on active cells (solver/optimized_ghost_cell.py:85-93)
        jp, ip = np.unravel_index(self.pi, self.pshape)
        n = len(self.pi)
        r = np.arange(n)
        fu = jp * (nx + 1) + ip
        fv = self.usize + jp * nx + ip
        self.Dfull = sp.csr_matrix(
            (np.concatenate((-np.ones(n) / dx, np.ones(n) / dx, -np.ones(n) / dy, np.ones(n) / dy)),
             (np.tile(r, 4), np.concatenate((fu, fu + 1, fv, fv + nx)))), shape=(n, self.E.shape[0]))
        self.D = (self.Dfull @ self.E).tocsr()
        self.div_offset = self.Dfull @ self.offset
        # gradient at active faces (solver/optimized_ghost_cell.py:94-107)
        ju, iu = np.unravel_index(self.ui, self.ushape)
        jv, iv = np.unravel_index(self.vi, self.vshape)
        self.outlet_u = np.flatnonzero(iu == nx)
        ru = np.arange(len(self.ui))
        inner = iu < nx
        rv = len(ru) + np.arange(len(self.vi))
        g_rows = np.concatenate((ru[inner], ru[inner], ru[~inner], rv, rv))
        g_cols = np.concatenate((ju[inner] * nx + iu[inner], ju[inner] * nx + iu[inner] - 1,
                                 ju[~inner] * nx + nx - 1, jv * nx + iv, (jv - 1) * nx + iv))
        g_vals = np.concatenate((np.full(inner.sum(), 1 / dx), np.full(inner.sum(), -1 / dx),
                                 np.full((~inner).sum(), -2 / dx), np.full(len(rv), 1 / dy),
                                 np.full(len(rv), -1 / dy)))
        raw_g = sp.csr_matrix((g_vals, (g_rows, g_cols)), shape=(self.qsize, nx * ny))
        self.G = (raw_g @ self.P / rho).tocsr()
        self.A = (self.D @ self.G).tocsc()
        rect_p, inv_p, shape_p = rectangle(nx, ny, dx, dy, 'pressure', rho=rho)
        self.pressure_solve, self.pressure_info = monitored_solver(
            self.A, self.pi, rect_p, inv_p, shape_p, iterative=pressure_solver == 'iterative')
        self.pressure_calls = []
        # viscous operator (solver/optimized_ghost_cell.py:113-128)
        L_rows, L_cols, L_vals = [], [], []

        def put(rw, cl, val):
            L_rows.append(rw)
            L_cols.append(cl)
            L_vals.append(np.broadcast_to(val, rw.shape))

        put(ru, self.ui, -2 / dx ** 2 - np.where((ju == 0) | (ju == ny - 1), 3.0, 2.0) / dy ** 2)
        put(ru, self.ui - 1, np.where(iu == nx, 2.0, 1.0) / dx ** 2)
        put(ru[inner], self.ui[inner] + 1, 1 / dx ** 2)
        put(ru[ju < ny - 1], self.ui[ju < ny - 1] + nx + 1, 1 / dy ** 2)
        put(ru[ju > 0], self.ui[ju > 0] - nx - 1, 1 / dy ** 2)
        put(rv, self.usize + self.vi, -np.where(iv == 0, 3.0, np.where(iv == nx - 1, 1.0, 2.0)) / dx ** 2 - 2 / dy ** 2)
        put(rv[iv < nx - 1], self.usize + self.vi[iv < nx - 1] + 1, 1 / dx ** 2)
        put(rv[iv > 0], self.usize + self.vi[iv > 0] - 1, 1 / dx ** 2)
        put(rv, self.usize + self.vi + nx, 1 / dy ** 2)
        put(rv, self.usize + self.vi - nx, 1 / dy ** 2)
        self.raw_l = sp.csr_matrix((np.concatenate(L_vals), (np.concatenate(L_rows), np.concatenate(L_cols))),
                                   shape=(self.qsize, self.E.shape[0]))
        self.L = (nu * self.raw_l @ self.E).tocsr()
        self.diff_offset = nu * (self.raw_l @ self.offset)
        # surface quadrature (solver/optimized_ghost_cell.py:142-148)
        self.geom = SimpleNamespace(nx=nx, ny=ny, dx=dx, dy=dy, Lx=Lx, Ly=Ly, xc=xc, yc=yc, R=D / 2,
                                    cell_type=np.where(act_p, 1, -1))
        self.surface_points, self.pressure_surface, self.normal_weights = surface_points(self.geom)
        self.normals = self.normal_weights / (np.pi * D / len(self.surface_points))
        self.du_dn = wall_normal_derivative(self.geom, *coords['u'], act_u, self.surface_points)
        self.dv_dn = wall_normal_derivative(self.geom, *coords['v'], act_v, self.surface_points)
        self.helmholtz_dt = None
        self.helmholtz = None

    # -- grid <-> packed vectors (solver/optimized_ghost_cell.py:174-184)
    def pack(self, u, v):
        return np.concatenate((u.ravel()[self.ui], v.ravel()[self.vi]))

    def unpack(self, q):
        f = self.E @ q + self.offset
        return f[:self.usize].reshape(self.ushape).copy(), f[self.usize:].reshape(self.vshape).copy()

    def set_inlet(self, u_inlet):
        """Refresh inlet-dependent offsets (solver/optimized_ghost_cell.py:238-242)."""
        col = self.offset[:self.usize].reshape(self.ushape)[:, 0]
        if not np.array_equal(col, u_inlet):
            col[:] = u_inlet
            self.div_offset = self.Dfull @ self.offset
            self.diff_offset = self.nu * (self.raw_l @ self.offset)

    # -- operators (solver/optimized_ghost_cell.py:186-234)
    def advection(self, q):
        u, v = self.unpack(q)
        ru, rv = advective_acceleration(u, v, self.dx, self.dy)
        out = self.pack(ru, rv) / (self.dx * self.dy)
        out[self.outlet_u] *= 2
        return out

    def diffusion(self, q):
        return self.L @ q + self.diff_offset

    def gradient(self, p):
        # The reference's CSR kernel indexes a raveled 2-D input without a size
        # check, so a full pressure grid acts through its first len(pi) entries
        # (solver/optimized_ghost_cell.py:207-210, solver/numba_kernels.py:347-354).
        x = p.ravel() if p.ndim > 1 else p
        return self.G @ x[:self.G.shape[1]]

    def divergence(self, q):
        return self.D @ q + self.div_offset

    def H_matvec(self, x, dt):
        return x - 0.5 * dt * (self.L @ x)

    def project(self, q, dt):
        rhs = self.divergence(q) / dt
        phi = self.pressure_solve(rhs)
        self.pressure_calls.append(dict(self.pressure_info['last_solve']))
        out = q - dt * (self.G @ phi)
        err = float(np.max(abs(self.divergence(out))))
        if err > 1e-10 or not np.isfinite(out).all():
            raise RuntimeError(f'Ghost projection failed: divergence={err:g}')
        return out, phi

    def build_helmholtz(self, dt):
        """Per-dt CN Helmholtz Schur solves (solver/optimized_ghost_cell.py:243-255)."""
        nx, ny, nq = self.nx, self.ny, self.nu_act
        ju, iu = np.unravel_index(self.ui, self.ushape)
        jv, iv = np.unravel_index(self.vi, self.vshape)
        solves, infos = [], []
        for kind, sel, block in (('u', ju * nx + iu - 1, self.L[:nq, :nq]),
                                 ('v', (jv - 1) * nx + iv, self.L[nq:, nq:])):
            rect, inv, shape = rectangle(nx, ny, self.dx, self.dy, kind, self.nu, dt, self.rho)
            actual = (sp.eye(block.shape[0], format='csc') - 0.5 * dt * block).tocsc()
            s, info = boundary_schur_inverse(actual, sel, rect, inv, shape)
            solves.append(s)
            infos.append(info)
        self.helmholtz_parts = solves
        self.helmholtz_info = infos
        self.helmholtz = lambda b: np.concatenate((solves[0](b[:nq]), solves[1](b[nq:])))
        self.helmholtz_dt = dt

    def surface_forces(self, u, v, p, mu):
        """Pressure and viscous force on the circle (solver/optimized_ghost_cell.py:280-286)."""
        ps = self.pressure_surface @ p.ravel()
        dn = np.column_stack((self.du_dn @ u.ravel(), self.dv_dn @ v.ravel()))
        tr = mu * (dn + self.normals * np.sum(dn * self.normals, axis=1)[:, None])
        fp = -np.sum(ps[:, None] * self.normal_weights, axis=0)
        fv = np.sum(tr, axis=0) * (np.pi * self.diameter / len(ps))
        return (*(fp + fv), *fp, *fv)


# ---------------------------------------------------------------------------
# AB2/CN step  (solver/time_integration.py:7-145)
# ---------------------------------------------------------------------------
def ab2_cn_step(ops, q, pressure, dt, prev_adv=None, prev_dt=None):
    """One AB2/CN step with discrete incremental pressure (solver/time_integration.py:7-145).

    Returns (q_new, half_pressure, output_pressure, advection_now, diagnostics).
    """
    if not np.isfinite(dt) or dt <= 0 or not np.isfinite(q).all() or not np.isfinite(pressure).all():
        raise ValueError('Finite fields and a positive timestep are required')
    now = ops.advection(q)
    if prev_adv is None:
        mid = q + 0.5 * dt * (now + ops.diffusion(q) - ops.gradient(pressure))
        half, _ = ops.project(mid, 0.5 * dt)
        explicit = ops.advection(half)
    else:
        if prev_dt is None or not np.isfinite(prev_dt) or prev_dt <= 0:
            raise ValueError('AB2 history requires a finite positive previous timestep')
        a = dt / (2 * prev_dt)
        explicit = (1 + a) * now - a * prev_adv
    off = ops.diff_offset
    diff_q = ops.diffusion(q)
    grad_p = ops.gradient(pressure)
    rhs = q + dt * (explicit + 0.5 * diff_q - grad_p) + 0.5 * dt * off
    if ops.helmholtz_dt != dt:
        ops.build_helmholtz(dt)
    star = ops.helmholtz(rhs)
    res = float(np.max(abs(ops.H_matvec(star, dt) - rhs)))
    if not np.isfinite(star).all() or res > 1e-10 * max(1.0, float(np.max(abs(rhs)))):
        raise RuntimeError(f'CN momentum solve failed: info=0, residual={res:g}')
    result, _ = ops.project(star, dt)
    action = ops.H_matvec(result, dt)
    defect = rhs - action
    _, inc = ops.project(result + defect, dt)
    half_p = pressure + inc
    factor = 1.0 if prev_adv is None else dt / (dt + prev_dt)
    out_p = half_p + factor * inc
    coupled = action - rhs + dt * ops.gradient(inc)
    return result, half_p, out_p, now, dict(momentum_iterations=0, momentum_residual_linf=res,
                                            coupled_momentum_residual_linf=float(np.max(abs(coupled))))


# ---------------------------------------------------------------------------
# case driver  (solver/main.py:40-242 ghost/ab2_cn branch, :245-501 loop)
# ---------------------------------------------------------------------------
class CylinderCase:
    """Ghost-cell AB2/CN cylinder case: constructor, step loop, forces and gates
    (solver/main.py:40-242, 245-501)."""

    def __init__(self, nx=400, ny=100, Lx=20.0, Ly=5.0, D=1.0, xc=5.0, yc=2.5, nu=0.01, rho=1.0,
                 U_inf=1.0, inflow='uniform', U_m=None, pressure_solver='direct',
                 ghost_pressure_extension='neumann', ghost_velocity_interpolation='bilinear'):
        if pressure_solver not in ('direct', 'iterative'):
            raise ValueError('Ghost AB2/CN requires direct/iterative pressure')
        if ghost_pressure_extension not in ('neumann', 'quadratic') or \
                ghost_velocity_interpolation not in ('bilinear', 'biquadratic'):
            raise ValueError('Unknown Ghost pressure extension or velocity interpolation')
        if any(isinstance(n, bool) or not isinstance(n, (int, np.integer)) or n < 4 for n in (nx, ny)):
            raise ValueError('nx and ny must be integers >= 4')
        if not all(np.isfinite(x) and x > 0 for x in (Lx, Ly, D, nu, rho, U_inf)):
            raise ValueError('Domain lengths, D, nu, rho and U_inf must be finite and positive')
        if inflow not in ('uniform', 'parabolic'):
            raise ValueError('inflow must be uniform or parabolic')
        if not (D / 2 < xc < Lx - D / 2 and D / 2 < yc < Ly - D / 2):
            raise ValueError('Cylinder must lie strictly inside the channel')
        self.nx, self.ny, self.Lx, self.Ly = nx, ny, Lx, Ly
        self.dx, self.dy = Lx / nx, Ly / ny
        self.D, self.xc, self.yc, self.nu, self.rho, self.U_inf = D, xc, yc, nu, rho, U_inf
        self.inflow = inflow
        if inflow == 'parabolic':
            self.U_m = 1.5 * U_inf if U_m is None else U_m
            self.U_ref = (2.0 / 3.0) * self.U_m
        else:
            self.U_m = self.U_ref = U_inf
        yc_ = (np.arange(ny) + 0.5) * self.dy
        xc_ = (np.arange(nx) + 0.5) * self.dx
        self.y_centers = yc_
        rr = (((xc_ - xc) / (D / 2.0)) ** 2)[None, :] + (((yc_ - yc) / (D / 2.0)) ** 2)[:, None]
        self.mask = rr <= (1.0 + 1e-13)
        if not self.mask.any() or self.mask[[0, -1], :].any() or self.mask[:, [0, -1]].any():
            raise ValueError('Grid must resolve the cylinder and a fluid layer at every outer boundary')
        if inflow == 'parabolic':
            self.u_inlet = 4.0 * self.U_m * yc_ * (Ly - yc_) / (Ly ** 2)
        else:
            self.u_inlet = np.full(ny, U_inf, dtype=float)
        self.u_inlet_base = self.u_inlet.copy()
        self.u = np.repeat(self.u_inlet[:, None], nx + 1, axis=1)
        self.v = np.zeros((ny + 1, nx))
        self.p = np.zeros((ny, nx))
        jj, ii = np.nonzero(self.mask)
        self.u[jj, ii] = 0.0
        self.u[jj, ii + 1] = 0.0
        self.v[jj, ii] = 0.0
        self.v[jj + 1, ii] = 0.0
        self.ops = GhostOperators(nx, ny, Lx, Ly, D, xc, yc, nu, rho, self.u_inlet,
                                  pressure_extension=ghost_pressure_extension,
                                  velocity_interpolation=ghost_velocity_interpolation,
                                  pressure_solver=pressure_solver)
        q0, _ = self.ops.project(self.ops.pack(self.u, self.v), 1.0)
        self.u, self.v = self.ops.unpack(q0)
        self.time = 0.0
        self.prev_adv = self.prev_dt = self.half_pressure = None
        self.last_step_diagnostics = {}

    def advance(self, dt):
        """solver/optimized_ghost_cell.py:236-278."""
        ops = self.ops
        ops.pressure_calls.clear()
        ops.set_inlet(self.u_inlet)
        pressure = self.p.ravel()[ops.pi] if self.half_pressure is None else self.half_pressure
        q = ops.pack(self.u, self.v)
        q, half, out_p, hist, diag = ab2_cn_step(ops, q, pressure, dt, self.prev_adv, self.prev_dt)
        self.half_pressure, self.prev_adv, self.prev_dt = half, hist, dt
        calls = ops.pressure_calls
        diag.update(pressure_backend=ops.pressure_info['backend'], pressure_solve_count=len(calls),
                    pressure_iterations=sum(c['iterations'] for c in calls),
                    pressure_refinement_iterations=sum(c['refinement_iterations'] for c in calls),
                    pressure_residual_linf=max(c['residual_linf'] for c in calls),
                    pressure_residual_relative_l2=max(c['residual_relative_l2'] for c in calls))
        self.u, self.v = ops.unpack(q)
        self.p = (ops.P @ out_p).reshape(self.p.shape)
        return diag

    def solve(self, n_steps, dt, perturb_transient=False, perturb_duration=None, perturb_amp=0.15,
              step_callback=None):
        """Step loop with CFL screen, inlet perturbation, forces and gates (solver/main.py:245-429)."""
        if perturb_duration is None:
            perturb_duration = 2.5 * (self.D / self.U_ref)
        start = self.time
        cd, cl, ts = [], [], []
        for s in range(n_steps):
            now_t = start + (s + 1) * dt
            if s % 100 == 0:
                rate = np.max(np.abs(self.u)) / self.dx + np.max(np.abs(self.v)) / self.dy
                if not np.isfinite(rate) or dt * rate > 0.5:
                    raise RuntimeError(f'Explicit timestep unsafe at t={self.time:g}')
            if perturb_transient and self.inflow == 'uniform' and now_t <= perturb_duration:
                decay = 1.0 - now_t / perturb_duration
                pert = perturb_amp * np.sin(2.0 * np.pi * self.y_centers / self.Ly) * decay
                self.u_inlet[:] = self.u_inlet_base * (1.0 + pert)
            else:
                self.u_inlet[:] = self.u_inlet_base
            diag = self.advance(dt)
            fx, fy, fxp, fyp, fxv, fyv = self.ops.surface_forces(self.u, self.v, self.p, self.nu * self.rho)
            denom = 0.5 * self.rho * self.U_ref ** 2 * self.D
            Cd, Cl = fx / denom, fy / denom
            if not np.isfinite(Cd) or not np.isfinite(Cl):
                raise FloatingPointError(f'Non-finite force at t={now_t:g}')
            self.time = now_t
            div = float(np.max(abs(self.ops.divergence(self.ops.pack(self.u, self.v)))))
            self.last_step_diagnostics = dict(diag, time=self.time, dt=dt, max_divergence=div,
                                              cfl=float(dt * (np.max(abs(self.u)) / self.dx + np.max(abs(self.v)) / self.dy)),
                                              cd=float(Cd), cl=float(Cl), cd_pressure=float(fxp / denom),
                                              cd_viscous=float(fxv / denom), cl_pressure=float(fyp / denom),
                                              cl_viscous=float(fyv / denom))
            if div >= 1e-10 or self.last_step_diagnostics['cfl'] >= 0.5:
                raise RuntimeError('Ghost step failed divergence/CFL gate')
            if step_callback is not None:
                step_callback(self, dict(self.last_step_diagnostics))
            cd.append(Cd)
            cl.append(Cl)
            ts.append(now_t)
        return np.array(ts), np.array(cd), np.array(cl)


def mac_divergence_stats(u, v, dx, dy, mask):
    """Fluid-cell divergence statistics (solver/src/bindings.cpp:343-390):
    (max |div|, sum div^2, count, core sum div^2, core count)."""
    div = (u[:, 1:] - u[:, :-1]) / dx + (v[1:] - v[:-1]) / dy
    fluid = ~mask
    core = fluid.copy()
    core[:, 1:] &= ~mask[:, :-1]
    core[:, :-1] &= ~mask[:, 1:]
    core[1:] &= ~mask[:-1]
    core[:-1] &= ~mask[1:]
    d = div[fluid]
    return (float(np.max(abs(d))) if d.size else 0.0, float(np.sum(d * d)), int(d.size),
            float(np.sum(div[core] ** 2)), int(core.sum()))


# ---------------------------------------------------------------------------
# periodic Taylor-Green verification  (verification/taylor_green.py:14-59)
# ---------------------------------------------------------------------------
class PeriodicOperators:
    """Operators of the periodic staggered Taylor-Green case on [0, 2 pi]^2.

    u[j, i] sits at (i h, (j + 1/2) h), v[j, i] at ((i + 1/2) h, j h), p at cell centres.
    advection / diffusion follow periodic_momentum_operator (solver/cut_cell_solver.py:108-130):
    the full-fluid flux form of compute_momentum_rhs (:790-957, centred transport, rho = 1)
    with a periodic halo, i.e. the face and corner fluxes below with wrapped indices, divided
    by the cell volume h^2.  gradient / divergence / project are verification/taylor_green.py:37-45;
    the CN Helmholtz system I - dt/2 nu L is solved exactly in Fourier space (the reference
    runs GMRES to rtol 1e-12 on the same operator, solver/time_integration.py:97-99).
    """

    def __init__(self, n, nu):
        self.n, self.nu = n, nu
        self.h = 2 * np.pi / n
        self.diff_offset = 0.0
        self.helmholtz_dt = None
        k = np.arange(n)
        s2 = np.sin(np.pi * k / n) ** 2
        self.symbol = -4 * (s2[:, None] + s2[None, :]) / self.h ** 2   # 5-point Laplacian symbol
        eig = self.symbol.copy()
        eig[0, 0] = 1.0
        self.eigenvalues = eig

    def unpack(self, q):
        return q.reshape(2, self.n, self.n)

    @staticmethod
    def pack(u, v):
        return np.r_[u.ravel(), v.ravel()]

    def _flux(self, q, nu, include_advection):
        u, v = self.unpack(q)
        h = self.h
        r = np.roll
        # u equation: east faces (cell centres) and north corners
        uE = 0.5 * (u + r(u, -1, 1))
        Fxx = nu * (r(u, -1, 1) - u) / h * h
        vN = 0.5 * (r(r(v, -1, 0), 1, 1) + r(v, -1, 0))          # v at the north corner of u[j, i]
        uN = 0.5 * (u + r(u, -1, 0))
        Fxy = nu * (r(u, -1, 0) - u) / h * h                        # flux through the north corner face
        if include_advection:
            Fxx = Fxx - uE * uE * h
            Fxy = Fxy - vN * uN * h
        au = ((Fxx - r(Fxx, 1, 1)) + (Fxy - r(Fxy, 1, 0))) / (h * h)
        # v equation: north faces (cell centres) and east corners
        vC = 0.5 * (v + r(v, -1, 0))
        Fyy = nu * (r(v, -1, 0) - v) / h * h
        uE2 = 0.5 * (r(r(u, -1, 1), 1, 0) + r(u, -1, 1))          # u at the east corner of v[j, i]
        vE = 0.5 * (v + r(v, -1, 1))
        Fyx = nu * (r(v, -1, 1) - v) / h * h
        if include_advection:
            Fyy = Fyy - vC * vC * h
            Fyx = Fyx - uE2 * vE * h
        av = ((Fyx - r(Fyx, 1, 1)) + (Fyy - r(Fyy, 1, 0))) / (h * h)
        return self.pack(au, av)

    def advection(self, q):
        return self._flux(q, 0.0, True)

    def diffusion(self, q):
        return self._flux(q, self.nu, False)

    def gradient(self, p):
        return self.pack(p - np.roll(p, 1, 1), p - np.roll(p, 1, 0)) / self.h

    def divergence(self, q):
        u, v = self.unpack(q)
        return (np.roll(u, -1, 1) - u + np.roll(v, -1, 0) - v) / self.h

    def project(self, q, step):
        from scipy.fft import fft2, ifft2
        rhs = fft2(self.divergence(q) / step)
        rhs[0, 0] = 0.0
        phi = ifft2(rhs / self.eigenvalues).real
        return q - step * self.gradient(phi), phi

    def build_helmholtz(self, dt):
        self.helmholtz_dt = dt

    def helmholtz(self, rhs):
        from scipy.fft import fft2, ifft2
        c = 0.5 * self.helmholtz_dt * self.nu
        u, v = self.unpack(rhs)
        den = 1.0 - c * self.symbol
        return self.pack(ifft2(fft2(u) / den).real, ifft2(fft2(v) / den).real)

    def H_matvec(self, q, dt):
        return q - 0.5 * dt * self.diffusion(q)


def taylor_green_exact(n, nu, t):
    """Analytic Taylor-Green fields on the staggered grid (verification/taylor_green.py:21-29)."""
    h = 2 * np.pi / n
    yu, xu = np.meshgrid((np.arange(n) + .5) * h, np.arange(n) * h, indexing='ij')
    yv, xv = np.meshgrid(np.arange(n) * h, (np.arange(n) + .5) * h, indexing='ij')
    yp, xp = np.meshgrid((np.arange(n) + .5) * h, (np.arange(n) + .5) * h, indexing='ij')
    a = np.exp(-2 * nu * t)
    q = PeriodicOperators.pack(a * np.sin(xu) * np.cos(yu), -a * np.cos(xv) * np.sin(yv))
    return q, .25 * a * a * (np.cos(2 * xp) + np.cos(2 * yp))


def taylor_green_run(n, dt, end_time=.4, nu=.1):
    """verification/taylor_green.py:14-59: AB2/CN steps from the analytic field, error norms
    against the analytic solution at end_time, maximum divergence."""
    if n < 8 or not np.isfinite([dt, end_time, nu]).all() or min(dt, end_time, nu) <= 0:
        raise ValueError('Require n>=8 and finite positive dt, end_time and nu')
    steps = round(end_time / dt)
    if steps < 1 or not np.isclose(steps * dt, end_time):
        raise ValueError('end_time must be an integer multiple of dt')
    ops = PeriodicOperators(n, nu)
    q, p = taylor_green_exact(n, nu, 0.0)
    history = previous_dt = None
    output = p
    max_divergence = 0.0
    for _ in range(steps):
        q, p, output, history, _ = ab2_cn_step(ops, q, p, dt, history, previous_dt)
        previous_dt = dt
        max_divergence = max(max_divergence, float(np.max(abs(ops.divergence(q)))))
    q_exact, p_exact = taylor_green_exact(n, nu, end_time)
    p_error = output - output.mean() - p_exact
    norms = lambda a: dict(l1=float(np.mean(abs(a))), l2=float(np.sqrt(np.mean(a * a))), linf=float(np.max(abs(a))))
    return dict(n=n, dt=dt, end_time=end_time, velocity=norms(q - q_exact), pressure=norms(p_error),
                max_divergence=max_divergence), q, output - output.mean()
