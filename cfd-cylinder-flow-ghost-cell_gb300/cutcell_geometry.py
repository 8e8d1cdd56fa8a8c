"""Host-side setup of the cut-cell (embedded-boundary) cylinder case.

Everything the GPU cut-cell step needs that depends only on the geometry is computed here,
once, on the host: the open fractions of the MAC faces and of the staggered momentum
control-volume faces, the fluid fractions of the pressure cells and of the u / v control
volumes (by adaptive quadrature of the solid chord), the small-cell merge tables, the owned
volumes with their covered-donor -> owner maps, the local streamfunction fits behind the
wall-shear stencil and the curved-face flux stencils, and the smooth ring correction of the
viscous face fluxes.  The results are plain numpy arrays and scipy CSR matrices over the
concatenated field [u.ravel(), v.ravel()]; cutcell.py hands them to libghostmac.so.

The arithmetic follows the reference's setup expression by expression where a result feeds
a classification (open-fraction snapping, the 0.3 merge threshold, covered / cut / fluid),
so that every such decision is taken on the same IEEE values:
  solver/cut_cell_geom.py:22-525        fractions, volumes, merge tables
  solver/staggered_wall.py:12-300       derivative bases, face stencils, ring correction,
                                        wall stencil, owned volumes
  solver/wall_reconstruction.py:25-135  open-face segments, local bases, streamfunction fit
"""
from __future__ import annotations

import math
from types import SimpleNamespace

import numpy as np
from scipy.integrate import quad
from scipy.sparse import csr_matrix, vstack

MERGE_THRESHOLD = 0.3
_EPS = np.finfo(float).eps


def _snap(val):
    """Open fractions within 1e-12 of 0 or 1 are exactly 0 or 1."""
    return np.where(val < 1e-12, 0.0, np.where(val > 1.0 - 1e-12, 1.0, val))


def _line_fraction(line_pos, c_line, c_span, R, lo, hi, length, always=False):
    """Open fraction of grid-line segments [lo, hi] at positions line_pos (one row per line,
    broadcast against the segments) cut by the circle's chord: 1 - overlap / length, snapped.
    With always=False a segment without overlap keeps 1 (the fraction is only assigned where
    the chord overlaps), which gives the same values."""
    d = np.abs(line_pos - c_line)
    inside = d < R
    half = np.sqrt(np.where(inside, R**2 - np.where(inside, d, 0.0)**2, 0.0))
    s1, s2 = c_span - half, c_span + half
    inter = np.minimum(hi, s2) - np.maximum(lo, s1)
    if always:
        frac = _snap(1.0 - np.maximum(0.0, inter) / length)
        return np.where(inside, frac, 1.0)
    frac = _snap(1.0 - inter / length)
    return np.where(inside & (inter > 0), frac, 1.0)


class CutCellGeometry:
    """Fractions, volumes and merge tables of a circle on a uniform MAC grid
    (solver/cut_cell_geom.py:22-61): ax (ny, nx+1), ay (ny+1, nx), volume_fraction and
    cell_type (1 fluid, 0 cut, -1 covered) on (ny, nx), u_volume_fraction (ny, nx+1),
    v_volume_fraction (ny+1, nx), ax_mid / ay_mid (ny, nx), ay_u / ax_v (ny+1, nx+1), and the
    merge lists of small staggered volumes."""

    def __init__(self, nx, ny, Lx, Ly, xc, yc, R):
        if nx < 4 or ny < 4:
            raise ValueError("nx and ny must be >= 4")
        if Lx <= 0 or Ly <= 0 or R <= 0:
            raise ValueError("Domain dimensions and radius must be positive")
        if not (R < xc < Lx - R and R < yc < Ly - R):
            raise ValueError("Cylinder must be located strictly inside the domain boundaries")
        self.nx, self.ny = int(nx), int(ny)
        self.Lx, self.Ly, self.xc, self.yc, self.R = float(Lx), float(Ly), float(xc), float(yc), float(R)
        self.dx = self.Lx / self.nx
        self.dy = self.Ly / self.ny
        self.cell_area = self.dx * self.dy
        self._face_fractions()
        self._cell_fractions()
        self._staggered_fractions()
        self._staggered_faces()
        self._merge_tables()

    # -- faces of the MAC grid (solver/cut_cell_geom.py:63-105) --------------------------------
    def _face_fractions(self):
        nx, ny, dx, dy = self.nx, self.ny, self.dx, self.dy
        xs = (np.arange(nx + 1) * dx)[None, :]
        yb = (np.arange(ny) * dy)[:, None]
        self.ax = _line_fraction(xs, self.xc, self.yc, self.R, yb, (np.arange(ny)[:, None] + 1) * dy, dy)
        ys = (np.arange(ny + 1) * dy)[:, None]
        xl = (np.arange(nx) * dx)[None, :]
        self.ay = _line_fraction(ys, self.yc, self.xc, self.R, xl, (np.arange(nx)[None, :] + 1) * dx, dx)

    # -- solid area of a box by quadrature of the chord height ---------------------------------
    def _solid_area(self, xl, xr, yb, yt):
        xc, yc, R = self.xc, self.yc, self.R

        def height(x):
            off = abs(x - xc)
            if off >= R:
                return 0.0
            half = np.sqrt(R**2 - off**2)
            return max(0.0, min(yt, yc + half) - max(yb, yc - half))

        breaks = [xe for xe in (xc - R, xc + R) if xl < xe < xr]
        for yh in (yb, yt):
            if abs(yh - yc) < R:
                ch = np.sqrt(R**2 - (yh - yc)**2)
                breaks.extend(xe for xe in (xc - ch, xc + ch) if xl < xe < xr)
        area, _ = quad(height, xl, xr, points=breaks, epsabs=1e-12, epsrel=1e-10)
        return area

    def _box_class(self, xl, xr, yb, yt):
        """Boolean arrays (fluid, covered) of boxes by the nearest-point and corner tests."""
        xc, yc, R = self.xc, self.yc, self.R
        cx, cy = np.clip(xc, xl, xr), np.clip(yc, yb, yt)
        fluid = (cx - xc)**2 + (cy - yc)**2 >= R**2 - 1e-13
        covered = np.ones(np.broadcast(xl, yb).shape, bool)
        for x in (xl, xr):
            for y in (yb, yt):
                covered &= (x - xc)**2 + (y - yc)**2 <= R**2 + 1e-12
        return fluid, covered & ~fluid

    # -- pressure cells (solver/cut_cell_geom.py:107-208; centroids are not needed) ------------
    def _cell_fractions(self):
        nx, ny, dx, dy = self.nx, self.ny, self.dx, self.dy
        xl = (np.arange(nx) * dx)[None, :]
        xr = ((np.arange(nx) + 1) * dx)[None, :]
        yb = (np.arange(ny) * dy)[:, None]
        yt = ((np.arange(ny) + 1) * dy)[:, None]
        fluid, covered = self._box_class(xl, xr, yb, yt)
        kappa = np.ones((ny, nx))
        kind = np.ones((ny, nx), dtype=np.int32)
        kappa[covered] = 0.0
        kind[covered] = -1
        area = self.cell_area
        for j, i in zip(*np.nonzero(~fluid & ~covered)):
            solid = self._solid_area(i * dx, (i + 1) * dx, j * dy, (j + 1) * dy)
            if solid >= area - 1e-12:
                kappa[j, i], kind[j, i] = 0.0, -1
            elif solid <= 1e-12:
                kappa[j, i], kind[j, i] = 1.0, 1
            else:
                kappa[j, i] = max(0.0, min(area, area - solid)) / area
                kind[j, i] = 0
        self.volume_fraction, self.cell_type = kappa, kind

    # -- staggered control volumes (solver/cut_cell_geom.py:293-393) ---------------------------
    def _staggered_fractions(self):
        nx, ny, dx, dy, Lx, Ly = self.nx, self.ny, self.dx, self.dy, self.Lx, self.Ly
        # u volumes [x_{i-1/2}, x_{i+1/2}] x [y_j, y_{j+1}], clipped to the channel
        frac_u = np.ones((ny, nx + 1))
        xl = np.array([max(0.0, (i - 0.5) * dx) for i in range(nx + 1)])[None, :]
        xr = np.array([min(Lx, (i + 0.5) * dx) for i in range(nx + 1)])[None, :]
        yb = (np.arange(ny) * dy)[:, None]
        yt = ((np.arange(ny) + 1) * dy)[:, None]
        fluid, covered = self._box_class(xl, xr, yb, yt)
        frac_u[covered] = 0.0
        for j, i in zip(*np.nonzero(~fluid & ~covered)):
            a, b = float(xl[0, i]), float(xr[0, i])
            box = (b - a) * dy
            if box <= 0:
                continue
            solid = self._solid_area(a, b, j * dy, (j + 1) * dy)
            frac_u[j, i] = max(0.0, min(1.0, 1.0 - solid / box))
        # v volumes [x_i, x_{i+1}] x [y_{j-1/2}, y_{j+1/2}]
        frac_v = np.ones((ny + 1, nx))
        xl = (np.arange(nx) * dx)[None, :]
        xr = ((np.arange(nx) + 1) * dx)[None, :]
        yb = np.array([max(0.0, (j - 0.5) * dy) for j in range(ny + 1)])[:, None]
        yt = np.array([min(Ly, (j + 0.5) * dy) for j in range(ny + 1)])[:, None]
        fluid, covered = self._box_class(xl, xr, yb, yt)
        frac_v[covered] = 0.0
        for j, i in zip(*np.nonzero(~fluid & ~covered)):
            a, b = float(yb[j, 0]), float(yt[j, 0])
            box = dx * (b - a)
            if box <= 0:
                continue
            solid = self._solid_area(i * dx, (i + 1) * dx, a, b)
            frac_v[j, i] = max(0.0, min(1.0, 1.0 - solid / box))
        self.u_volume_fraction, self.v_volume_fraction = frac_u, frac_v

    # -- faces of the staggered volumes (solver/cut_cell_geom.py:395-465) ----------------------
    def _staggered_faces(self):
        nx, ny, dx, dy, Lx, Ly = self.nx, self.ny, self.dx, self.dy, self.Lx, self.Ly
        xc, yc, R = self.xc, self.yc, self.R
        jj, ii = np.arange(ny)[:, None], np.arange(nx)[None, :]
        self.ax_mid = _line_fraction((ii + 0.5) * dx, xc, yc, R, jj * dy, (jj + 1) * dy, dy, always=True)
        self.ay_mid = _line_fraction((jj + 0.5) * dy, yc, xc, R, ii * dx, (ii + 1) * dx, dx, always=True)
        # ay_u: horizontal lines y_j over [x_{i-1/2}, x_{i+1/2}] clipped; ax_v the transpose case
        jj, ii = np.arange(ny + 1)[:, None], np.arange(nx + 1)[None, :]
        lo = np.maximum(0.0, (ii - 0.5) * dx)
        hi = np.minimum(Lx, (ii + 0.5) * dx)
        self.ay_u = _line_fraction(jj * dy, yc, xc, R, lo, hi, hi - lo, always=True)
        lo = np.maximum(0.0, (jj - 0.5) * dy)
        hi = np.minimum(Ly, (jj + 0.5) * dy)
        self.ax_v = _line_fraction(ii * dx, xc, yc, R, lo, hi, hi - lo, always=True)

    # -- merge tables (solver/cut_cell_geom.py:467-525) ----------------------------------------
    def _merge_walk(self, fraction, j, i, x, y, jmax):
        rx, ry = x - self.xc, y - self.yc
        r = np.hypot(rx, ry)
        unx = rx / r if r > 0 else 1.0
        uny = ry / r if r > 0 else 0.0
        if abs(unx) >= abs(uny):
            dj, di = 0, (1 if unx > 0 else -1)
        else:
            dj, di = (1 if uny > 0 else -1), 0
        tj, ti = j + dj, i + di
        while 0 <= tj <= jmax and 0 <= ti < self.nx and fraction[tj, ti] < MERGE_THRESHOLD:
            tj, ti = tj + dj, ti + di
        if 0 <= tj <= jmax and 0 <= ti < self.nx:
            return (tj, ti)
        return None

    def _merge_tables(self):
        self.u_merge_list, self.v_merge_list = [], []
        small_u = (self.ax > 0.0) & (self.u_volume_fraction > 0.0) & (self.u_volume_fraction < MERGE_THRESHOLD)
        small_u[:, 0] = small_u[:, self.nx] = False
        for j, i in zip(*np.nonzero(small_u)):
            m = self._merge_walk(self.u_volume_fraction, j, i, i * self.dx, (j + 0.5) * self.dy, self.ny - 1)
            if m is not None:
                self.u_merge_list.append(((int(j), int(i)), (int(m[0]), int(m[1]))))
        small_v = (self.ay > 0.0) & (self.v_volume_fraction > 0.0) & (self.v_volume_fraction < MERGE_THRESHOLD)
        small_v[0, :] = small_v[self.ny, :] = False
        for j, i in zip(*np.nonzero(small_v)):
            m = self._merge_walk(self.v_volume_fraction, j, i, (i + 0.5) * self.dx, j * self.dy, self.ny)
            if m is not None:
                self.v_merge_list.append(((int(j), int(i)), (int(m[0]), int(m[1]))))


# ---------------------------------------------------------------------------------------------
# local polynomial bases and the streamfunction fit (solver/wall_reconstruction.py:25-135)
# ---------------------------------------------------------------------------------------------
def open_segments(lo, hi, coordinate, normal_center, tangent_center, radius):
    """The parts of the grid-line segment [lo, hi] (at `coordinate` across the line) outside
    the circle, as (a, b) pairs longer than 1e-14."""
    offset = coordinate - normal_center
    if abs(offset) >= radius:
        return [(lo, hi)]
    half = np.sqrt(max(0., radius**2 - offset**2))
    out = []
    for a, b in ((lo, min(hi, tangent_center - half)), (max(lo, tangent_center + half), hi)):
        if b - a > 1e-14:
            out.append((a, b))
    return out


def _local_basis(x, y, g, angle, h, cartesian):
    """The six streamfunction basis values psi_k at one point for the fit around `angle`."""
    xx, yy = x - g.xc, y - g.yc
    if cartesian:
        q = (xx - g.R * np.cos(angle)) / h
        z = (yy - g.R * np.sin(angle)) / h
        s = (xx * xx + yy * yy - g.R**2) / (2 * g.R * h)
        return h * s * s * np.array([1., q, z, q * q, q * z, z * z])
    d = (np.hypot(xx, yy) - g.R) / h
    polar = np.arctan2(yy, xx)
    t = g.R * np.arctan2(np.sin(polar - angle), np.cos(polar - angle)) / h
    return h * d**2 * np.array([1., d, t, d**2, d * t, t**2])


def _face_average(g, component, j, i, angle, h, cartesian):
    """Basis average over the open part of velocity face (component, j, i): the difference
    of psi over each open segment (u faces: along y at x_i; v faces: minus along x at y_j),
    divided by the open length; (average, open length, centroid coordinate)."""
    if component == 'u':
        x = i * g.dx
        spans = open_segments(j * g.dy, (j + 1) * g.dy, x, g.xc, g.yc, g.R)
        total = np.zeros(6)
        for a, b in spans:
            total = total + (_local_basis(x, b, g, angle, h, cartesian) - _local_basis(x, a, g, angle, h, cartesian))
    else:
        y = j * g.dy
        spans = open_segments(i * g.dx, (i + 1) * g.dx, y, g.yc, g.xc, g.R)
        total = np.zeros(6)
        for a, b in spans:
            total = total + (_local_basis(b, y, g, angle, h, cartesian) - _local_basis(a, y, g, angle, h, cartesian))
        total = -total
    length = sum(b - a for a, b in spans)
    centre = sum((a + b) / 2 * (b - a) for a, b in spans) / length if length else 0.0
    return total, length, centre


def streamfunction_fit(g, angles, cartesian=False):
    """Six local streamfunction coefficients per wall angle as a CSR over the concatenated
    face field: weighted minimum-norm least squares against the open-face averages within
    3, 4 or 5 h of the wall point (the first width with full rank).  Rows 6 k .. 6 k + 5 are
    the coefficients of angle k (solver/wall_reconstruction.py:70-129)."""
    angles = np.asarray(angles, dtype=float)
    if angles.ndim != 1 or not np.isfinite(angles).all():
        raise ValueError('Wall angles must be a finite one-dimensional array')
    h = max(g.dx, g.dy)
    u_size = g.ny * (g.nx + 1)
    rows, cols, vals = [], [], []
    slack = 64 * _EPS * max(g.Lx, g.Ly) / h
    for row, angle in enumerate(angles):
        xw, yw = g.xc + g.R * np.cos(angle), g.yc + g.R * np.sin(angle)
        for width in (3., 4., 5.):
            design, idx, wts = [], [], []
            for comp in ('u', 'v'):
                nxc, nyc = (g.nx + 1, g.ny) if comp == 'u' else (g.nx, g.ny + 1)
                aperture = g.ax if comp == 'u' else g.ay
                for j in range(max(0, int((yw - width * h) / g.dy) - 1), min(nyc, int((yw + width * h) / g.dy) + 2)):
                    for i in range(max(0, int((xw - width * h) / g.dx) - 1),
                                   min(nxc, int((xw + width * h) / g.dx) + 2)):
                        if aperture[j, i] <= 0:
                            continue
                        avg, length, centre = _face_average(g, comp, j, i, angle, h, cartesian)
                        if not length:
                            continue
                        if comp == 'u':
                            x, y, flat = i * g.dx, centre, j * (g.nx + 1) + i
                        else:
                            x, y, flat = centre, j * g.dy, u_size + j * g.nx + i
                        dist = np.hypot(x - xw, y - yw) / h
                        if dist > width + slack:
                            continue
                        design.append(avg / length)
                        idx.append(flat)
                        wts.append(1 / (1 + dist**2))
            if len(design) < 6:
                continue
            weighted = np.asarray(design) * np.asarray(wts)[:, None]
            if np.linalg.matrix_rank(weighted, tol=1e-11) == 6:
                coef = np.linalg.pinv(weighted, rcond=1e-12) * wts
                for k in range(6):
                    rows.extend([6 * row + k] * len(idx))
                    cols.extend(idx)
                    vals.extend(coef[k])
                break
        else:
            raise ValueError('Insufficient independent open faces for wall reconstruction')
    return csr_matrix((vals, (rows, cols)), shape=(6 * len(angles), u_size + (g.ny + 1) * g.nx))


def _cartesian_derivatives(x, y, g, angles):
    """Velocity and velocity-gradient bases of the Cartesian streamfunction family at points
    (x, y) for the fits around `angles` (solver/wall_reconstruction.py:34-53)."""
    h = max(g.dx, g.dy)
    xx, yy = np.asarray(x) - g.xc, np.asarray(y) - g.yc
    q = (xx - g.R * np.cos(angles)) / h
    z = (yy - g.R * np.sin(angles)) / h
    s = (xx * xx + yy * yy - g.R**2) / (2 * g.R * h)
    sx, sy = xx / (g.R * h), yy / (g.R * h)
    one, zero = np.ones_like(q), np.zeros_like(q)
    poly = np.stack((one, q, z, q * q, q * z, z * z), axis=-1)
    px = np.stack((zero, one, zero, 2 * q, z, zero), axis=-1) / h
    py = np.stack((zero, zero, one, zero, q, 2 * z), axis=-1) / h
    pxx = np.array([0, 0, 0, 2, 0, 0]) / h**2
    pxy = np.array([0, 0, 0, 0, 1, 0]) / h**2
    pyy = np.array([0, 0, 0, 0, 0, 2]) / h**2
    s, sx, sy = s[..., None], sx[..., None], sy[..., None]
    dxx = h * (2 * (sx * sx + s / (g.R * h)) * poly + 4 * s * sx * px + s * s * pxx)
    dxy = h * (2 * sx * sy * poly + 2 * s * sx * py + 2 * s * sy * px + s * s * pxy)
    dyy = h * (2 * (sy * sy + s / (g.R * h)) * poly + 4 * s * sy * py + s * s * pyy)
    return dict(u=h * (2 * s * sy * poly + s * s * py), v=-h * (2 * s * sx * poly + s * s * px),
                ux=dxy, uy=dyy, vx=-dxx, vy=-dxy)


def derivative_basis(x, y, angles, g, cartesian=False):
    """Velocity, velocity-gradient and wall-rate bases at points (x, y) for the fits around
    `angles` (one angle per point; solver/staggered_wall.py:12-36)."""
    if cartesian:
        return _cartesian_derivatives(x, y, g, angles)
    h = max(g.dx, g.dy)
    xx, yy = np.asarray(x) - g.xc, np.asarray(y) - g.yc
    r = np.hypot(xx, yy)
    theta = np.arctan2(yy, xx)
    d = ((r - g.R) / h)[:, None]
    s = (g.R / h * np.arctan2(np.sin(theta - angles), np.cos(theta - angles)))[:, None]
    a, b = np.array([2, 3, 2, 4, 3, 2]), np.array([0, 0, 1, 0, 1, 2])
    radial = a * d**(a - 1) * s**b
    angular = g.R * b * d**a * s**np.maximum(b - 1, 0)
    rr = a * (a - 1) / h * d**(a - 2) * s**b
    rt = g.R / h * a * b * d**(a - 1) * s**np.maximum(b - 1, 0)
    tt = g.R**2 / h * b * (b - 1) * d**a * s**np.maximum(b - 2, 0)
    nx, ny = (xx / r)[:, None], (yy / r)[:, None]
    tx, ty = -ny, nx
    transverse = radial / r[:, None] + tt / r[:, None]**2
    cross = rt / r[:, None] - angular / r[:, None]**2
    ux = rr * nx * ny + transverse * tx * ty + cross * (nx * ty + tx * ny)
    uy = rr * ny**2 + transverse * ty**2 + 2 * cross * ny * ty
    vx = -(rr * nx**2 + transverse * tx**2 + 2 * cross * nx * tx)
    return dict(u=radial * ny + angular * ty / r[:, None], v=-radial * nx - angular * tx / r[:, None],
                ux=ux, uy=uy, vx=vx, vy=-ux, wall_rate=-rr)


def point_operator(fit, patch, basis):
    """Rows = points: basis (points x 6) applied to the six coefficients of each point's fit."""
    count = len(patch)
    gather = csr_matrix((basis.ravel(), (np.repeat(np.arange(count), 6),
                                         (6 * np.asarray(patch)[:, None] + np.arange(6)).ravel())),
                        shape=(count, fit.shape[0]))
    return gather @ fit


# ---------------------------------------------------------------------------------------------
# face stencils of the curved momentum fluxes (solver/staggered_wall.py:46-131)
# ---------------------------------------------------------------------------------------------
FACE_APERTURE = {('u', 'x'): 'ax_mid', ('u', 'y'): 'ay_u', ('v', 'x'): 'ax_v', ('v', 'y'): 'ay_mid'}


def _face_ends(component, axis, j, i):
    """(low, high) velocity faces whose difference a flux face carries."""
    centered = (component, axis) in (('u', 'x'), ('v', 'y'))
    if centered:
        return (j, i), ((j, i + 1) if axis == 'x' else (j + 1, i))
    return ((j - 1, i) if axis == 'y' else (j, i - 1)), (j, i)


def face_stencil(g, component, axis, reach=2., cartesian=False):
    """Flux faces of family (component, axis) within R + reach h of the centre: velocity
    values at three Gauss points per open interval (CSR u, v over the field), the open-face
    average of the viscous gradient plus the two-point diffusion of the fit residual
    (CSR gradient), the flux-face flat indices, the point -> face map and the Gauss weights."""
    aperture = getattr(g, FACE_APERTURE[component, axis])
    centered = (component, axis) in (('u', 'x'), ('v', 'y'))
    offset = .5 if centered else 0.
    h = max(g.dx, g.dy)
    nodes, weights = np.polynomial.legendre.leggauss(3)
    faces, angles, points, lengths, patch = [], [], [], [], []
    tol = 64 * _EPS * max(g.Lx, g.Ly)
    for j in range(max(0, int((g.yc - g.R - reach * h) / g.dy) - 1),
                   min(aperture.shape[0], int((g.yc + g.R + reach * h) / g.dy) + 2)):
        for i in range(max(0, int((g.xc - g.R - reach * h) / g.dx) - 1),
                       min(aperture.shape[1], int((g.xc + g.R + reach * h) / g.dx) + 2)):
            if not centered and ((axis == 'x' and i in (0, g.nx)) or (axis == 'y' and j in (0, g.ny))):
                continue  # outer-boundary faces carry their own boundary flux
            x, y = (i + offset) * g.dx, (j + offset) * g.dy
            if aperture[j, i] <= 0 or np.hypot(x - g.xc, y - g.yc) > g.R + reach * h + tol:
                continue
            if axis == 'x':
                lo, hi = (j * g.dy, (j + 1) * g.dy) if centered else (max(0., (j - .5) * g.dy),
                                                                     min(g.Ly, (j + .5) * g.dy))
                spans = open_segments(lo, hi, x, g.xc, g.yc, g.R)
            else:
                lo, hi = (i * g.dx, (i + 1) * g.dx) if centered else (max(0., (i - .5) * g.dx),
                                                                     min(g.Lx, (i + .5) * g.dx))
                spans = open_segments(lo, hi, y, g.yc, g.xc, g.R)
            if not spans:
                continue
            k = len(faces)
            faces.append(j * aperture.shape[1] + i)
            angles.append(np.arctan2(y - g.yc, x - g.xc))
            for a, b in spans:
                coord = (a + b) / 2 + (b - a) / 2 * nodes
                points.extend([(x, t) if axis == 'x' else (t, y) for t in coord])
                lengths.extend((b - a) / 2 * weights)
                patch.extend([k] * len(nodes))
    fit = streamfunction_fit(g, angles, cartesian)
    patch = np.asarray(patch, dtype=int)
    xy = np.asarray(points).reshape(-1, 2)
    basis = derivative_basis(xy[:, 0], xy[:, 1], np.asarray(angles)[patch], g, cartesian)
    average = csr_matrix((lengths, (patch, np.arange(len(patch)))), shape=(len(faces), len(patch)))
    # two-point diffusion of the part of the face values the fit does not reproduce
    link_rows, link_cols, link_vals, residual_basis = [], [], [], []
    vshape = g.ax.shape if component == 'u' else g.ay.shape
    voff = 0 if component == 'u' else g.ax.size
    spacing = g.dx if axis == 'x' else g.dy
    vel_aperture = g.ax if component == 'u' else g.ay
    for k, face in enumerate(faces):
        j, i = np.unravel_index(face, aperture.shape)
        low, high = _face_ends(component, axis, j, i)
        scale = aperture[j, i] * (g.dy if axis == 'x' else g.dx) / spacing
        avg_hi = _face_average(g, component, *high, angles[k], h, cartesian)
        avg_lo = _face_average(g, component, *low, angles[k], h, cartesian)
        hi_v = avg_hi[0] / avg_hi[1] if avg_hi[1] > 0 else np.zeros(6)
        lo_v = avg_lo[0] / avg_lo[1] if avg_lo[1] > 0 else np.zeros(6)
        residual_basis.append(scale * (hi_v - lo_v))
        for pos, sign in ((low, -1), (high, 1)):
            if vel_aperture[pos] == 0:
                continue  # covered velocity faces are not unknowns
            link_rows.append(k)
            link_cols.append(voff + np.ravel_multi_index(pos, vshape))
            link_vals.append(sign * scale)
    links = csr_matrix((link_vals, (link_rows, link_cols)), shape=(len(faces), fit.shape[1]))
    residual = links - point_operator(fit, np.arange(len(faces)), np.asarray(residual_basis).reshape(-1, 6))
    return SimpleNamespace(indices=np.asarray(faces, dtype=int),
                           u=point_operator(fit, patch, basis['u']), v=point_operator(fit, patch, basis['v']),
                           gradient=average @ point_operator(fit, patch, basis[component + axis]) + residual,
                           patch=patch, lengths=np.asarray(lengths))


def ring_correction(g, component, axis, near):
    """Fourth-order smooth correction of the ordinary two-point viscous flux on full faces of
    a ring around the cylinder (weight 1 inside R + max(3h, R/2), blended to 0 over R/2 and
    away from the channel walls); faces of `near` are excluded
    (solver/staggered_wall.py:143-200).  Returns (indices, base + correction, correction)."""
    aperture = getattr(g, FACE_APERTURE[component, axis])
    vel_aperture = g.ax if component == 'u' else g.ay
    centered = (component, axis) in (('u', 'x'), ('v', 'y'))
    normal = g.dx if axis == 'x' else g.dy
    length = g.dy if axis == 'x' else g.dx
    voff = 0 if component == 'u' else g.ax.size
    excluded = set(int(f) for f in near.indices)
    h = max(g.dx, g.dy)
    inner, width = max(3 * h, .5 * g.R), .5 * g.R
    rows, cols, vals, faces = [], [], [], []
    for j in range(max(0, int((g.yc - g.R - inner - width) / g.dy) - 1),
                   min(aperture.shape[0], int((g.yc + g.R + inner + width) / g.dy) + 2)):
        for i in range(max(0, int((g.xc - g.R - inner - width) / g.dx) - 1),
                       min(aperture.shape[1], int((g.xc + g.R + inner + width) / g.dx) + 2)):
            face = j * aperture.shape[1] + i
            if face in excluded or aperture[j, i] < 1 - 1e-12:
                continue
            x, y = (i + (.5 if centered else 0)) * g.dx, (j + (.5 if centered else 0)) * g.dy
            t = np.clip((np.hypot(x - g.xc, y - g.yc) - g.R - inner) / width, 0., 1.)
            edge = np.clip((min(x, g.Lx - x, y, g.Ly - y) - 2 * h) / width, 0., 1.)
            weight = (1 - t * t * (3 - 2 * t)) * edge * edge * (3 - 2 * edge)
            if weight <= 0:
                continue
            entries = []
            if centered:
                for shift, c in zip((-1, 0, 1, 2), (1, -3, 3, -1)):
                    entries.append(((j, i + shift) if axis == 'x' else (j + shift, i), c / (24 * normal)))
            else:
                for tr, avg in zip((-1, 0, 1), (1 / 24, 22 / 24, 1 / 24)):
                    for shift, c in zip((-2, -1, 0, 1), (1, -15, 15, -1)):
                        pos = (j + shift, i + tr) if axis == 'y' else (j + tr, i + shift)
                        entries.append((pos, avg * c / (12 * normal)))
                low = (j - 1, i) if axis == 'y' else (j, i - 1)
                entries.extend([(low, 1 / normal), ((j, i), -1 / normal)])
            if any(not (0 <= jj < vel_aperture.shape[0] and 0 <= ii < vel_aperture.shape[1])
                   or vel_aperture[jj, ii] < 1 - 1e-12 for (jj, ii), _ in entries):
                continue
            row = len(faces)
            faces.append(face)
            for pos, val in entries:
                rows.append(row)
                cols.append(voff + np.ravel_multi_index(pos, vel_aperture.shape))
                vals.append(weight * length * val)
    nfield = g.ax.size + g.ay.size
    correction = csr_matrix((vals, (rows, cols)), shape=(len(faces), nfield))
    brows, bcols, bvals = [], [], []
    for row, face in enumerate(faces):
        j, i = np.unravel_index(face, aperture.shape)
        low, high = _face_ends(component, axis, j, i)
        for pos, sign in ((low, -1), (high, 1)):
            brows.append(row)
            bcols.append(voff + np.ravel_multi_index(pos, vel_aperture.shape))
            bvals.append(sign * length / normal)
    base = csr_matrix((bvals, (brows, bcols)), shape=correction.shape)
    return np.asarray(faces, dtype=int), base + correction


def diffusion_faces(g, component, axis, original, near):
    """The viscous flux faces of one family with their full gradient rows: the faces of the
    Cartesian reconstruction `near` (its gradient), then the ring faces (two-point flux plus
    the smooth correction).  The GPU overwrites the plain flux of these faces with
    rho nu (gradient @ field) (solver/staggered_wall.py:203-232)."""
    ring_idx, ring_grad = ring_correction(g, component, axis, near)
    indices = np.r_[near.indices, ring_idx]
    gradient = vstack((near.gradient, ring_grad), format='csr')
    return SimpleNamespace(indices=indices, gradient=gradient, original=original)


def wall_stencil(g):
    """Gauss points on the circle between the crossings of the grid and half-grid lines,
    with the wall shear-rate operator (rows = points) of the fit around each arc's midpoint,
    tangents, arc weights and the u / v faces whose control volumes own each point
    (solver/staggered_wall.py:235-261)."""
    cuts = [0., 2 * np.pi]
    for center, spacing, kind in ((g.xc, g.dx, 'x'), (g.yc, g.dy, 'y')):
        for k in range(int(np.floor(2 * (center - g.R) / spacing)), int(np.ceil(2 * (center + g.R) / spacing)) + 1):
            val = (k * spacing / 2 - center) / g.R
            if abs(val) < 1:
                th = np.arccos(val) if kind == 'x' else np.arcsin(val)
                cuts.extend([th % (2 * np.pi), (-th if kind == 'x' else np.pi - th) % (2 * np.pi)])
    cuts = np.unique(cuts)
    nodes, weights = np.polynomial.legendre.leggauss(3)
    angles, theta, ds, patch = [], [], [], []
    for lo, hi in zip(cuts[:-1], cuts[1:]):
        if hi - lo < 1e-12:
            continue
        patch.extend([len(angles)] * 3)
        angles.append((lo + hi) / 2)
        theta.extend((lo + hi) / 2 + (hi - lo) / 2 * nodes)
        ds.extend(g.R * (hi - lo) / 2 * weights)
    theta, patch = np.asarray(theta), np.asarray(patch, dtype=int)
    x, y = g.xc + g.R * np.cos(theta), g.yc + g.R * np.sin(theta)
    fit = streamfunction_fit(g, angles)
    basis = derivative_basis(x, y, np.asarray(angles)[patch], g)
    return SimpleNamespace(rate=point_operator(fit, patch, basis['wall_rate']),
                           tx=-np.sin(theta), ty=np.cos(theta), ds=np.asarray(ds),
                           u_indices=(np.floor(y / g.dy).astype(int) * (g.nx + 1)
                                      + np.floor(x / g.dx + .5).astype(int)),
                           v_indices=(np.floor(y / g.dy + .5).astype(int) * g.nx
                                      + np.floor(x / g.dx).astype(int)))


def owned_volumes(g, component):
    """Physical volumes of the staggered control volumes (half width at the channel ends),
    with each partly fluid volume of a covered face (donor) handed to the first open face
    with fraction >= 0.3 along the dominant direction away from the centre (its owner):
    (volumes, donors, owners) (solver/staggered_wall.py:264-299)."""
    aperture = g.ax if component == 'u' else g.ay
    fraction = g.u_volume_fraction if component == 'u' else g.v_volume_fraction
    volume = fraction.copy() * g.dx * g.dy
    if component == 'u':
        volume[:, [0, -1]] *= .5
    else:
        volume[[0, -1], :] *= .5
    donors = np.flatnonzero((aperture == 0) & (fraction > 0))
    owners = []
    for donor in donors:
        j, i = np.unravel_index(donor, aperture.shape)
        x = (i + (0 if component == 'u' else .5)) * g.dx - g.xc
        y = (j + (.5 if component == 'u' else 0)) * g.dy - g.yc
        sxs, sys_ = abs(x / g.dx), abs(y / g.dy)
        tie = 64 * _EPS * max(1., sxs, sys_)
        sj, si = ((0, 1 if x >= 0 else -1) if sxs >= sys_ - tie else (1 if y >= 0 else -1, 0))
        while True:
            j, i = j + sj, i + si
            if not (0 <= j < aperture.shape[0] and 0 <= i < aperture.shape[1]):
                raise ValueError('Covered momentum volume has no exterior owner')
            if aperture[j, i] > 0 and fraction[j, i] >= .3:
                owners.append(np.ravel_multi_index((j, i), aperture.shape))
                break
    owners = np.asarray(owners, dtype=int)
    np.add.at(volume.ravel(), owners, volume.ravel()[donors])
    volume.ravel()[donors] = 0.
    return volume, donors, owners


class CutCellSetup:
    """All geometry-dependent data of one cut-cell case (the geometric part of
    CutCellBoundary.__init__, solver/cut_cell_solver.py:376-478)."""

    def __init__(self, nx, ny, Lx, Ly, xc, yc, R):
        g = self.geom = CutCellGeometry(nx, ny, Lx, Ly, xc, yc, R)
        self.wall = wall_stencil(g)
        self.momentum_faces = {(c, a): face_stencil(g, c, a) for c in ('u', 'v') for a in ('x', 'y')}
        reach = max(np.hypot(g.dx, 2 * g.dy), np.hypot(2 * g.dx, g.dy)) / max(g.dx, g.dy)
        near = {key: face_stencil(g, *key, reach=reach, cartesian=True) for key in self.momentum_faces}
        self.diffusion_faces = {key: diffusion_faces(g, *key, st, near[key])
                                for key, st in self.momentum_faces.items()}
        self.u_vol, self.u_covered, self.u_owner = owned_volumes(g, 'u')
        self.v_vol, self.v_covered, self.v_owner = owned_volumes(g, 'v')
        self.u_vol_eff = self.u_vol.copy()
        for (js, is_), (jm, im) in g.u_merge_list:
            vm = self.u_vol[js, is_] + self.u_vol[jm, im]
            self.u_vol_eff[js, is_] = vm
            self.u_vol_eff[jm, im] = vm
        self.v_vol_eff = self.v_vol.copy()
        for (js, is_), (jm, im) in g.v_merge_list:
            vm = self.v_vol[js, is_] + self.v_vol[jm, im]
            self.v_vol_eff[js, is_] = vm
            self.v_vol_eff[jm, im] = vm
