"""Wake-centre-line and stagnation-pressure samples of a running case, and their window means.

Counterpart of postprocessing/cylinder_observables.py for the GPU ghost-cell solver: the same
sample file format (schema 1: a JSON header next to a raw little-endian float64 file of rows
``time, p_front, p_back, u_centerline...``), the same recording rule and the same trapezoidal
window integration, so files written here and by the reference are interchangeable.  The point
pressures use the library's quadratic reconstruction (gm_pressure_reconstruction, the
reference's build_pressure_reconstruction); the centre line interpolates u linearly in y.
"""
from __future__ import annotations

import json
from pathlib import Path

import numpy as np


def recirculation_length(x, velocity, rear, diameter):
    """First reattachment of the mean reverse-flow region attached to the cylinder rear
    (postprocessing/cylinder_observables.py:8-27): distance from the rear over D."""
    x, velocity = np.asarray(x, dtype=float), np.asarray(velocity, dtype=float)
    valid = (x.ndim == 1 and x.shape == velocity.shape and len(x) >= 2 and np.isfinite([rear, diameter]).all()
             and diameter > 0 and np.isfinite(x).all() and np.isfinite(velocity).all()
             and not np.any(np.diff(x) <= 0) and x[0] >= rear - 1e-10)
    if not valid:
        raise ValueError('Invalid wake centerline')
    reverse = np.nonzero(velocity < 0)[0]
    if reverse.size == 0:
        return dict(status='no_resolved_reverse_flow', length_D=None)
    first = int(reverse[0])
    if first > 1:
        return dict(status='detached_negative_region', length_D=None)
    up = np.nonzero((velocity[first:-1] < 0) & (velocity[first + 1:] >= 0))[0]
    if up.size == 0:
        return dict(status='reattachment_outside_sampled_domain', length_D=None)
    i = first + int(up[0])
    # zero of the linear interpolant between samples i and i + 1
    x0 = x[i] - velocity[i] * (x[i + 1] - x[i]) / (velocity[i + 1] - velocity[i])
    return dict(status='resolved', length_D=float((x0 - rear) / diameter), x_reattachment=float(x0),
                definition='First reattachment of the connected mean reverse-flow region; distance from cylinder rear / D')


class CylinderSamples:
    """Records, every `stride` calls, the time, the pressures at the cylinder's front and rear
    stagnation points and u along the wake centre line y = yc, from the rear to the outlet
    (postprocessing/cylinder_observables.py:30-79)."""

    def __init__(self, solver, path, stride=10):
        if getattr(solver, 'gg', None) is None or isinstance(stride, bool) or not isinstance(stride, int) \
                or stride < 1:
            raise ValueError('Cylinder sampling requires Ghost AB2/CN and a positive integer stride')
        self.solver, self.path, self.stride = solver, Path(path), stride
        self.calls, self.last = 0, -np.inf
        front_back = np.array([[solver.yc, solver.xc - solver.D / 2], [solver.yc, solver.xc + solver.D / 2]])
        self.pressure_operator = solver.gg.pressure_reconstruction(front_back)
        # first u column at or behind the rear of the cylinder, to the outlet
        self.first = int(np.ceil((solver.xc + solver.D / 2) / solver.dx - 1e-12))
        self.x = np.arange(self.first, solver.nx + 1) * solver.dx
        # u rows sit at (j + 1/2) dy: the centre line lies between rows j and j + 1
        frac = solver.yc / solver.dy - .5
        self.j = int(np.floor(frac))
        self.weight = frac - self.j
        if not 0 <= self.j < solver.ny - 1:
            raise ValueError('Wake centerline interpolation reaches an outer wall')
        header = dict(schema=1, columns=3 + len(self.x), dtype='<f8', stride=stride, x=self.x.tolist(),
                      rear=solver.xc + solver.D / 2, diameter=solver.D,
                      quantities=['time', 'p_front', 'p_back', 'u_centerline'],
                      sampling='Linear MAC interpolation in y; temporal trapezoids clipped to the requested window')
        self.path.parent.mkdir(parents=True, exist_ok=True)
        with self.path.with_suffix('.json').open('x', encoding='utf-8') as stream:
            json.dump(header, stream, indent=2)
        self.stream = self.path.open('xb')

    def pressures(self):
        return self.pressure_operator @ np.asarray(self.solver.p).ravel()

    def record(self, *, force=False, pressures=None):
        self.calls += 1
        if not force and self.calls % self.stride:
            return
        s = self.solver
        if s.time == self.last:
            return
        if s.time < self.last:
            raise ValueError('Sample times must increase')
        p = self.pressures() if pressures is None else pressures
        u = np.asarray(s.u)
        centre = (1 - self.weight) * u[self.j, self.first:] + self.weight * u[self.j + 1, self.first:]
        row = np.concatenate(([s.time], p, centre)).astype('<f8')
        if not np.isfinite(row).all():
            raise ValueError('Nonfinite cylinder sample')
        self.stream.write(row.tobytes())
        self.last = s.time

    def flush(self):
        self.stream.flush()

    def close(self):
        self.stream.close()


def mean_observables(path, left, right):
    """Time means over [left, right] of a sample file by exact trapezoids of the piecewise-linear
    samples clipped to the window (postprocessing/cylinder_observables.py:82-120)."""
    path = Path(path)
    meta = json.loads(path.with_suffix('.json').read_text(encoding='utf-8'))
    ncol = meta['columns']
    if (meta['schema'] != 1 or ncol != 3 + len(meta['x']) or meta['dtype'] != '<f8'
            or path.stat().st_size % (8 * ncol) or not np.isfinite([left, right]).all() or right <= left):
        raise ValueError('Invalid sample file or integration window')
    nrow = path.stat().st_size // (8 * ncol)
    if nrow < 2:
        raise ValueError('At least two samples are required')
    rows = np.fromfile(path, dtype='<f8').reshape(nrow, ncol)
    if rows[0, 0] > left or rows[-1, 0] < right:
        raise ValueError('Samples do not cover the full requested window')
    if not np.isfinite(rows).all() or np.any(np.diff(rows[:, 0]) <= 0):
        # the reference reports the first offending row in time order; same message either way
        bad = next(k for k in range(nrow) if not np.isfinite(rows[k]).all()
                   or (k > 0 and rows[k, 0] <= rows[k - 1, 0]))
        raise ValueError('Nonfinite sample' if bad == 0 else 'Nonfinite, duplicate or unordered sample')
    integral = np.zeros(ncol - 1)
    duration, max_dt = 0.0, 0.0
    for k in range(1, nrow):
        prev, cur = rows[k - 1], rows[k]
        a, b = max(left, prev[0]), min(right, cur[0])
        if b <= a:
            continue
        step = cur[0] - prev[0]
        slope = (cur[1:] - prev[1:]) / step
        va = prev[1:] + (a - prev[0]) * slope
        vb = prev[1:] + (b - prev[0]) * slope
        integral += .5 * (b - a) * (va + vb)
        duration += b - a
        max_dt = max(max_dt, float(step))
    if not np.isclose(duration, right - left, rtol=1e-12, atol=1e-12):
        raise ValueError('Incomplete integration window')
    mean = integral / duration
    return dict(window=[float(left), float(right)], p_front_mean=float(mean[0]), p_back_mean=float(mean[1]),
                delta_p_mean=float(mean[0] - mean[1]), x=meta['x'], u_centerline_mean=mean[2:].tolist(),
                sample_max_dt=max_dt,
                recirculation=recirculation_length(meta['x'], mean[2:], meta['rear'], meta['diameter']),
                caveat='Temporal profile sampling error requires a stride-sensitivity check; no instantaneous '
                       'checkpoint is substituted for the mean.')
