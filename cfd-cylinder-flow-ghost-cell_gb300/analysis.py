"""Force-history analysis on the host (postprocessing/analysis.py:8-103).

``periodic_metrics(t, cd, cl, t_start, D, U_ref)`` turns the C_D / C_L series of a run into
window statistics, the shedding period and Strouhal number from upward zero crossings of the
mean-free lift, and drift measures over the resolved cycles; no frequency is reported when
fewer than two periods are resolved.  Same arguments, keys and error behaviour as the
reference (config 3 reports its shedding frequency through it).
"""
from __future__ import annotations

import numpy as np


def _trapezoid(y, x):
    return float(np.sum(np.diff(x) * (y[:-1] + y[1:]) / 2))


def window_statistics(t, values, left, right):
    """Time-weighted statistics of piecewise-linear series on [left, right]: mean, centred
    rms, minimum, maximum, mid-extrema, half amplitude and amplitude per column."""
    t, values = np.asarray(t, float), np.asarray(values, float)
    ok = (t.ndim == 1 and len(t) >= 2 and values.ndim == 2 and len(values) == len(t)
          and np.isfinite(t).all() and np.isfinite(values).all() and not np.any(np.diff(t) <= 0)
          and np.isfinite([left, right]).all() and t[0] <= left < right <= t[-1])
    if not ok:
        raise ValueError('Require finite increasing times, vector data and a covered window')
    inner = (t > left) & (t < right)
    knots = np.concatenate(([left], t[inner], [right]))
    ends = np.array([[np.interp(x, t, col) for col in values.T] for x in (left, right)])
    data = np.concatenate((ends[:1], values[inner], ends[1:]))
    w = np.diff(knots)[:, None]
    span = right - left
    mean = np.sum(w * (data[:-1] + data[1:]) / 2, axis=0) / span
    c = data - mean
    # exact integral of the square of a linear segment: (a^2 + a b + b^2) / 3 per unit length
    var = np.sum(w * (c[:-1] ** 2 + c[:-1] * c[1:] + c[1:] ** 2) / 3, axis=0) / span
    lo, hi = data.min(axis=0), data.max(axis=0)
    return dict(mean=mean.tolist(), rms=np.sqrt(np.maximum(0.0, var)).tolist(), minimum=lo.tolist(),
                maximum=hi.tolist(), mid_extrema=((lo + hi) / 2).tolist(), half_amplitude=((hi - lo) / 2).tolist(),
                amplitude=(hi - lo).tolist(), window=[float(left), float(right)])


def periodic_metrics(t, cd, cl, t_start, D=.4, U_ref=1.):
    """Shedding metrics of a force history (postprocessing/analysis.py:47-103)."""
    t, cd, cl = (np.asarray(x, dtype=float) for x in (t, cd, cl))
    shapes_ok = all(x.ndim == 1 for x in (t, cd, cl)) and len(t) == len(cd) == len(cl) and len(t) >= 3
    if (not shapes_ok or not all(np.isfinite(x).all() for x in (t, cd, cl)) or np.any(np.diff(t) <= 0)):
        raise ValueError('Histories must be finite, equal-length vectors with strictly increasing time')
    if not all(np.isfinite(x) for x in (t_start, D, U_ref)) or D <= 0 or U_ref <= 0:
        raise ValueError('Require finite t_start and positive D, U_ref')
    sel = t >= t_start
    t, cd, cl = t[sel], cd[sel], cl[sel]
    if len(t) < 3:
        raise ValueError('Analysis window contains fewer than three samples')
    lift = cl - _trapezoid(cl, t) / (t[-1] - t[0])
    # upward crossings of the mean-free lift, located by linear interpolation
    up = np.flatnonzero((lift[:-1] < 0) & (lift[1:] >= 0))
    crossings = t[up] - lift[up] * (t[up + 1] - t[up]) / (lift[up + 1] - lift[up])
    periods = np.diff(crossings)
    resolved = bool(len(periods) >= 2 and np.ptp(cl) > 1e-10 and periods.min() >= 10 * np.diff(t).max())
    cycles = len(periods) if resolved else 0
    a, b = (crossings[0], crossings[-1]) if resolved else (t[0], t[-1])
    st = window_statistics(t, np.column_stack((cd, cl)), a, b)
    out = {}
    for k, name in enumerate(('cd', 'cl')):
        out[f'{name}_mean'] = float(st['mean'][k])
        out[f'{name}_max'] = float(st['maximum'][k])
        out[f'{name}_min'] = float(st['minimum'][k])
        out[f'{name}_mid_extrema'] = float(st['mid_extrema'][k])
        out[f'{name}_half_amplitude'] = float(st['half_amplitude'][k])
        out[f'{name}_amplitude'] = float(st['amplitude'][k])
        out[f'{name}_rms'] = float(st['rms'][k])
    out['cl_amp'] = out['cl_half_amplitude']
    mean_period = float(periods.mean()) if resolved else float('nan')
    out.update(period=mean_period, strouhal=float(D / U_ref / mean_period) if resolved else float('nan'),
               cycles=cycles, sample_start=float(a), sample_end=float(b), stationary=False,
               amplitude_drift=float('nan'), period_drift=float('nan'), drag_drift=float('nan'))
    if cycles >= 4:
        amplitudes, drags = [], []
        for left, right in zip(crossings[:-1], crossings[1:]):
            tt = np.concatenate(([left], t[(t > left) & (t < right)], [right]))
            amplitudes.append(np.ptp(np.interp(tt, t, cl)) / 2)
            drags.append(_trapezoid(np.interp(tt, t, cd), tt) / (right - left))
        half = cycles // 2

        def drift(v):
            v = np.asarray(v, float)
            late, early = np.mean(v[-half:]), np.mean(v[:half])
            return float(abs(late - early) / max(abs(late), 1e-12))
        out.update(amplitude_drift=drift(amplitudes), period_drift=drift(periods), drag_drift=drift(drags))
        # screening threshold of the reference (not a proof of a limit cycle)
        out['stationary'] = max(out['amplitude_drift'], out['period_drift'], out['drag_drift']) < .02
    return out


def calculate_gci(f1, f2, f3, r=2., Fs=1.25, r32=None):
    """Three-grid observed order and grid convergence index (postprocessing/analysis.py:106-151):
    a conditional estimate for monotone data, not an error bound.  f1, f2, f3 run from the fine
    grid to the coarse one; r = h2 / h1 and, for unequal ratios, r32 = h3 / h2 (the order then
    solves r^p (r32^p - 1) / (r^p - 1) = |e32 / e21| by bracketing and Brent's method).  Same
    keys, statuses and error messages as the reference."""
    if not all(np.isfinite(x) for x in (f1, f2, f3, r, Fs)) or r <= 1 or Fs < 1:
        raise ValueError('GCI requires finite values, r > 1 and Fs >= 1')
    if r32 is not None and (not np.isfinite(r32) or r32 <= 1):
        raise ValueError('The coarser spacing ratio must exceed one')
    out = dict(p=None, f_ext=None, e_a21_pct=None, gci_fine_pct=None, status='not estimable',
               reason='Nonmonotone, divergent, constant or nearly zero data')
    scale = max(abs(f1), abs(f2), abs(f3), np.finfo(float).tiny)
    e21, e32 = f2 - f1, f3 - f2
    if abs(f1) > 1e-12 * scale:
        out['e_a21_pct'] = float(100 * abs(e21 / f1))
    if min(abs(e21), abs(e32), abs(f1)) <= 1e-12 * scale or e21 * e32 <= 0:
        return out
    if r32 is None or np.isclose(r32, r):
        p = float(np.log(abs(e32 / e21)) / np.log(r))
    else:
        from scipy.optimize import brentq

        def residual(order):
            return np.exp(order * np.log(r)) * np.expm1(order * np.log(r32)) / np.expm1(order * np.log(r)) \
                - abs(e32 / e21)
        top = 10.
        while residual(.01) * residual(top) > 0 and top < 80.:
            top *= 2
        out['order_search_upper'] = top
        if residual(.01) * residual(top) >= 0:
            out['reason'] = f'No positive resolved order in [0.01, {top:g}] for these unequal spacings'
            return out
        p = float(brentq(residual, .01, top))
    out['p'] = p
    if p <= 0:
        return out
    if p < .1:
        out['reason'] = 'Near-zero observed order; extrapolation is ill-conditioned'
        return out
    out.update(f_ext=float(f1 - e21 / (r ** p - 1)), gci_fine_pct=float(100 * Fs * abs(e21 / f1) / (r ** p - 1)),
               status='conditional estimate',
               reason='Requires asymptotic behaviour and negligible time/sampling error; not established by three '
                      'points alone')
    return out
