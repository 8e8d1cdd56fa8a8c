"""Long-run comparison of the FP32 mode with the plain FP64 step on the wide shedding case.

The case is the 40D x 41D domain with the cylinder at (10D, 20.5D): an 800x820 grid (h = 0.05),
Re = 100, dt = 0.002, started from u = 1 with a seeded 1e-2 perturbation of v. Both precisions
run the same number of steps from the same state. The force histories are compared
step by step and through ``analysis.periodic_metrics`` (postprocessing/analysis.py:47-103):
mean C_D, C_L amplitude and, once two shedding periods are resolved, the Strouhal number.

    python -m <package>.validation --steps 10000
"""
from __future__ import annotations

import numpy as np

from . import analysis
from .ghost import MAC_CylinderFlow

WIDE = dict(nx=800, ny=820, Lx=40.0, Ly=41.0, D=1.0, xc=10.0, yc=20.5, nu=0.01)


def seeded_case(precision, seed=0, amp=1e-2, **case):
    kw = dict(WIDE, **case)
    s = MAC_CylinderFlow(boundary='ghost_cell', time_scheme='ab2_cn', verbose=False, precision=precision, **kw)
    q = s.gg.pack(s.u, s.v)
    nu_faces = len(s.gg.ui)
    q[nu_faces:] += amp * np.random.default_rng(seed).standard_normal(q.size - nu_faces)
    s.u[:], s.v[:] = s.gg.unpack(q)
    return s


def histories(precision, steps, dt=0.002, **case):
    """(t, C_D, C_L, max divergence over the run) of `steps` AB2/CN steps."""
    s = seeded_case(precision, **case)
    t, cd, cl = s.solve(n_steps=steps, dt=dt, perturb_transient=False, save_artifacts=False, verbose=False)
    return np.asarray(t), np.asarray(cd), np.asarray(cl), float(s.last_step_diagnostics['max_divergence'])


def compare(steps, dt=0.002, **case):
    """Both precisions over `steps` steps: per-step force differences and the periodic metrics
    of the second half of the run (None where fewer than two periods are resolved)."""
    out = {}
    runs = {p: histories(p, steps, dt, **case) for p in ('fp64', 'fp32')}
    for p, (t, cd, cl, div) in runs.items():
        try:
            m = analysis.periodic_metrics(t, cd, cl, t_start=t[-1] / 2, D=case.get('D', WIDE['D']), U_ref=1.0)
        except ValueError:
            m = None
        out[p] = dict(final_cd=float(cd[-1]), final_cl=float(cl[-1]), max_divergence_last=div, metrics=m)
    t64, cd64, cl64, _ = runs['fp64']
    _, cd32, cl32, _ = runs['fp32']
    scale_cl = max(float(np.max(np.abs(cl64))), 1e-12)
    rel_cd = np.abs(cd32 - cd64) / np.abs(cd64)
    out['difference'] = dict(
        max_rel_cd=float(rel_cd.max()),
        max_rel_cd_first_1000=float(rel_cd[:1000].max()),
        max_abs_cl_over_max_cl=float(np.max(np.abs(cl32 - cl64)) / scale_cl),
        steps=int(steps), end_time=float(t64[-1]))
    return out


if __name__ == '__main__':
    import argparse
    import json
    ap = argparse.ArgumentParser(description=__doc__)
    ap.add_argument('--steps', type=int, default=10000)
    a = ap.parse_args()
    print(json.dumps(compare(a.steps), default=float))
