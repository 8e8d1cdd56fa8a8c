"""Time the reference's own ghost-cell AB2/CN step on the host (test infrastructure).

The reference's Numba kernels cannot be compiled here (numba is not installed), so this runs the
reference's code under the same harness as tests/golden/make_golden.py: its ``solver/`` copied to
a temporary directory, ``mac_engine`` built from ``solver/src/bindings.cpp``, ``numba.njit``
replaced by the plain Python function.  Two figures, both on one host thread (FFT_WORKERS=1):

* ``stub``        the reference's code with its arithmetic unchanged (Numba kernels as plain
                  Python loops);
* ``stub+scipy``  the same with the two CSR kernels (apply_csr_spmv_numba,
                  evaluate_H_matvec_fused_numba) replaced by scipy.sparse products, a closer
                  stand-in for compiled Numba speed.

and the oracle port (oracle/ghost_oracle.py, the bench's CPU baseline) on the same workload for
the ratio.  The workload is bench.py's default (800x820, seeded v perturbation); the first,
Helmholtz-building step is excluded.  Run here, not on the GPU machine (the reference is not there):

    python oracle/time_reference_stub.py --reference <path of the reference checkout> [--steps 2]

With ``--path staircase``, ``--path legacy_ghost`` or ``--path cutcell_legacy`` it times the
reference's legacy loop (MAC_CylinderFlow(time_scheme='legacy', transport='centered') with
boundary='staircase', 'ghost_cell' or 'cut_cell': mac_engine compiled with OpenMP, the sparse LU
factored in setup, the ghost-cell branch's Python image-point loops, the cut-cell branch's numpy
predictor) on bench.py's matching workload, after setup and three steps, with all the host's
threads.

With ``--path cut_cell`` it times the reference's cut-cell AB2/CN step instead
(MAC_CylinderFlow(boundary='cut_cell'), CutCellBoundary.advance_ab2_cn: numpy and scipy, no
Numba kernel on that path) on bench.py's cutcell_800x820_re100 workload, after setup and the
start-up step.
"""
from __future__ import annotations

import argparse
import json
import shutil
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[1]


def seeded(s, w, pack, unpack, nu_active):
    rng = np.random.default_rng(w['seed'])
    q = pack(s.u, s.v).copy()
    q[nu_active:] += w['amp'] * rng.standard_normal(q.size - nu_active)
    u, v = unpack(q)
    s.u[:], s.v[:] = u, v


def time_reference(w, steps, scipy_spmv):
    import scipy.sparse as sp
    import numba_kernels as nk
    import optimized_ghost_cell as ogc
    from main import MAC_CylinderFlow
    if scipy_spmv:
        def spmv(data, indices, indptr, x, out):
            n = len(indptr) - 1
            out[:] = sp.csr_matrix((data, indices, indptr), shape=(n, x.size)) @ x

        def hmat(data, indices, indptr, x, dt, out):
            n = len(indptr) - 1
            out[:] = x - 0.5 * dt * (sp.csr_matrix((data, indices, indptr), shape=(n, x.size)) @ x)
        nk.apply_csr_spmv_numba = spmv
        nk.evaluate_H_matvec_fused_numba = hmat
        ogc.nk = nk
    kw = {k: w[k] for k in ('nx', 'ny', 'Lx', 'Ly', 'D', 'xc', 'yc', 'nu')}
    s = MAC_CylinderFlow(boundary='ghost_cell', time_scheme='ab2_cn', verbose=False, **kw)
    seeded(s, w, s.gg.pack, s.gg.unpack, len(s.gg.ui))
    s.solve(n_steps=1, dt=w['dt'], perturb_transient=False, save_artifacts=False, verbose=False)
    t0 = time.perf_counter()
    for _ in range(steps):
        s.solve(n_steps=1, dt=w['dt'], perturb_transient=False, save_artifacts=False, verbose=False)
    el = time.perf_counter() - t0
    return w['nx'] * w['ny'] * steps / el, el


def time_cut_cell(w, steps):
    from main import MAC_CylinderFlow
    kw = {k: w[k] for k in ('nx', 'ny', 'Lx', 'Ly', 'D', 'xc', 'yc', 'nu')}
    t0 = time.perf_counter()
    s = MAC_CylinderFlow(boundary='cut_cell', time_scheme='ab2_cn', pressure_solver='direct', verbose=False, **kw)
    setup = time.perf_counter() - t0
    active_u = s.cut_geom.ax[:, 1:] > 0
    active_v = s.cut_geom.ay[1:-1, :] > 0
    nu_active = int(active_u.sum())

    def pack(u, v):
        return np.r_[u[:, 1:][active_u], v[1:-1][active_v]]

    def unpack(q):
        u, v = s.u.copy(), np.zeros_like(s.v)
        u[:, 1:][active_u] = q[:nu_active]
        v[1:-1][active_v] = q[nu_active:]
        return u, v
    seeded(s, w, pack, unpack, nu_active)
    s.solve(n_steps=1, dt=w['dt'], perturb_transient=False, save_artifacts=False, verbose=False)
    t0 = time.perf_counter()
    s.solve(n_steps=steps, dt=w['dt'], perturb_transient=False, save_artifacts=False, verbose=False)
    el = time.perf_counter() - t0
    return w['nx'] * w['ny'] * steps / el, el, setup


def time_legacy(w, steps):
    from main import MAC_CylinderFlow
    kw = {k: w[k] for k in ('nx', 'ny', 'Lx', 'Ly', 'D', 'xc', 'yc', 'nu')}
    t0 = time.perf_counter()
    s = MAC_CylinderFlow(boundary=w['boundary'], time_scheme='legacy', transport='centered',
                         pressure_solver='direct', verbose=False, **kw)
    setup = time.perf_counter() - t0
    s.solve(n_steps=3, dt=w['dt'], perturb_transient=False, save_artifacts=False, verbose=False)
    t0 = time.perf_counter()
    s.solve(n_steps=steps, dt=w['dt'], perturb_transient=False, save_artifacts=False, verbose=False)
    el = time.perf_counter() - t0
    return w['nx'] * w['ny'] * steps / el, el, setup


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--reference', type=Path, required=True, help='path of the reference checkout')
    ap.add_argument('--steps', type=int, default=2)
    ap.add_argument('--path', choices=('ghost_cell', 'cut_cell', 'staircase', 'legacy_ghost', 'cutcell_legacy'),
                    default='ghost_cell')
    args = ap.parse_args()
    sys.path.insert(0, str(ROOT))
    sys.path.insert(0, str(ROOT / 'tests' / 'golden'))
    import bench
    import make_golden
    if args.path in ('staircase', 'legacy_ghost', 'cutcell_legacy'):
        name = f'{args.path}_800x820_re100'
        w = bench.LEGACY_WORKLOADS[name]
        work = Path(tempfile.mkdtemp(prefix='ghost_ref_time_'))
        try:
            make_golden.build_harness(args.reference, work)
            rate, el, setup = time_legacy(w, args.steps)
        finally:
            shutil.rmtree(work, ignore_errors=True)
        import os
        print(json.dumps(dict(workload=name, threads=os.cpu_count(),
                              reference=dict(value=rate, steps=args.steps, seconds=el, ms_per_step=el / args.steps * 1e3,
                                             setup_seconds=setup)), indent=2))
        return
    if args.path == 'cut_cell':
        w = bench.CUTCELL_WORKLOADS['cutcell_800x820_re100']
        work = Path(tempfile.mkdtemp(prefix='ghost_ref_time_'))
        try:
            make_golden.build_harness(args.reference, work)
            rate, el, setup = time_cut_cell(w, args.steps)
        finally:
            shutil.rmtree(work, ignore_errors=True)
        print(json.dumps(dict(workload='cutcell_800x820_re100', threads=1,
                              reference=dict(value=rate, steps=args.steps, seconds=el, setup_seconds=setup)),
                         indent=2))
        return
    w = bench.WORKLOADS[bench.DEFAULT_WORKLOAD]
    out = dict(workload=bench.DEFAULT_WORKLOAD, threads=1)
    rate, steps, el = bench.oracle_rate(w, args.steps, 600.0, 1)
    out['port'] = dict(value=rate, steps=steps, seconds=el)
    for tag, scipy_spmv in (('stub', False), ('stub+scipy', True)):
        work = Path(tempfile.mkdtemp(prefix='ghost_ref_time_'))
        saved = list(sys.path)
        try:
            make_golden.build_harness(args.reference, work)
            rate, el = time_reference(w, args.steps, scipy_spmv)
            out[tag] = dict(value=rate, steps=args.steps, seconds=el)
        finally:
            sys.path[:] = saved
            for name in [m for m in sys.modules if m in ('main', 'numba_kernels', 'optimized_ghost_cell',
                                                          'rectangular_inverse', 'pressure_schur',
                                                          'time_integration', 'ghost_cell', 'cut_cell_solver',
                                                          'ghost_reconstruction', 'mac_engine', 'numba')]:
                del sys.modules[name]
            shutil.rmtree(work, ignore_errors=True)
    print(json.dumps(out, indent=2))


if __name__ == '__main__':
    main()
