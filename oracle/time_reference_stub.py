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


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--reference', type=Path, required=True, help='path of the reference checkout')
    ap.add_argument('--steps', type=int, default=2)
    args = ap.parse_args()
    sys.path.insert(0, str(ROOT))
    sys.path.insert(0, str(ROOT / 'tests' / 'golden'))
    import bench
    import make_golden
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
