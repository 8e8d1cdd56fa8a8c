"""Generate golden vectors by running the reference's own ghost-cell code.

Run once in a container that holds the reference checkout:

    python tests/golden/make_golden.py --reference <path of the reference checkout>

The reference's ``solver/`` is copied to a temporary directory, its compiled
``mac_engine`` is built from ``solver/src/bindings.cpp`` (the shipped Windows
binary is deleted, never loaded), ``numba`` is replaced by a stand-in whose
``njit`` returns the plain Python function (numba is not installed here), and
``matplotlib`` by a no-op module.  The outputs are small ``.npz`` files in this
directory; the tests read only those files.
"""
from __future__ import annotations

import argparse
import os
import shutil
import subprocess
import sys
import sysconfig
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent

NUMBA_STUB = '''
def njit(*args, **kwargs):
    def wrap(function):
        function.py_func = function
        function.nopython_signatures = [()]
        return function
    if args and callable(args[0]) and not kwargs:
        return wrap(args[0])
    return wrap
prange = range
'''
PYPLOT_STUB = '''
def __getattr__(name):
    return lambda *a, **k: None
'''


def build_harness(reference: Path, work: Path) -> Path:
    solver = work / 'solver'
    shutil.copytree(reference / 'solver', solver, ignore=shutil.ignore_patterns('*.pyd', '__pycache__'))
    shutil.copytree(reference / 'postprocessing', work / 'postprocessing',
                    ignore=shutil.ignore_patterns('__pycache__'))
    shutil.copytree(reference / 'verification', work / 'verification',
                    ignore=shutil.ignore_patterns('__pycache__'))
    (work / 'validation').mkdir()
    for name in ('__init__.py', 'run_ghost_validation.py'):
        shutil.copy(reference / 'validation' / name, work / 'validation' / name)
    stubs = work / 'stubs'
    (stubs / 'matplotlib').mkdir(parents=True)
    (stubs / 'numba.py').write_text(NUMBA_STUB)
    (stubs / 'matplotlib' / '__init__.py').write_text('')
    (stubs / 'matplotlib' / 'pyplot.py').write_text(PYPLOT_STUB)
    import pybind11
    suffix = sysconfig.get_config_var('EXT_SUFFIX')
    inc = sysconfig.get_paths()['include']
    subprocess.run(['g++', '-O3', '-std=c++17', '-fopenmp', '-shared', '-fPIC', f'-I{inc}',
                    f'-I{pybind11.get_include()}', str(solver / 'src' / 'bindings.cpp'),
                    '-o', str(solver / f'mac_engine{suffix}')], check=True)
    sys.path[:0] = [str(stubs), str(solver), str(work)]
    os.environ['FFT_WORKERS'] = '1'
    return solver


def csr_parts(m):
    m = m.tocsr()
    return dict(data=m.data.copy(), indices=m.indices.astype(np.int64), indptr=m.indptr.astype(np.int64),
                shape=np.array(m.shape))


def ghost_rows(E, ids):
    """The rows of an extension matrix that are not identity rows of active entries."""
    E = E.tocsr()
    identity = np.zeros(E.shape[0], bool)
    identity[ids] = True
    rows = np.flatnonzero(~identity & (np.diff(E.indptr) > 0))
    sub = E[rows]
    sub.sort_indices()
    return dict(rows=rows.astype(np.int64), indptr=sub.indptr.astype(np.int64),
                cols=sub.indices.astype(np.int64), vals=sub.data.copy())


def save(name, **arrays):
    flat = {}
    for key, value in arrays.items():
        if isinstance(value, dict):
            for k2, v2 in value.items():
                flat[f'{key}__{k2}'] = np.asarray(v2)
        else:
            flat[key] = np.asarray(value)
    np.savez_compressed(HERE / f'{name}.npz', **flat)
    print('wrote', name, sum(v.nbytes for v in flat.values()), 'bytes raw')


def geometry_record(s):
    g = s.gg
    return dict(ui=g.ui.astype(np.int64), vi=g.vi.astype(np.int64), pi=g.pi.astype(np.int64),
                Eu=ghost_rows(g.E[:s.u.size, :len(g.ui)], g.ui), Ev=ghost_rows(g.E[s.u.size:, len(g.ui):], g.vi),
                P=ghost_rows(g.P, g.pi))


def schur_rows_of(actual, indices, rect):
    """Same rule as the reference's boundary_row_inverse, restated to expose the rows."""
    import scipy.sparse as sp
    indices = np.asarray(indices)
    covered = np.ones(rect.shape[0], bool)
    covered[indices] = False
    coo = actual.tocoo()
    ext = sp.csr_matrix((coo.data, (indices[coo.row], indices[coo.col])), shape=rect.shape)
    virt = rect.tocoo()
    keep = covered[virt.row] & covered[virt.col]
    ext += sp.csr_matrix((virt.data[keep], (virt.row[keep], virt.col[keep])), shape=rect.shape)
    delta = (ext - rect).tocsr()
    tol = 8 * np.finfo(float).eps * max(1., float(np.max(abs(rect.diagonal()))))
    delta.data[abs(delta.data) < tol] = 0.
    delta.eliminate_zeros()
    return np.flatnonzero(np.diff(delta.indptr)).astype(np.int64)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--reference', type=Path, required=True, help='path of the reference checkout')
    ap.add_argument('--skip-large', action='store_true')
    ap.add_argument('--only', choices=('taylor_green', 'analysis', 'runner', 'legacy', 'modal', 'cutcell',
                                       'staircase', 'legacy_ghost', 'cutcell_legacy', 'legacy_options',
                                       'legacy_wide', 'cutcell_gate'),
                    help='generate one group of fixtures only')
    args = ap.parse_args()
    work = Path(tempfile.mkdtemp(prefix='ghost_golden_'))
    try:
        build_harness(args.reference, work)
        if args.only == 'taylor_green':
            run_taylor_green(work)
        elif args.only == 'analysis':
            run_analysis(work)
        elif args.only == 'runner':
            run_runner(work)
        elif args.only == 'legacy':
            run_legacy(work)
        elif args.only == 'modal':
            run_modal(work)
        elif args.only == 'cutcell':
            run_cutcell(work)
        elif args.only == 'staircase':
            run_staircase(work)
        elif args.only == 'legacy_ghost':
            run_legacy_ghost(work)
        elif args.only == 'cutcell_legacy':
            run_cutcell_legacy(work)
        elif args.only == 'legacy_options':
            run_legacy_options(work)
        elif args.only == 'legacy_wide':
            run_legacy_wide(work)
        elif args.only == 'cutcell_gate':
            run_cutcell_gate(work)
        else:
            run_all(args)
            run_taylor_green(work)
            run_analysis(work)
            run_runner(work)
            run_legacy(work)
            run_modal(work)
            run_cutcell(work)
            run_staircase(work)
            run_legacy_ghost(work)
            run_cutcell_legacy(work)
            run_legacy_options(work)
            if not args.skip_large:
                run_legacy_wide(work)
                run_cutcell_gate(work)
    finally:
        shutil.rmtree(work, ignore_errors=True)


RUNNER_CASE = dict(kind='steady', dt=0.002, end_time=0.03, sample_start=0.01, profile_stride=2,
                   solver=dict(nx=88, ny=16, Lx=22., Ly=4.1, D=1., xc=2., yc=2., nu=0.02,
                               boundary='ghost_cell', time_scheme='ab2_cn'))


def run_runner(work):
    """A checkpoint written by the reference's own save_checkpoint (solver/main.py:503-530) and
    the fields after the reference resumes it; the reference's runner contract
    (validation/run_ghost_validation.py:19-102) on a small case: its history rows, summary,
    mean observables and centre-line samples; the pressure reconstruction operator and
    recirculation lengths of postprocessing/cylinder_observables.py."""
    import json
    from main import MAC_CylinderFlow
    from cut_cell_solver import build_pressure_reconstruction
    from postprocessing.cylinder_observables import recirculation_length
    from validation import run_ghost_validation as runner

    # 1. checkpoint after 4 noisy steps, then 3 more steps from the reloaded checkpoint
    kw = dict(RUNNER_CASE['solver'])
    s = MAC_CylinderFlow(verbose=False, **kw)
    q = s.gg.pack(s.u, s.v).copy()
    q += 1e-2 * np.random.default_rng(9).standard_normal(q.size)
    u0, v0 = s.gg.unpack(q)
    s.u[:], s.v[:] = u0, v0
    s.solve(n_steps=4, dt=.002, perturb_transient=False, save_artifacts=False, verbose=False)
    ck = work / 'reference_checkpoint.npz'
    s.save_checkpoint(ck)
    shutil.copy(ck, HERE / 'reference_checkpoint_88x16.npz')
    r = MAC_CylinderFlow.from_checkpoint(ck)
    scal = []
    for _ in range(3):
        r.solve(n_steps=1, dt=.002, perturb_transient=False, save_artifacts=False, verbose=False)
        d = r.last_step_diagnostics
        scal.append([r.time, d['cd'], d['cl'], d['max_divergence']])
    save('reference_resume_88x16', u=r.u, v=r.v, p=r.p, scalars=np.array(scal))

    # 2. the runner on a small steady case
    cfg = work / 'case.json'
    cfg.write_text(json.dumps(RUNNER_CASE))
    out = work / 'run'
    runner.run(cfg, out)
    rows = [json.loads(line) for line in (out / 'history.jsonl').read_text().splitlines()]
    keys = sorted(k for k in rows[0] if isinstance(rows[0][k], (int, float)) and k != 'wall_seconds')
    history = np.array([[float(row[k]) for k in keys] for row in rows])
    centre = np.fromfile(out / 'centerline.bin', dtype='<f8')
    s2 = MAC_CylinderFlow(verbose=False, **kw)
    pts = np.array([[s2.yc, s2.xc - s2.D / 2], [s2.yc, s2.xc + s2.D / 2], [1.3, 3.7], [3.0, 1.2], [2.0, 10.0]])
    rec = build_pressure_reconstruction(s2.gg.geom, pts)
    x = np.linspace(1.5, 6.0, 10)
    recirc, status = [], []
    for vel in (np.linspace(-1, 1, 10), np.linspace(0.1, 1, 10), np.r_[0.2, 0.3, -0.1, -0.2, np.linspace(.1, 1, 6)],
                -np.ones(10)):
        res = recirculation_length(x, vel, 1.5, 1.0)
        recirc.append([np.nan if res.get('length_D') is None else res['length_D']])
        status.append(res['status'])
    save('runner_88x16', case=json.dumps(RUNNER_CASE), history_keys=np.array(keys), history=history,
         summary=(out / 'summary.json').read_text(), mean_observables=(out / 'mean_observables.json').read_text(),
         centerline_meta=(out / 'centerline.json').read_text(), centerline=centre,
         rec_points=pts, rec_indptr=rec.indptr.astype(np.int64), rec_indices=rec.indices.astype(np.int64),
         rec_data=rec.data.copy(), recirc_x=x, recirc_lengths=np.array(recirc), recirc_status=np.array(status))


def run_legacy(work):
    """The reference's native kernels of the legacy staircase path (solver/src/bindings.cpp,
    module mac_engine built from source) on seeded fields with a staircase cylinder mask."""
    import mac_engine
    out = {}
    for tag, (nx, ny) in {'a': (64, 40), 'b': (37, 23)}.items():
        rng = np.random.default_rng(21 if tag == 'a' else 22)
        dx, dy = 0.11, 0.13
        xc, yc, r = nx * dx * 0.35, ny * dy * 0.5, 0.9
        xx, yy = np.meshgrid((np.arange(nx) + .5) * dx, (np.arange(ny) + .5) * dy)
        mask = np.ascontiguousarray((xx - xc) ** 2 + (yy - yc) ** 2 <= r * r)
        u = rng.standard_normal((ny, nx + 1))
        v = rng.standard_normal((ny + 1, nx))
        p = rng.standard_normal((ny, nx))
        phi = rng.standard_normal((ny, nx))
        inlet = 1.0 + 0.1 * rng.standard_normal(ny)
        dt, nu, rho = 0.003, 0.02, 1.3
        out[f'{tag}_in'] = np.array([nx, ny, dx, dy, dt, nu, rho])
        for name, a in (('u', u), ('v', v), ('p', p), ('phi', phi), ('inlet', inlet), ('mask', mask)):
            out[f'{tag}_{name}'] = a
        for slip in (0, 1):
            for centered in (0, 1):
                us, vs, rhs = np.zeros_like(u), np.zeros_like(v), np.zeros_like(p)
                mac_engine.predictor_rhs_cpp(u, v, us, vs, rhs, p, mask, inlet, dx, dy, dt, nu, rho, bool(slip),
                                             bool(centered))
                key = f'{tag}_pred_s{slip}c{centered}'
                out[key + '_us'], out[key + '_vs'], out[key + '_rhs'] = us, vs, rhs
        us, vs = rng.standard_normal(u.shape), rng.standard_normal(v.shape)
        uc, vc = u.copy(), v.copy()
        mac_engine.corrector_cpp(uc, vc, us, vs, phi, mask, inlet, dx, dy, dt, rho, False)
        out[f'{tag}_corr_us'], out[f'{tag}_corr_vs'] = us, vs
        out[f'{tag}_corr_u'], out[f'{tag}_corr_v'] = uc, vc
        out[f'{tag}_forces'] = np.array(mac_engine.calculate_mac_forces_cpp(u, v, p, mask, dx, dy, nu * rho))
        d = mac_engine.calculate_mac_divergence_cpp(u, v, mask, dx, dy)
        out[f'{tag}_div'] = np.array([d[0], d[1], d[2], d[3], d[4]], dtype=float)
    save('legacy_kernels', **out)


CUTCELL_CASES = {
    'cc40x20': dict(nx=40, ny=20, Lx=4., Ly=2., D=1., xc=1., yc=1., nu=0.02, rho=1.),
    'cc48x30': dict(nx=48, ny=30, Lx=4.8, Ly=2.4, D=1., xc=1.3, yc=1.15, nu=0.01, rho=1.3),
}


def run_cutcell(work):
    """The reference's cut-cell AB2/CN path (MAC_CylinderFlow(boundary='cut_cell',
    time_scheme='ab2_cn'), CutCellBoundary of solver/cut_cell_solver.py) on two small grids,
    one with dx != dy and rho != 1: the geometry (solver/cut_cell_geom.py), the wall, face and
    viscous stencils (solver/staggered_wall.py), owned volumes, the surface pressure operator,
    the momentum right-hand side in its advective and viscous forms on seeded fields, a
    pressure solve, the initial projection, and the fields and diagnostics of steps from a
    seeded perturbation of the initial state."""
    from main import MAC_CylinderFlow
    from cut_cell_solver import calculate_cut_cell_divergence
    for tag, kw in CUTCELL_CASES.items():
        s = MAC_CylinderFlow(boundary='cut_cell', time_scheme='ab2_cn', pressure_solver='direct',
                             verbose=False, **kw)
        cc, g = s.cc, s.cc.geom
        out = dict(config=np.array([kw[k] for k in ('nx', 'ny', 'Lx', 'Ly', 'D', 'xc', 'yc', 'nu', 'rho')]))
        for name in ('ax', 'ay', 'volume_fraction', 'cell_type', 'u_volume_fraction', 'v_volume_fraction',
                     'ax_mid', 'ay_mid', 'ay_u', 'ax_v'):
            out['geom_' + name] = getattr(g, name)
        out['u_merge'] = np.array(g.u_merge_list, dtype=np.int64).reshape(-1, 4)
        out['v_merge'] = np.array(g.v_merge_list, dtype=np.int64).reshape(-1, 4)
        for c in ('u', 'v'):
            out[f'{c}_vol'] = getattr(cc, f'{c}_vol')
            out[f'{c}_vol_eff'] = getattr(cc, f'{c}_vol_eff')
            out[f'{c}_covered'] = np.asarray(getattr(cc, f'{c}_covered'), dtype=np.int64)
            out[f'{c}_owner'] = np.asarray(getattr(cc, f'{c}_owner'), dtype=np.int64)
        # the stencil operators by their action on a seeded field (the CSRs are large)
        rng = np.random.default_rng(40 if tag == 'cc40x20' else 43)
        fu = rng.standard_normal(s.u.shape)
        fv = rng.standard_normal(s.v.shape)
        fu[g.ax == 0] = 0.
        fv[g.ay == 0] = 0.
        field = np.r_[fu.ravel(), fv.ravel()]
        out['probe_field'] = field
        w = cc.wall
        out['wall_rate_action'] = w.rate @ field
        out['wall_rate_nnz'] = w.rate.nnz
        for name in ('tx', 'ty', 'ds', 'u_indices', 'v_indices'):
            out['wall_' + name] = np.asarray(getattr(w, name))
        for (c, a), st in cc.momentum_faces.items():
            key = f'mf_{c}{a}'
            out[key + '_indices'] = np.asarray(st.indices, dtype=np.int64)
            out[key + '_u_action'] = st.u @ field
            out[key + '_v_action'] = st.v @ field
            out[key + '_gradient_action'] = st.gradient @ field
            out[key + '_nnz'] = np.array([st.u.nnz, st.v.nnz, st.gradient.nnz])
            out[key + '_patch'] = np.asarray(st.patch, dtype=np.int64)
            out[key + '_lengths'] = np.asarray(st.lengths)
            df = cc.diffusion_faces[c, a]
            out[f'df_{c}{a}_indices'] = np.asarray(df.indices, dtype=np.int64)
            out[f'df_{c}{a}_gradient_action'] = df.gradient @ field
        out['surface_points'] = cc.pressure_points
        out['surface_pressure'] = csr_parts(cc.surface_pressure_operator)
        out['surface_weights'] = cc.pressure_normal_weights
        out['init_u'], out['init_v'] = s.u.copy(), s.v.copy()
        rng = np.random.default_rng(41 if tag == 'cc40x20' else 42)
        u = rng.standard_normal(s.u.shape)
        v = rng.standard_normal(s.v.shape)
        u[g.ax == 0] = 0.
        v[g.ay == 0] = 0.
        out['rand_u'], out['rand_v'] = u, v
        for mode, (nu, adv) in {'adv': (0., True), 'dif': (s.nu, False)}.items():
            au, av, ru, rv = cc.compute_momentum_rhs(u, v, nu, s.rho, transport='centered', include_advection=adv)
            out[f'{mode}_au'], out[f'{mode}_av'], out[f'{mode}_ru'], out[f'{mode}_rv'] = au, av, ru, rv
        prhs = rng.standard_normal(s.p.shape)
        out['prhs'] = prhs
        out['psol'] = cc.solve_pressure(prhs, 0.01, s.rho)
        prand = rng.standard_normal(s.p.shape)
        out['rand_p'] = prand
        out['forces_rand'] = np.array(cc.extract_true_surface_forces(u, v, prand, s.nu * s.rho))
        md, rd, mf, _, _ = calculate_cut_cell_divergence(u, v, g)
        out['divergence_rand'] = np.array([md, rd, mf])
        # steps from a seeded perturbation of the projected initial state
        du = 1e-2 * rng.standard_normal(s.u.shape)
        dv = 1e-2 * rng.standard_normal(s.v.shape)
        du[g.ax == 0] = 0.
        dv[g.ay == 0] = 0.
        du[:, 0] = 0.
        dv[[0, -1], :] = 0.
        s.u += du
        s.v += dv
        out['start_u'], out['start_v'] = s.u.copy(), s.v.copy()
        keys = ('cd', 'cl', 'cd_pressure', 'cd_viscous', 'cl_pressure', 'cl_viscous', 'max_divergence', 'cfl',
                'momentum_iterations', 'coupled_momentum_residual_linf', 'pressure_solves')
        fields, scal = [], []
        for k in range(6):
            s.solve(n_steps=1, dt=.002, perturb_transient=False, save_artifacts=False, verbose=False)
            d = s.last_step_diagnostics
            scal.append([float(d[key]) for key in keys])
            fields.append((s.u.copy(), s.v.copy(), s.p.copy()))
        out['step_keys'] = np.array(keys)
        out['step_scalars'] = np.array(scal)
        out['step_u'] = np.array([f[0] for f in fields])
        out['step_v'] = np.array([f[1] for f in fields])
        out['step_p'] = np.array([f[2] for f in fields])
        out['history_half_p'] = cc.cn_pressure.copy()
        out['history_adv'] = cc.cn_advection.copy()
        if tag == 'cc40x20':
            # a checkpoint written by the reference's own save_checkpoint after the six steps, and
            # the fields after the reference resumes it for three steps (solver/main.py:503-567)
            ck = work / 'reference_checkpoint_cutcell.npz'
            s.save_checkpoint(ck)
            shutil.copy(ck, HERE / 'reference_checkpoint_cutcell_cc40x20.npz')
            r = MAC_CylinderFlow.from_checkpoint(ck)
            r.solve(n_steps=3, dt=.002, perturb_transient=False, save_artifacts=False, verbose=False)
            out['resume_u'], out['resume_v'], out['resume_p'] = r.u.copy(), r.v.copy(), r.p.copy()
            out['resume_scalars'] = np.array([r.time, r.last_step_diagnostics['cd'], r.last_step_diagnostics['cl']])
        if tag == 'cc40x20':
            # a longer run with the inlet perturbation (solver/main.py:281-286)
            s.solve(n_steps=60, dt=.002, perturb_transient=True, perturb_duration=0.3, save_artifacts=False,
                    verbose=False)
            d = s.last_step_diagnostics
            out['long_u'], out['long_v'], out['long_p'] = s.u.copy(), s.v.copy(), s.p.copy()
            out['long_scalars'] = np.array([float(d[key]) for key in keys] + [s.time])
        save(f'cutcell_{tag}', **out)
    run_cutcell_options(work)
    run_cutcell_wide(work)


def run_cutcell_options(work):
    """The cut-cell options on the 40x20 grid: parabolic inflow, slip channel walls and the
    reference's CG/boundary-Schur-DCT pressure solver ('cg_dct'); four steps from the projected
    initial state."""
    from main import MAC_CylinderFlow
    kw = dict(nx=40, ny=20, Lx=4., Ly=2., D=1., xc=1.1, yc=0.95, nu=0.02, inflow='parabolic', U_m=1.2,
              slip_walls=True, pressure_solver='cg_dct')
    s = MAC_CylinderFlow(boundary='cut_cell', time_scheme='ab2_cn', verbose=False, **kw)
    out = dict(init_u=s.u.copy(), init_v=s.v.copy(), u_inlet=s.u_inlet.copy())
    scal, fields = [], []
    for k in range(4):
        s.solve(n_steps=1, dt=.002, perturb_transient=False, save_artifacts=False, verbose=False)
        d = s.last_step_diagnostics
        scal.append([d['cd'], d['cl'], d['max_divergence'], d['cfl']])
        fields.append((s.u.copy(), s.v.copy(), s.p.copy()))
    save('cutcell_options_40x20', **out, step_u=np.array([f[0] for f in fields]),
         step_v=np.array([f[1] for f in fields]), step_p=np.array([f[2] for f in fields]),
         scalars=np.array(scal))


def run_cutcell_wide(work):
    """The benched cut-cell grid (bench.py workload cutcell_800x820_re100: 800x820, 40D x 41D,
    Re 100, the seeded 1e-2 v perturbation of the projected initial state): three reference
    steps, stored as 4000 seeded sample values per field and per step plus the field norms and
    the force coefficients (the full fields would be tens of megabytes)."""
    from main import MAC_CylinderFlow
    kw = dict(nx=800, ny=820, Lx=40.0, Ly=41.0, D=1.0, xc=10.0, yc=20.5, nu=0.01)
    s = MAC_CylinderFlow(boundary='cut_cell', time_scheme='ab2_cn', pressure_solver='direct', verbose=False, **kw)
    g = s.cut_geom
    active_u, active_v = g.ax[:, 1:] > 0, g.ay[1:-1, :] > 0
    nu_active = int(active_u.sum())
    q = np.r_[s.u[:, 1:][active_u], s.v[1:-1][active_v]]
    q[nu_active:] += 1e-2 * np.random.default_rng(0).standard_normal(q.size - nu_active)
    s.u[:, 1:][active_u] = q[:nu_active]
    s.v[1:-1][active_v] = q[nu_active:]
    pick = np.random.default_rng(1)
    su = np.sort(pick.choice(s.u.size, 4000, replace=False))
    sv = np.sort(pick.choice(s.v.size, 4000, replace=False))
    sp_ = np.sort(pick.choice(s.p.size, 4000, replace=False))
    fields, scal = [], []
    for k in range(3):
        s.solve(n_steps=1, dt=.002, perturb_transient=False, save_artifacts=False, verbose=False)
        d = s.last_step_diagnostics
        scal.append([d['cd'], d['cl'], d['max_divergence'], d['cfl'], d['momentum_iterations']])
        fields.append((s.u.ravel()[su].copy(), s.v.ravel()[sv].copy(), s.p.ravel()[sp_].copy(),
                       np.abs(s.u).max(), np.abs(s.v).max(), np.abs(s.p).max(),
                       float(np.sqrt(np.mean(s.u ** 2))), float(np.sqrt(np.mean(s.v ** 2))),
                       float(np.sqrt(np.mean(s.p ** 2)))))
    save('cutcell_wide_800x820', sample_u=su, sample_v=sv, sample_p=sp_,
         u_samples=np.array([f[0] for f in fields]), v_samples=np.array([f[1] for f in fields]),
         p_samples=np.array([f[2] for f in fields]), norms=np.array([f[3:] for f in fields]),
         scalars=np.array(scal))


def run_staircase(work):
    """The reference's legacy staircase loop (MAC_CylinderFlow(boundary='staircase',
    time_scheme='legacy'), solver/main.py:303-381 with mac_engine built from
    solver/src/bindings.cpp and the sparse-LU pressure solve) on a 48x24 grid: centred transport
    (the loop's AB2 step) and upwind transport, 20 steps each, the second with the transient inlet
    perturbation; fields at steps 1, 5 and 20 and the force coefficients of every step."""
    from main import MAC_CylinderFlow
    out = {}
    for tag, transport, perturb in (('centered', 'centered', False), ('upwind', 'upwind', True)):
        s = MAC_CylinderFlow(nx=48, ny=24, Lx=4.8, Ly=2.4, D=1.0, xc=1.3, yc=1.15, nu=0.02, boundary='staircase',
                             time_scheme='legacy', transport=transport, pressure_solver='direct', verbose=False)
        out[f'{tag}_init_u'], out[f'{tag}_init_v'] = s.u.copy(), s.v.copy()
        fields, coef = {}, []
        for k in range(20):
            _, cd, cl = s.solve(n_steps=1, dt=0.002, perturb_transient=perturb, perturb_duration=0.03,
                                save_artifacts=False, verbose=False)
            coef.append([float(cd[0]), float(cl[0])])
            if k + 1 in (1, 5, 20):
                fields[k + 1] = (s.u.copy(), s.v.copy(), s.p.copy())
        for k, (u, v, p) in fields.items():
            out[f'{tag}_u{k}'], out[f'{tag}_v{k}'], out[f'{tag}_p{k}'] = u, v, p
        out[f'{tag}_coef'] = np.array(coef)
        out[f'{tag}_time'] = s.time
    save('staircase_48x24', **out)


def run_legacy_ghost(work):
    """The reference's legacy ghost-cell loop (MAC_CylinderFlow(boundary='ghost_cell',
    time_scheme='legacy'), solver/main.py:303-381 with GhostCellBoundary of solver/ghost_cell.py,
    mac_engine built from solver/src/bindings.cpp and the sparse-LU pressure solve) on the 48x24
    grid of the staircase case: centred and upwind transport, 20 steps each, the second with the
    transient inlet perturbation; its ghost-face tables, fields at steps 1, 5 and 20 and the force
    coefficients of every step."""
    from main import MAC_CylinderFlow
    out = {}
    for tag, transport, perturb in (('centered', 'centered', False), ('upwind', 'upwind', True)):
        s = MAC_CylinderFlow(nx=48, ny=24, Lx=4.8, Ly=2.4, D=1.0, xc=1.3, yc=1.15, nu=0.02, boundary='ghost_cell',
                             time_scheme='legacy', transport=transport, pressure_solver='direct', verbose=False)
        if tag == 'centered':
            gc = s.gc
            for f in ('u', 'v'):
                out[f'ghost_{f}_faces'] = np.array(getattr(gc, f'ghost_{f}_indices'), np.int64).reshape(-1, 2)
                out[f'ghost_{f}_cells'] = np.array(getattr(gc, f'{f}_ip_cells'), np.int64).reshape(-1, 2)
                out[f'ghost_{f}_weights'] = np.asarray(getattr(gc, f'{f}_ip_weights'), float).reshape(-1, 4)
                out[f'ghost_{f}_gammas'] = np.asarray(getattr(gc, f'{f}_gammas'), float)
        out[f'{tag}_init_u'], out[f'{tag}_init_v'] = s.u.copy(), s.v.copy()
        fields, coef = {}, []
        for k in range(20):
            _, cd, cl = s.solve(n_steps=1, dt=0.002, perturb_transient=perturb, perturb_duration=0.03,
                                save_artifacts=False, verbose=False)
            coef.append([float(cd[0]), float(cl[0])])
            if k + 1 in (1, 5, 20):
                fields[k + 1] = (s.u.copy(), s.v.copy(), s.p.copy())
        for k, (u, v, p) in fields.items():
            out[f'{tag}_u{k}'], out[f'{tag}_v{k}'], out[f'{tag}_p{k}'] = u, v, p
        out[f'{tag}_coef'] = np.array(coef)
        out[f'{tag}_time'] = s.time
    save('legacy_ghost_48x24', **out)


def run_cutcell_legacy(work):
    """The reference's legacy cut-cell loop (MAC_CylinderFlow(boundary='cut_cell') with its
    default time_scheme='legacy': advance_momentum_predictor, compute_rhs, solve_pressure and
    apply_corrector of solver/cut_cell_solver.py, stepped by solver/main.py:297-333) on the
    40x20 cut-cell grid and on the 48x30 grid with rho = 1.3: centred transport (AB2 after an
    Euler first step) and upwind transport (forward Euler) with the transient inlet
    perturbation, 20 steps each; the initial field, fields at steps 1, 5 and 20, the force
    coefficients and the pressure record of every step, the predictor history after the last
    step, and an upwind momentum right-hand side on a seeded field."""
    from main import MAC_CylinderFlow
    out = {}
    for case, kw in CUTCELL_CASES.items():
        for tag, transport, perturb in (('centered', 'centered', False), ('upwind', 'upwind', True)):
            s = MAC_CylinderFlow(boundary='cut_cell', transport=transport, pressure_solver='direct', verbose=False,
                                 **kw)
            assert s.time_scheme == 'legacy'
            key = f'{case}_{tag}'
            out[f'{key}_init_u'], out[f'{key}_init_v'] = s.u.copy(), s.v.copy()
            if tag == 'upwind':
                rng = np.random.default_rng(7)
                fu = rng.standard_normal(s.u.shape)
                fv = rng.standard_normal(s.v.shape)
                fu[s.cut_geom.ax == 0] = 0.
                fv[s.cut_geom.ay == 0] = 0.
                a_u, a_v, r_u, r_v = s.cc.compute_momentum_rhs(fu, fv, s.nu, s.rho, transport='upwind')
                out[f'{case}_probe_u'], out[f'{case}_probe_v'] = fu, fv
                out[f'{case}_upwind_au'], out[f'{case}_upwind_av'] = a_u, a_v
                out[f'{case}_upwind_ru'], out[f'{case}_upwind_rv'] = r_u, r_v
            fields, coef, rec = {}, [], []
            for k in range(20):
                _, cd, cl = s.solve(n_steps=1, dt=0.002, perturb_transient=perturb, perturb_duration=0.03,
                                    save_artifacts=False, verbose=False)
                d = s.last_step_diagnostics
                coef.append([float(cd[0]), float(cl[0])])
                rec.append([d['residual_linf'], d['residual_l2'], d['predicted_divergence'], d['max_divergence'],
                            d['cfl']])
                if k + 1 in (1, 5, 20):
                    fields[k + 1] = (s.u.copy(), s.v.copy(), s.p.copy())
            for k, (u, v, p) in fields.items():
                out[f'{key}_u{k}'], out[f'{key}_v{k}'], out[f'{key}_p{k}'] = u, v, p
            out[f'{key}_coef'] = np.array(coef)
            out[f'{key}_record'] = np.array(rec)
            out[f'{key}_time'] = s.time
            out[f'{key}_prev_au'], out[f'{key}_prev_av'] = s.cc.prev_au.copy(), s.cc.prev_av.copy()
            out[f'{key}_prev_dt'] = s.cc.prev_dt
    save('cutcell_legacy', **out)


LEGACY_OPTION_CASES = {
    'staircase_slip_parabolic_upwind': dict(nx=48, ny=24, Lx=4.8, Ly=2.4, D=1.0, xc=1.3, yc=1.15, nu=0.02,
                                            boundary='staircase', transport='upwind', slip_walls=True,
                                            inflow='parabolic', U_m=1.2, pressure_solver='direct'),
    'ghost_parabolic_rho': dict(nx=48, ny=24, Lx=4.8, Ly=2.4, D=1.0, xc=1.3, yc=1.15, nu=0.02, rho=1.3,
                                boundary='ghost_cell', transport='centered', inflow='parabolic',
                                pressure_solver='direct'),
    'cutcell_slip_parabolic_cgdct': dict(nx=40, ny=20, Lx=4., Ly=2., D=1., xc=1.1, yc=0.95, nu=0.02,
                                         boundary='cut_cell', transport='upwind', slip_walls=True,
                                         inflow='parabolic', U_m=1.2, pressure_solver='cg_dct'),
}


def run_legacy_options(work):
    """The reference's legacy loop with its options (solver/main.py:40-240, 303-381): slip
    channel walls, parabolic inflow, rho != 1, upwind transport, the sparse-LU and cg_dct pressure
    solvers, on the staircase, ghost-cell and cut-cell branches;
    12 steps each from the loop's own initial field, with the transient inlet perturbation
    (which the reference applies to uniform inflow only)."""
    from main import MAC_CylinderFlow
    out = {}
    for tag, kw in LEGACY_OPTION_CASES.items():
        s = MAC_CylinderFlow(time_scheme='legacy', verbose=False, **kw)
        out[f'{tag}_init_u'], out[f'{tag}_init_v'] = s.u.copy(), s.v.copy()
        out[f'{tag}_inlet'] = s.u_inlet.copy()
        coef = []
        for k in range(12):
            _, cd, cl = s.solve(n_steps=1, dt=0.002, perturb_transient=True, perturb_duration=0.03,
                                save_artifacts=False, verbose=False)
            coef.append([float(cd[0]), float(cl[0])])
        out[f'{tag}_u'], out[f'{tag}_v'], out[f'{tag}_p'] = s.u.copy(), s.v.copy(), s.p.copy()
        out[f'{tag}_coef'] = np.array(coef)
    save('legacy_options', **out)


def run_legacy_wide(work):
    """The three legacy loops on the benched grid (bench.py workloads staircase_800x820_re100,
    legacy_ghost_800x820_re100, cutcell_legacy_800x820_re100: 800x820, 40D x 41D, Re 100,
    centred transport, the loops' own initial fields): three reference steps each, stored as
    2000 seeded sample values per field and step plus the field maxima and the force
    coefficients of every step."""
    from main import MAC_CylinderFlow
    kw = dict(nx=800, ny=820, Lx=40.0, Ly=41.0, D=1.0, xc=10.0, yc=20.5, nu=0.01)
    out = {}
    pick = np.random.default_rng(2)
    su = np.sort(pick.choice(820 * 801, 2000, replace=False))
    sv = np.sort(pick.choice(821 * 800, 2000, replace=False))
    sp_ = np.sort(pick.choice(820 * 800, 2000, replace=False))
    out.update(sample_u=su, sample_v=sv, sample_p=sp_)
    for tag, boundary in (('staircase', 'staircase'), ('ghost', 'ghost_cell'), ('cutcell', 'cut_cell')):
        s = MAC_CylinderFlow(boundary=boundary, time_scheme='legacy', transport='centered', pressure_solver='direct',
                             verbose=False, **kw)
        coef, us, vs, ps, mx = [], [], [], [], []
        for k in range(3):
            _, cd, cl = s.solve(n_steps=1, dt=0.002, perturb_transient=False, save_artifacts=False, verbose=False)
            coef.append([float(cd[0]), float(cl[0])])
            us.append(s.u.ravel()[su].copy())
            vs.append(s.v.ravel()[sv].copy())
            ps.append(s.p.ravel()[sp_].copy())
            mx.append([np.abs(s.u).max(), np.abs(s.v).max(), np.abs(s.p).max()])
        out[f'{tag}_coef'], out[f'{tag}_maxima'] = np.array(coef), np.array(mx)
        out[f'{tag}_u'], out[f'{tag}_v'], out[f'{tag}_p'] = np.array(us), np.array(vs), np.array(ps)
    save('legacy_wide_800x820', **out)


def run_cutcell_gate(work):
    """The benched cut-cell AB2/CN workload (800x820, Re 100, the seeded 1e-2 v perturbation of the
    projected initial state, as in run_cutcell_wide) stepped until the reference's CN momentum
    gate (solver/time_integration.py:100-104) raises: the momentum residual of every step, the
    step that raised and its message."""
    from main import MAC_CylinderFlow
    kw = dict(nx=800, ny=820, Lx=40.0, Ly=41.0, D=1.0, xc=10.0, yc=20.5, nu=0.01)
    s = MAC_CylinderFlow(boundary='cut_cell', time_scheme='ab2_cn', pressure_solver='direct', verbose=False, **kw)
    g = s.cut_geom
    active_u, active_v = g.ax[:, 1:] > 0, g.ay[1:-1, :] > 0
    nu_active = int(active_u.sum())
    q = np.r_[s.u[:, 1:][active_u], s.v[1:-1][active_v]]
    q[nu_active:] += 1e-2 * np.random.default_rng(0).standard_normal(q.size - nu_active)
    s.u[:, 1:][active_u] = q[:nu_active]
    s.v[1:-1][active_v] = q[nu_active:]
    residuals, its, raised, message = [], [], -1, ''
    for k in range(120):
        try:
            s.solve(n_steps=1, dt=.002, perturb_transient=False, save_artifacts=False, verbose=False)
        except RuntimeError as e:
            raised, message = k + 1, str(e)
            break
        d = s.last_step_diagnostics
        residuals.append(d['momentum_residual_linf'])
        its.append(d['momentum_iterations'])
    save('cutcell_gate_800x820', residuals=np.array(residuals), iterations=np.array(its), raised=raised,
         message=np.array(message))


def run_modal(work):
    """The reference's snapshot POD (postprocessing/modal_analysis.py) on a seeded synthetic wake:
    two travelling modes plus noise on a 24 x 40 grid, 30 snapshots."""
    from postprocessing.modal_analysis import SnapshotPOD, compute_phase_portrait_metrics
    rng = np.random.default_rng(31)
    ny, nx, m = 24, 40, 30
    y, x = np.meshgrid(np.linspace(-1, 1, ny), np.linspace(0, 4, nx), indexing='ij')
    t = np.linspace(0, 6, m)
    snaps = np.array([0.3 + np.sin(2 * x - 1.7 * tt) * np.exp(-4 * y * y) + 0.4 * np.cos(3 * x - 3.4 * tt) * y
                      + 1e-3 * rng.standard_normal((ny, nx)) for tt in t])
    pod = SnapshotPOD(n_modes=6).fit(snaps)
    pp = compute_phase_portrait_metrics(pod.temporal_coeffs[0], pod.temporal_coeffs[1])
    save('modal', snapshots=snaps, mean_field=pod.mean_field, spatial_modes=pod.spatial_modes,
         temporal_coeffs=pod.temporal_coeffs, singular_values=pod.singular_values,
         modal_energies=pod.modal_energies, energy_ratios=pod.energy_ratios,
         cumulative_energy=pod.cumulative_energy, phase=np.array([pp['mean_amplitude'], pp['circularity_error']]))


def run_analysis(work):
    """postprocessing/analysis.py periodic_metrics on seeded synthetic force histories: a
    resolved, drifting shedding signal and an unresolved one."""
    from postprocessing.analysis import periodic_metrics
    rng = np.random.default_rng(4)
    t = np.linspace(0, 60, 3001)
    cl = 0.3 * (1 + 0.01 * t) * np.sin(2 * np.pi * 0.17 * t + 0.3) + 1e-3 * rng.standard_normal(t.size)
    cd = 1.3 + 0.02 * np.sin(4 * np.pi * 0.17 * t) + 1e-3 * rng.standard_normal(t.size)
    keys = None
    rows = []
    for (tt, a, b, ts) in ((t, cd, cl, 5.0), (t[:200], cd[:200], cl[:200] * 0 + 1e-3 * t[:200], 0.0)):
        m = periodic_metrics(tt, a, b, ts, D=1.0, U_ref=1.0)
        keys = sorted(m)
        rows.append([float(m[k]) for k in keys])
    # calculate_gci (postprocessing/analysis.py:106-151): equal and unequal ratios, the
    # non-estimable branches
    from postprocessing.analysis import calculate_gci
    import json
    gci_cases = [(1.0, 1.04, 1.2, 2.0, 1.25, None), (1.0, 1.04, 1.2, 2.0, 1.25, 1.5), (1.0, 1.1, 1.05, 2.0, 1.25, None),
                 (2.0, 2.0, 2.0, 2.0, 1.25, None), (1.0, 1.001, 1.0021, 2.0, 3.0, None),
                 (0.5, 0.52, 0.53, 1.5, 1.25, 2.5), (1.0, 1.0000001, 1.0000002, 2.0, 1.25, None)]
    gci = [calculate_gci(*c[:3], r=c[3], Fs=c[4], r32=c[5]) for c in gci_cases]
    save('analysis', t=t, cd=cd, cl=cl, keys=np.array(keys), values=np.array(rows),
         gci_cases=json.dumps(gci_cases), gci=json.dumps(gci))


def run_taylor_green(work):
    """The reference's periodic Taylor-Green verification (verification/taylor_green.py:14-59):
    error norms, final velocity and pressure for two small grids."""
    sys.path.insert(0, str(work / 'verification'))
    import taylor_green
    out = {}
    for tag, (n, dt, end, nu) in {'n16': (16, .01, .05, .1), 'n32': (32, .0025, .1, .1)}.items():
        info, q, p = taylor_green.run(n, dt, end_time=end, nu=nu)
        out[f'{tag}_q'] = q
        out[f'{tag}_p'] = p
        out[f'{tag}_norms'] = np.array([info['velocity'][k] for k in ('l1', 'l2', 'linf')] +
                                       [info['pressure'][k] for k in ('l1', 'l2', 'linf')] +
                                       [info['max_divergence']])
        out[f'{tag}_params'] = np.array([n, dt, end, nu])
    save('taylor_green', **out)


def run_all(args):
    import scipy.sparse as sp
    from main import MAC_CylinderFlow
    import optimized_ghost_cell as ghost
    import rectangular_inverse
    import mac_engine

    # 1. the reference's own small test grid (tests/test_numba_ghost_cell.py:12-14)
    def small(**kw):
        return MAC_CylinderFlow(nx=88, ny=16, Lx=22., Ly=4.1, xc=2., yc=2., boundary='ghost_cell',
                                time_scheme='ab2_cn', verbose=False, **kw)

    s = small()
    g = s.gg
    rng = np.random.default_rng(6)
    q = rng.normal(size=g.qsize)
    p_rand = rng.normal(size=s.p.shape)
    adv = g.advection(q).copy()
    dif = g.diffusion(q).copy()
    grad = g.gradient(p_rand).copy()
    div = g.divergence(q).copy()
    hq = g.H_matvec(q, 0.003).copy()
    uu, vv = g.unpack(q)
    uu, vv = uu.copy(), vv.copy()
    proj, phi = g.project(q, .003)
    proj, phi = proj.copy(), phi.copy()
    rhs_p = rng.normal(size=len(g.pi))
    sol_p = g.pressure_solve(rhs_p).copy()
    jp, ip = np.unravel_index(g.pi, s.p.shape)
    rect_p = rectangular_inverse.rectangle(s.nx, s.ny, s.dx, s.dy, 'pressure', rho=s.rho)[0]
    rows_p = schur_rows_of(g.A, g.pi, rect_p)
    nq = len(g.ui)
    dt_h = 0.001
    ju, iu = np.unravel_index(g.ui, s.u.shape)
    jv, iv = np.unravel_index(g.vi, s.v.shape)
    rect_u = rectangular_inverse.rectangle(s.nx, s.ny, s.dx, s.dy, 'u', s.nu, dt_h, s.rho)[0]
    rect_v = rectangular_inverse.rectangle(s.nx, s.ny, s.dx, s.dy, 'v', s.nu, dt_h, s.rho)[0]
    act_u = (sp.eye(nq, format='csc') - .5 * dt_h * g.L[:nq, :nq]).tocsc()
    act_v = (sp.eye(g.qsize - nq, format='csc') - .5 * dt_h * g.L[nq:, nq:]).tocsc()
    rows_u = schur_rows_of(act_u, ju * s.nx + iu - 1, rect_u)
    rows_v = schur_rows_of(act_v, (jv - 1) * s.nx + iv, rect_v)
    geo = geometry_record(s)
    init_u, init_v = s.u.copy(), s.v.copy()
    steps = []
    for k in range(5):
        s.solve(n_steps=1, dt=.001, perturb_transient=False, save_artifacts=False, verbose=False)
        d = s.last_step_diagnostics
        steps.append((s.u.copy(), s.v.copy(), s.p.copy(), d['cd'], d['cl'], d['max_divergence'], d['cfl'],
                      d['cd_pressure'], d['cd_viscous'], d['cl_pressure'], d['cl_viscous'],
                      d['coupled_momentum_residual_linf'], d['momentum_residual_linf']))
    forces = g.surface_forces(s.u, s.v, s.p, s.nu * s.rho)
    stats = mac_engine.calculate_mac_divergence_cpp(s.u, s.v, s.mask, s.dx, s.dy)
    save('small_88x16', q=q, p_rand=p_rand, advection=adv, diffusion=dif, gradient=grad, divergence=div,
         H_q=hq, unpack_u=uu, unpack_v=vv, project_q=proj, project_phi=phi, rhs_p=rhs_p, sol_p=sol_p,
         schur_rows_p=rows_p, schur_rows_u=rows_u, schur_rows_v=rows_v, helmholtz_dt=dt_h, **geo,
         init_u=init_u, init_v=init_v,
         step_u=np.array([t[0] for t in steps]), step_v=np.array([t[1] for t in steps]),
         step_p=np.array([t[2] for t in steps]), step_scalars=np.array([t[3:] for t in steps]),
         forces=np.array(forces), mac_divergence=np.array(stats[:1] + stats[1:2] + stats[3:4]),
         mac_divergence_counts=np.array([stats[2], stats[4]]),
         surface_points=g.surface_points, pressure_surface=csr_parts(g.pressure_surface),
         du_dn=csr_parts(g.du_dn), dv_dn=csr_parts(g.dv_dn))

    # 2. the 40x30 grid with the extension options (tests/test_gemini_followup.py:24-26,64-66)
    for tag, opts in (('bq', dict(ghost_velocity_interpolation='biquadratic')),
                      ('qp', dict(ghost_pressure_extension='quadratic')),
                      ('iter', dict(pressure_solver='iterative'))):
        s = MAC_CylinderFlow(nx=40, ny=30, Lx=4., Ly=3., xc=1.5, yc=1.5, boundary='ghost_cell',
                             time_scheme='ab2_cn', verbose=False, **opts)
        geo = geometry_record(s)
        s.solve(n_steps=3, dt=.001, perturb_transient=False, save_artifacts=False, verbose=False)
        d = s.last_step_diagnostics
        save(f'opt40x30_{tag}', **geo, u=s.u, v=s.v, p=s.p,
             scalars=np.array([d['cd'], d['cl'], d['max_divergence'], d['pressure_iterations']]))

    # 3. analytic traction fields (tests/test_numba_ghost_cell.py:49-69)
    out = []
    for nx, ny in ((40, 30), (80, 60), (120, 90)):
        s = MAC_CylinderFlow(nx=nx, ny=ny, Lx=4., Ly=3., xc=1.5, yc=1.5, boundary='ghost_cell',
                             time_scheme='ab2_cn', verbose=False)
        gc, g = s.gc, s.gg
        xx, yy = np.meshgrid(gc.xu, gc.yu)
        rr = np.hypot(xx - s.xc, yy - s.yc)
        u = -(rr - s.D / 2) * (yy - s.yc) / rr
        xx, yy = np.meshgrid(gc.xv, gc.yv)
        rr = np.hypot(xx - s.xc, yy - s.yc)
        v = (rr - s.D / 2) * (xx - s.xc) / rr
        p = np.broadcast_to(gc.xp, s.p.shape)
        out.append(g.surface_forces(u, v, p, s.nu * s.rho))
    save('traction', forces=np.array(out))

    # 4. rectangle transforms on a small grid (solver/rectangular_inverse.py)
    rec = {}
    for kind in ('pressure', 'u', 'v'):
        _, solve, shape = rectangular_inverse.rectangle(24, 10, 0.3, 0.25, kind, 0.02, 0.004, 1.3)
        b = np.random.default_rng(3).normal(size=shape)
        rec[f'{kind}_in'] = b
        rec[f'{kind}_out'] = solve(b.copy())
    save('rectangle_24x10', **rec)

    if args.skip_large:
        return
    # 5. the 400x200 Re=40 case with seeded noise, two steps (config of the plain FP64 method)
    s = MAC_CylinderFlow(nx=400, ny=200, Lx=20., Ly=10., D=1., xc=5., yc=5., nu=1 / 40, rho=1., U_inf=1.,
                         inflow='uniform', boundary='ghost_cell', time_scheme='ab2_cn',
                         pressure_solver='direct', verbose=False)
    g = s.gg
    q = g.pack(s.u, s.v).copy()
    q += 1e-3 * np.random.default_rng(0).standard_normal(q.size)
    u0, v0 = g.unpack(q)
    s.u[:], s.v[:] = u0, v0
    geo = geometry_record(s)
    pick = np.random.default_rng(1)
    su = np.sort(pick.choice(s.u.size, 4000, replace=False))
    sv = np.sort(pick.choice(s.v.size, 4000, replace=False))
    spp = np.sort(pick.choice(s.p.size, 4000, replace=False))
    scal, fields = [], []
    for k in range(2):
        s.solve(n_steps=1, dt=.002, perturb_transient=False, save_artifacts=False, verbose=False)
        d = s.last_step_diagnostics
        scal.append([d['cd'], d['cl'], d['max_divergence'], d['cfl'], d['cd_pressure'], d['cd_viscous']])
        fields.append((s.u.ravel()[su].copy(), s.v.ravel()[sv].copy(), s.p.ravel()[spp].copy(),
                       np.abs(s.u).max(), np.abs(s.v).max(), np.abs(s.p).max(),
                       float(np.sqrt(np.mean(s.u ** 2))), float(np.sqrt(np.mean(s.v ** 2))),
                       float(np.sqrt(np.mean(s.p ** 2)))))
    save('config1_400x200', active_u=np.packbits(g.E[:s.u.size].getnnz(axis=1) > 0),
         ui_count=len(g.ui), vi_count=len(g.vi), pi_count=len(g.pi),
         Eu=geo['Eu'], Ev=geo['Ev'], P=geo['P'],
         ui=np.packbits(np.isin(np.arange(s.u.size), g.ui)), vi=np.packbits(np.isin(np.arange(s.v.size), g.vi)),
         pi=np.packbits(np.isin(np.arange(s.p.size), g.pi)),
         sample_u=su, sample_v=sv, sample_p=spp,
         u_samples=np.array([f[0] for f in fields]), v_samples=np.array([f[1] for f in fields]),
         p_samples=np.array([f[2] for f in fields]), norms=np.array([f[3:] for f in fields]),
         scalars=np.array(scal), pressure_rank=g.pressure_inverse_info['rank'],
         helmholtz_ranks=np.array([i['rank'] for i in g.helmholtz_inverse_info]))


if __name__ == '__main__':
    main()
