"""Benchmark of the ghost-cell MAC AB2/CN step on GB300: cell-updates/s.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--workload NAME]

One step = one AB2/CN time step of one cylinder case (momentum right-hand side,
two CN Helmholtz solves, two pressure projections with the FFT + boundary Schur
solver, force quadrature and the divergence/CFL gates), exactly the loop body of
MAC_CylinderFlow.solve for boundary='ghost_cell', time_scheme='ab2_cn'.
Synthetic seeded inputs: the reference case geometry with a seeded Gaussian
perturbation (no external data).

By default the step runs in the FP32 mode (FP32 inverses and stencils, FP64 refinement to the
reference's residual targets) and the line's `comparison` holds the plain FP64 step timed the
same way on the same GPU; --precision fp64 times the plain step alone.

Our arm prints one JSON line: device-timed throughput (CUDA events on the
library's stream, L2 flushed between timed steps), an end-to-end figure through
the public MAC_CylinderFlow.solve API with host arrays, the roofline of the
dominant kernel, the CPU baseline (the oracle port on this host) and the SM
clocks sampled during the timed region.  --impl reference times the CPU oracle
port of the reference algorithm on the host cores for the same workload.
Under torchrun each rank runs an independent replica (the case does not shard).

Other workloads (--workload) time one path alone on one GPU: the 64-case sweep, Taylor-Green,
the GMRES pressure path, the cut-cell AB2/CN path (cutcell_800x820_re100) and the three legacy
loops (staircase_800x820_re100, legacy_ghost_800x820_re100, cutcell_legacy_800x820_re100).
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

# The batch workload's graph runs many independent chains; let the CUDA runtime open its
# maximum of 32 hardware work queues for this process (the default 8 serialises the chains).
# It only takes effect before the CUDA context exists, i.e. before torch touches the GPU.
os.environ.setdefault('CUDA_DEVICE_MAX_CONNECTIONS', '32')

ROOT = Path(__file__).resolve().parent
METRIC = 'cell-updates/s at div<1e-10: FP32+refine/learned-PC vs plain FP64, same GB300'

WORKLOADS = {
    # 40D x 41D wide domain, cylinder at (10D, 20.5D), Re=100, seeded 1e-2 v perturbation
    'wide_800x820_re100': dict(nx=800, ny=820, Lx=40.0, Ly=41.0, D=1.0, xc=10.0, yc=20.5, nu=0.01, dt=0.002,
                               noise='v', amp=1e-2, seed=0),
    # 20D x 10D channel, cylinder at (5D, 5D), Re=40, seeded 1e-3 noise on u and v
    'channel_400x200_re40': dict(nx=400, ny=200, Lx=20.0, Ly=10.0, D=1.0, xc=5.0, yc=5.0, nu=1 / 40, dt=0.002,
                                 noise='uv', amp=1e-3, seed=0),
}
# 64 seeded cases in one CUDA graph per step: Re ~ U[40,200], D ~ U[0.8,1.2], grid drawn from
# {256x128, 400x200, 800x410} at h=0.05, centre (Lx/4, Ly/2) jittered by U[-0.5D,0.5D] per axis
BATCH_WORKLOADS = {
    'sweep64_batch': dict(batch=64, seed=0, dt=0.002, h=0.05, grids=((256, 128), (400, 200), (800, 410)),
                          re=(40.0, 200.0), diameter=(0.8, 1.2), jitter=0.5, amp=1e-3),
}
# periodic Taylor-Green vortex on [0, 2 pi]^2 (verification/taylor_green.py), nu = 0.01, dt = 1e-3,
# 1000 steps to t = 1 for the error check (the timed steps are --steps of them)
TG_WORKLOADS = {
    'taylor_green_1024': dict(n=1024, nu=0.01, dt=1e-3, end_time=1.0),
    'taylor_green_256': dict(n=256, nu=0.01, dt=1e-3, end_time=1.0),
}
# GMRES pressure path with the learned preconditioner (config 5): 1024x512 (h = 0.04), Re = 150,
# cylinder at (8D, 10.24D), dt = 0.0015; the network trains on the case's own first solves
GMRES_WORKLOADS = {
    'gmres_1024x512_re150': dict(nx=1024, ny=512, Lx=40.96, Ly=20.48, D=1.0, xc=8.0, yc=10.24, nu=1 / 150,
                                 dt=0.0015, noise='v', amp=1e-2, seed=0, record_steps=40, epochs=600),
}
# the cut-cell AB2/CN path (boundary='cut_cell') on the headline grid: same domain, Re = 100,
# seeded 1e-2 v perturbation; FP64 (the reference's precision), direct pressure
CUTCELL_WORKLOADS = {
    'cutcell_800x820_re100': dict(nx=800, ny=820, Lx=40.0, Ly=41.0, D=1.0, xc=10.0, yc=20.5, nu=0.01, dt=0.002,
                                  noise='v', amp=1e-2, seed=0),
}
# the legacy loops (time_scheme='legacy', centred transport with the loop's AB2 step) on the same
# grid and Re: the staircase branch, the ghost-cell branch (image-point ghost velocities) and the
# cut-cell branch (aperture-weighted predictor), from the loop's own initial field (uniform
# inflow, masked faces zero)
LEGACY_WORKLOADS = {
    'staircase_800x820_re100': dict(nx=800, ny=820, Lx=40.0, Ly=41.0, D=1.0, xc=10.0, yc=20.5, nu=0.01, dt=0.002,
                                    boundary='staircase'),
    'legacy_ghost_800x820_re100': dict(nx=800, ny=820, Lx=40.0, Ly=41.0, D=1.0, xc=10.0, yc=20.5, nu=0.01,
                                       dt=0.002, boundary='ghost_cell'),
    'cutcell_legacy_800x820_re100': dict(nx=800, ny=820, Lx=40.0, Ly=41.0, D=1.0, xc=10.0, yc=20.5, nu=0.01,
                                         dt=0.002, boundary='cut_cell'),
}
DEFAULT_WORKLOAD = 'wide_800x820_re100'
# FP64 instructions (dadd + dmul + dfma, thread level) per cell update of the plain FP64 step on
# the 800x820 case, and the measured FP64 instruction rate of a GB300 (independent FMA chains on
# every SM, profiles/gb300_rates.md); the count comes from the ncu capture in FP64_OPS_SOURCE.
FP64_OPS_PER_CELL_UPDATE = 424.4
FP64_OPS_SOURCE = 'profiles/fp64_instructions_wide_800x820.md'
FP64_INST_RATE = 499e9
# DRAM bytes (read + write) per launch of the dominant kernel class, averaged over the launches
# of one ncu --set full capture of the same command (the capture's file under profiles/ gives the
# command and the per-launch figures).  Within a step the working set stays in L2, so DRAM
# traffic is far below the algorithmic bytes.
DRAM_TRAFFIC = {
    # profiles/k_xpass_fp64_wide_800x820.md: the forward and inverse row passes of the first
    # Helmholtz solve, (768 + 1024 + 4608 + 1024) / 2
    ('wide_800x820_re100', 'fp64', 1): 3712.0,
    # profiles/fp32_mode_wide_800x820.md: the two row passes of the first sweep, (256 + 1024) / 2
    ('wide_800x820_re100', 'fp32', 1): 640.0,
    # profiles/k_residual_fp32_wide_800x820.md: the u, u and v Helmholtz residuals,
    # (7168 + 6656 + 12032) / 3
    ('wide_800x820_re100', 'fp32', 4): 8618.7,
}
KERNEL_CLASSES = {1: 'row transforms (k_xpass)', 2: 'column solves (k_ysolve, k_yband)',
                  3: 'momentum rhs (k_momentum, k_shadow)', 4: 'operator residual (k_residual)',
                  5: 'boundary term (k_band_first, k_band_gemv, k_band_fwd_solve)', 6: 'projection (k_divergence, k_project_update, k_set_inlet)',
                  7: 'defect / pressure output (k_defect, k_pressure_out)', 8: 'ghost rows (k_ghost)',
                  9: 'forces / maxima (k_forces, k_maxabs)', 10: 'gates and loop control',
                  11: 'Helmholtz Jacobi iterations (k_helm_jacobi)',
                  12: 'row transforms on the tensor cores (k_row_gemm)'}


def replica_step_ms(step_ms, world, device='cuda'):
    """Replicas only: every rank times its own case; the job's step time is the slowest rank's
    (max over ranks through the default process group when world > 1)."""
    if world <= 1:
        return step_ms
    import torch
    import torch.distributed as dist
    t = torch.tensor([step_ms], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def load_package():
    sys.path.insert(0, str(ROOT))
    import __graft_entry__ as ge
    return ge.load_package()


def peaks():
    p = ROOT / 'MEASURED_PEAKS.json'
    if p.exists():
        d = json.loads(p.read_text())
        return float(d['hbm_gbs']), 'measured'
    return 6800.0, 'fallback'


class ClockSampler:
    """nvidia-smi clocks and throttle reasons while the timed region runs."""

    def __init__(self, index=0):
        self.index = index
        self.rows = []
        self.proc = None

    def __enter__(self):
        q = ('clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,'
             'clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,'
             'clocks_event_reasons.sw_power_cap')
        try:
            self.proc = subprocess.Popen(['nvidia-smi', '-i', str(self.index), f'--query-gpu={q}',
                                          '--format=csv,noheader,nounits', '-lms', '50'],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except FileNotFoundError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(',')])

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm = [float(r[0]) for r in self.rows if len(r) >= 7 and r[0].replace('.', '').isdigit()]
        mx = [float(r[1]) for r in self.rows if len(r) >= 7 and r[1].replace('.', '').isdigit()]
        names = ['hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown', 'sw_power_cap']
        reasons = sorted({names[k] for r in self.rows if len(r) >= 7 for k in range(4) if r[3 + k] == 'Active'})
        return dict(sm_mhz=statistics.median(sm) if sm else None, sm_max_mhz=max(mx) if mx else None,
                    reasons=reasons, samples=len(sm))


def seeded_state(s, w):
    """Seeded Gaussian perturbation of the active faces (the reference has no noise API)."""
    rng = np.random.default_rng(w['seed'])
    integ = s.cc if hasattr(s, 'cc') else s.gg
    q = integ.pack(s.u, s.v)
    nu = len(integ.ui)
    if w['noise'] == 'uv':
        q += w['amp'] * rng.standard_normal(q.size)
    else:
        q[nu:] += w['amp'] * rng.standard_normal(q.size - nu)
    u, v = integ.unpack(q)
    s.u[:], s.v[:] = u, v


def sweep_draws(w, make):
    """The seeded cases of a batch workload: make(kw) builds one case from the constructor
    arguments and returns None for draws that violate the geometry checks (cylinder inside
    the domain, probes inside the grid); those are redrawn.  Yields (case, kw, Re, noise seed)."""
    rng = np.random.default_rng(w['seed'])
    made = 0
    while made < w['batch']:
        nx, ny = w['grids'][int(rng.integers(len(w['grids'])))]
        re = rng.uniform(*w['re'])
        d = rng.uniform(*w['diameter'])
        lx, ly = nx * w['h'], ny * w['h']
        xc = lx / 4 + rng.uniform(-w['jitter'], w['jitter']) * d
        yc = ly / 2 + rng.uniform(-w['jitter'], w['jitter']) * d
        kw = dict(nx=nx, ny=ny, Lx=lx, Ly=ly, D=d, xc=xc, yc=yc, nu=1.0 * d / re)
        s = make(kw)
        if s is None:
            continue
        made += 1
        yield s, kw, re, int(rng.integers(2 ** 31))


def sweep_cases(pkg, w, precision):
    """The batch workload's cases as MAC_CylinderFlow objects with their seeded perturbation."""
    def make(kw):
        try:
            return pkg.MAC_CylinderFlow(boundary='ghost_cell', time_scheme='ab2_cn', verbose=False, precision=precision, **kw)
        except ValueError:
            return None
    cases, params = [], []
    for s, kw, re, seed in sweep_draws(w, make):
        q = s.gg.pack(s.u, s.v)
        q += w['amp'] * np.random.default_rng(seed).standard_normal(q.size)
        u, v = s.gg.unpack(q)
        s.u[:], s.v[:] = u, v
        cases.append(s)
        params.append(dict(kw, Re=re))
    return cases, params


def oracle_batch_rate(w, seconds, workers):
    """Cell-updates/s of the CPU oracle port over a bounded sample of a batch workload: the
    workload's first cases (same draws and perturbations), one AB2/CN step each after the
    start-up step, until `seconds` of stepping have run.  Returns (rate, steps, cells, seconds)."""
    sys.path.insert(0, str(ROOT / 'oracle'))
    import ghost_oracle as go
    import scipy.fft
    def make(kw):
        try:
            return go.CylinderCase(**kw)
        except ValueError:
            return None
    cells = steps = 0
    el = 0.0
    with scipy.fft.set_workers(workers):
        for c, kw, _, seed in sweep_draws(w, make):
            q = c.ops.pack(c.u, c.v)
            q += w['amp'] * np.random.default_rng(seed).standard_normal(q.size)
            c.u, c.v = c.ops.unpack(q)
            c.solve(1, w['dt'])
            t0 = time.perf_counter()
            c.solve(1, w['dt'])
            el += time.perf_counter() - t0
            cells += kw['nx'] * kw['ny']
            steps += 1
            if el >= seconds:
                break
    return cells / el, steps, cells, el


def oracle_rate(w, steps, seconds, workers):
    """Cell-updates/s of the CPU oracle port of the reference algorithm (setup and the first,
    Helmholtz-building step excluded)."""
    sys.path.insert(0, str(ROOT / 'oracle'))
    import ghost_oracle as go
    import scipy.fft
    kw = {k: w[k] for k in ('nx', 'ny', 'Lx', 'Ly', 'D', 'xc', 'yc', 'nu')}
    with scipy.fft.set_workers(workers):
        c = go.CylinderCase(**kw)
        rng = np.random.default_rng(w['seed'])
        q = c.ops.pack(c.u, c.v)
        if w['noise'] == 'uv':
            q += w['amp'] * rng.standard_normal(q.size)
        else:
            q[len(c.ops.ui):] += w['amp'] * rng.standard_normal(q.size - len(c.ops.ui))
        c.u, c.v = c.ops.unpack(q)
        c.solve(1, w['dt'])
        done, t0 = 0, time.perf_counter()
        while done < steps and (time.perf_counter() - t0) < seconds:
            c.solve(1, w['dt'])
            done += 1
        el = time.perf_counter() - t0
    return w['nx'] * w['ny'] * done / el, done, el


def run_reference(args, w, rank):
    if rank != 0:
        return
    workers = os.cpu_count() or 1
    if args.workload in CUTCELL_WORKLOADS or args.workload in LEGACY_WORKLOADS:
        path = 'cut_cell' if args.workload in CUTCELL_WORKLOADS else args.workload.replace('_800x820_re100', '')
        print(json.dumps(dict(impl='reference', workload=args.workload, unavailable=(
            f'the reference\'s {path} loop runs from its own source tree, which this machine does not hold; '
            f'oracle/time_reference_stub.py --path {path} times it where the source is'))), flush=True)
        return
    if args.workload in TG_WORKLOADS:
        rate, done, el = oracle_tg_rate(w, 60.0)
        line = dict(metric=METRIC, value=rate, unit='cell-updates/s', n_gpus=args.gpus, steps=done,
                    warmup=args.warmup, ms_per_step=el / max(done, 1) * 1e3, higher_is_better=True, scaling='weak',
                    vs_baseline=None, dtype='f64', data='synthetic (analytic field)', impl='reference',
                    config=dict(workload=args.workload, grid=f"{w['n']}x{w['n']}", dt=w['dt'], precision='fp64'),
                    cpu_baseline=dict(value=rate, unit='cell-updates/s', cores=1, kind='port',
                                      sample=f'{done} Taylor-Green steps at n={w["n"]} (set-up excluded)'),
                    e2e=dict(value=rate, unit='cell-updates/s', h2d_bytes_per_step=0, d2h_bytes_per_step=0))
        print(json.dumps(line), flush=True)
        return
    if 'batch' in w:
        rate, done, cells, el = oracle_batch_rate(w, 60.0, workers)
        line = dict(metric=METRIC, value=rate, unit='cell-updates/s', n_gpus=args.gpus, steps=done,
                    warmup=args.warmup, ms_per_step=el / max(done, 1) * 1e3, higher_is_better=True, scaling='weak',
                    vs_baseline=None, dtype='f64', data='synthetic', impl='reference',
                    config=dict(workload=args.workload, cases=w['batch'], dt=w['dt'], precision='fp64'),
                    cpu_baseline=dict(value=rate, unit='cell-updates/s', cores=workers, kind='port',
                                      sample=f'one AB2/CN step (after the start-up step) of each of the first {done} '
                                             f'cases of {args.workload} ({cells} cells)'),
                    e2e=dict(value=rate, unit='cell-updates/s', h2d_bytes_per_step=0, d2h_bytes_per_step=0))
        print(json.dumps(line), flush=True)
        return
    # the oracle's first step (Helmholtz build) is the warm-up, taken inside oracle_rate
    rate, done, el = oracle_rate(w, args.steps, 120.0, workers)
    line = dict(metric=METRIC, value=rate, unit='cell-updates/s', n_gpus=args.gpus, steps=done, warmup=args.warmup,
                ms_per_step=el / max(done, 1) * 1e3, higher_is_better=True, scaling='weak', vs_baseline=None,
                dtype='f64', data='synthetic', impl='reference',
                config=dict(workload=args.workload, grid=f"{w['nx']}x{w['ny']}", dt=w['dt'], precision='fp64'),
                cpu_baseline=dict(value=rate, unit='cell-updates/s', cores=workers, kind='port',
                                  sample=f'{done} AB2/CN steps of {args.workload} after setup and the start-up step'),
                e2e=dict(value=rate, unit='cell-updates/s', h2d_bytes_per_step=0, d2h_bytes_per_step=0))
    print(json.dumps(line), flush=True)


def run_ours(args, w, rank, world):
    import torch
    pkg = load_package()
    L = pkg._lib
    dev = int(os.environ.get('LOCAL_RANK', 0))
    torch.cuda.set_device(dev)
    kw = {k: w[k] for k in ('nx', 'ny', 'Lx', 'Ly', 'D', 'xc', 'yc', 'nu')}
    dt = w['dt']
    cells = w['nx'] * w['ny']
    s = pkg.MAC_CylinderFlow(boundary='ghost_cell', time_scheme='ab2_cn', verbose=False, precision=args.precision, **kw)
    seeded_state(s, w)
    stream = torch.cuda.Stream()
    L.check(L.lib.gm_set_stream(s._h, C.c_void_p(stream.cuda_stream)), s._h)
    s._push()
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device='cuda')  # 256 MB > L2 (129 MB)

    def one_step(k):
        rc, diag = s.step_raw(dt, 1, first_index=k, start_time=s.time + 0.0)
        if rc != L.GM_OK:
            L.check(rc, s._h)
        s.time = diag[0].time
        return diag[0]

    # warm-up (also captures the step graphs)
    for k in range(max(args.warmup, 3)):
        one_step(k)
    # timed region: K steps in graph mode, each bracketed by CUDA events on the library stream,
    # L2 flushed (256 MB write) between timed steps
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    launches0 = L.lib.gm_kernel_launches()
    times, sweeps = [], []
    with ClockSampler(dev) as clocks:
        for k in range(args.steps):
            with torch.cuda.stream(stream):
                flush.zero_()
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
            d = one_step(k + 1)
            with torch.cuda.stream(stream):
                e1.record(stream)
            e1.synchronize()
            times.append(e0.elapsed_time(e1))
            sweeps.append((d.pressure_refinement_iterations, d.momentum_refinement_iterations))
            assert d.max_divergence < 1e-10
    torch.cuda.synchronize()
    launches = L.lib.gm_kernel_launches() - launches0
    step_ms = sum(times) / len(times)
    step_ms = replica_step_ms(step_ms, world)
    value = cells * world / (step_ms * 1e-3)
    # phase times of graph-replayed steps (timing events captured into the step graphs)
    os.environ['GHOSTMAC_PHASE_TIMING'] = '1'
    phases = []
    for k in range(5):
        with torch.cuda.stream(stream):
            flush.zero_()
        one_step(k + 1)
        if k >= 2:
            out = (C.c_double * 14)()
            L.lib.gm_phase_timing(s._h, out)
            phases.append(list(out))
    os.environ.pop('GHOSTMAC_PHASE_TIMING', None)
    # p1_sweep0_band_1..4: the boundary chain (row inverse of the C rows, Schur GEMV, band row
    # forward, band solve); with the fused chain kernel band_1 holds all four and 2..4 are empty
    phase_names = ['momentum', 'helmholtz_uv', 'projection_1', 'defect', 'projection_2', 'pressure_forces_gates',
                   'p1_sweep0_row_pass', 'p1_sweep0_column_solve', 'p1_sweep0_band_1', 'p1_sweep0_band_2',
                   'p1_sweep0_band_3', 'p1_sweep0_band_4', 'p1_sweep0_final_row_pass', 'p1_sweep0_residual']
    phase_ms = {n: float(np.mean([p[i] for p in phases])) for i, n in enumerate(phase_names)}
    # dominant kernel class: per-class CUDA-event time of one launch-by-launch step with the
    # refinement sweeps decided on the host (every launched kernel does work; this NVTX range
    # is what the profiles capture), then that class timed over min(K, 10) such steps with L2
    # flushed between them.  The library sums each launch's algorithmic bytes per class.
    os.environ['GHOSTMAC_HOST_REFINE'] = '1'
    per_class = {}
    torch.cuda.nvtx.range_push('kernel_classes')
    L.lib.gm_kernel_timing(0, 1, None, None, None)
    one_step(0)
    torch.cuda.nvtx.range_pop()
    for cls in KERNEL_CLASSES:
        tot, cnt, by = C.c_double(), C.c_int64(), C.c_double()
        L.lib.gm_kernel_timing(cls, 0, C.byref(tot), C.byref(cnt), C.byref(by))
        per_class[cls] = (tot.value, cnt.value, by.value)
    dominant = max(per_class, key=lambda c: per_class[c][0])
    L.lib.gm_kernel_timing(0, 1, None, None, None)
    for k in range(min(args.steps, 10)):
        with torch.cuda.stream(stream):
            flush.zero_()
        one_step(k + 1)
    tot, cnt, by = C.c_double(), C.c_int64(), C.c_double()
    L.lib.gm_kernel_timing(dominant, 0, C.byref(tot), C.byref(cnt), C.byref(by))
    L.lib.gm_kernel_timing(0, 0, None, None, None)
    os.environ.pop('GHOSTMAC_HOST_REFINE', None)
    # the headline metric compares this mode with the plain FP64 step on the same GPU:
    # time the plain FP64 case with the same protocol (graph mode, L2 flushed between steps)
    compare = None
    if args.precision == 'fp32' and not args.no_compare:
        s64 = pkg.MAC_CylinderFlow(boundary='ghost_cell', time_scheme='ab2_cn', verbose=False, precision='fp64', **kw)
        seeded_state(s64, w)
        L.check(L.lib.gm_set_stream(s64._h, C.c_void_p(stream.cuda_stream)), s64._h)
        s64._push()
        for k in range(max(args.warmup, 3)):
            rc, dg = s64.step_raw(dt, 1, first_index=k)
            L.check(rc, s64._h)
        t64 = []
        for k in range(args.steps):
            with torch.cuda.stream(stream):
                flush.zero_()
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
            rc, dg = s64.step_raw(dt, 1, first_index=k + 1)
            L.check(rc, s64._h)
            with torch.cuda.stream(stream):
                e1.record(stream)
            e1.synchronize()
            t64.append(e0.elapsed_time(e1))
        ms64 = sum(t64) / len(t64)
        # the bound of the plain FP64 step: its HBM roofline (880 algorithmic bytes per cell
        # update) and its FP64-pipe roofline (FP64 instructions per cell update counted by ncu,
        # against the measured FP64 instruction rate)
        peak_gbs, _ = peaks()
        fp64_gbs = 880.0 * cells / (ms64 * 1e-3) / 1e9
        fp64_ops = FP64_OPS_PER_CELL_UPDATE * cells / (ms64 * 1e-3)
        compare = dict(plain_fp64_value=cells / (ms64 * 1e-3), plain_fp64_ms_per_step=ms64,
                       speedup_vs_plain_fp64=ms64 / step_ms,
                       plain_fp64_step_roofline=dict(bound='fp64 pipe',
                                                     hbm=dict(algorithmic_bytes_per_cell_update=880,
                                                              achieved_gbs=fp64_gbs, peak_gbs=peak_gbs,
                                                              frac=fp64_gbs / peak_gbs),
                                                     fp64_pipe=dict(fp64_instructions_per_cell_update=FP64_OPS_PER_CELL_UPDATE,
                                                                    achieved_ginst_s=fp64_ops / 1e9,
                                                                    peak_ginst_s=FP64_INST_RATE / 1e9,
                                                                    frac=fp64_ops / FP64_INST_RATE,
                                                                    source=FP64_OPS_SOURCE)))
        del s64
    # roofline of the dominant kernel class: its launches' algorithmic bytes / their event time
    nx, ny = w['nx'], w['ny']
    mean_ms = tot.value / max(cnt.value, 1)
    bytes_per_launch = by.value / max(cnt.value, 1)
    peak, peak_kind = peaks()
    achieved = by.value / max(tot.value * 1e-3, 1e-12) / 1e9
    traffic = DRAM_TRAFFIC.get((args.workload, args.precision, dominant))
    # end to end through the public API with host numpy arrays: warm-up calls first (the
    # timing runs above leave the step graphs to be captured again), then K calls timed
    e2e_steps = max(1, min(args.steps, 20))
    for _ in range(max(args.warmup, 3)):
        s.solve(n_steps=1, dt=dt, perturb_transient=False, save_artifacts=False, verbose=False)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        s.solve(n_steps=1, dt=dt, perturb_transient=False, save_artifacts=False, verbose=False)
    e2e_s = (time.perf_counter() - t0) / e2e_steps
    state_bytes = 8 * (ny * (nx + 1) + (ny + 1) * nx + nx * ny)
    cpu = None
    if rank == 0 and not args.no_cpu:
        rate, done, el = oracle_rate(w, 50, 20.0, 1)
        cpu = dict(value=rate, unit='cell-updates/s', cores=1, kind='port',
                   sample=f'{done} AB2/CN steps of {args.workload} ({el:.1f} s) after setup and the start-up step')
    # config 4 beside the single case: the 64-case sweep in both precisions (after the
    # single-case figures, so that its gigabyte of state does not touch them)
    sweep = tgs = gms = ccs = None
    if args.precision == 'fp32' and not args.no_batch and world == 1:
        sweep = batch_summary(pkg, L, BATCH_WORKLOADS['sweep64_batch'], max(1, min(args.steps, 10)), args.warmup)
    # configs 2 and 5 beside it, so that one default run observes every configuration; the
    # batch's cases are released first (their graphs, streams and gigabyte of state), so the
    # host-driven Taylor-Green step is timed without them
    if args.precision == 'fp32' and not args.no_extra and world == 1:
        import gc
        gc.collect()
        import torch
        torch.cuda.synchronize()
        tgs = tg_summary(pkg, TG_WORKLOADS['taylor_green_1024'], max(1, min(args.steps, 50)))
        gms = gmres_summary(pkg, GMRES_WORKLOADS['gmres_1024x512_re150'], max(1, min(args.steps, 10)))
        ccs = cutcell_summary(pkg, CUTCELL_WORKLOADS['cutcell_800x820_re100'], max(1, min(args.steps, 20)))
    if rank == 0:
        line = dict(metric=METRIC, value=value, unit='cell-updates/s', n_gpus=world, steps=args.steps,
                    warmup=args.warmup, ms_per_step=step_ms, higher_is_better=True, scaling='weak',
                    vs_baseline=None, dtype='f64' if args.precision == 'fp64' else 'f32+f64-refine', data='synthetic',
                    config=dict(workload=args.workload, grid=f'{nx}x{ny}', dt=dt,
                                precision='fp64 plain' if args.precision == 'fp64' else 'fp32 inverses/stencils, fp64 refinement',
                                cases_per_gpu=1, parallelism='replicas', l2='flushed (256 MB write) between timed steps',
                                pressure='DCT/DST fast inverse + boundary Schur (direct)'),
                    roofline=dict(bound='hbm', achieved=achieved, peak=peak, unit='GB/s', frac=achieved / peak,
                                  traffic=traffic, kernel=KERNEL_CLASSES[dominant], peak_source=peak_kind,
                                  launches_timed=int(cnt.value), mean_launch_ms=mean_ms,
                                  bytes_per_launch=bytes_per_launch),
                    step_roofline=dict(algorithmic_bytes_per_cell_update=880, achieved_gbs=880.0 * cells / (step_ms * 1e-3) / 1e9),
                    cpu_baseline=cpu,
                    e2e=dict(value=cells / e2e_s, unit='cell-updates/s', h2d_bytes_per_step=state_bytes + 8 * ny,
                             d2h_bytes_per_step=state_bytes + C.sizeof(L.StepDiag)),
                    clocks=clocks.summary(), gpu_launches=int(launches), launches_before_timed=int(launches0),
                    refinement_sweeps_per_step=dict(pressure=float(np.mean([a for a, _ in sweeps])),
                                                    momentum=float(np.mean([b for _, b in sweeps]))),
                    kernel_class_ms_per_step={KERNEL_CLASSES[c]: v[0] for c, v in per_class.items() if v[1]},
                    graph_phase_ms=phase_ms, comparison=compare, sweep64_batch=sweep, taylor_green_1024=tgs,
                    gmres_1024x512_re150=gms, cutcell_800x820_re100=ccs)
        print(json.dumps(line), flush=True)


def oracle_tg_rate(w, seconds):
    """Cell-updates/s of the CPU oracle's Taylor-Green step (numpy/scipy, one thread per FFT
    call as scipy runs it) over a bounded number of steps after the start-up step."""
    sys.path.insert(0, str(ROOT / 'oracle'))
    import ghost_oracle as go
    n, dt = w['n'], w['dt']
    done, el = 0, 0.0
    k = 2
    while el < seconds and k <= 64:
        t0 = time.perf_counter()
        go.taylor_green_run(n, dt, end_time=k * dt, nu=w['nu'])
        el1 = time.perf_counter() - t0
        t0 = time.perf_counter()
        go.taylor_green_run(n, dt, end_time=(2 * k) * dt, nu=w['nu'])
        el2 = time.perf_counter() - t0
        done, el = k, max(el2 - el1, 1e-9)  # k more steps; set-up and start-up cancel
        k *= 2
    return n * n * done / el, done, el


def run_ours_tg(args, w, rank, world):
    """Periodic Taylor-Green step (config 2): K steps timed, and the full run to end_time in
    this precision and in FP64 for the error norms against the analytic solution."""
    import torch
    pkg = load_package()
    tg = pkg.taylor_green
    n, nu, dt = w['n'], w['nu'], w['dt']
    case = tg.TaylorGreen(n, nu, args.precision)
    q0, p0 = tg.exact(n, nu, 0.0)
    case.set_state(q0, p0)
    case.step(dt, max(args.warmup, 3))
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    launches0 = pkg._lib.lib.gm_kernel_launches()
    with ClockSampler(int(os.environ.get('LOCAL_RANK', 0))) as clocks:
        t0 = time.perf_counter()
        case.step(dt, args.steps)  # one call: the library synchronises its stream before returning
        el = time.perf_counter() - t0
    launches = pkg._lib.lib.gm_kernel_launches() - launches0
    case.close()
    step_ms = el * 1e3 / args.steps
    step_ms = replica_step_ms(step_ms, world)
    cells = n * n
    # end to end through taylor_green.run (host arrays in and out) to end_time, both precisions
    t0 = time.perf_counter()
    info, _, _ = tg.run(n, dt, w['end_time'], nu, args.precision)
    e2e_s = time.perf_counter() - t0
    steps_total = round(w['end_time'] / dt)
    info64 = info if args.precision == 'fp64' else tg.run(n, dt, w['end_time'], nu, 'fp64')[0]
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        rate, done, cel = oracle_tg_rate(w, 10.0)
        cpu = dict(value=rate, unit='cell-updates/s', cores=1, kind='port',
                   sample=f'{done} Taylor-Green steps at n={n} ({cel:.1f} s, set-up and start-up excluded)')
    if rank == 0:
        line = dict(metric=METRIC, value=cells * world / (step_ms * 1e-3), unit='cell-updates/s', n_gpus=world,
                    steps=args.steps, warmup=args.warmup, ms_per_step=step_ms, higher_is_better=True,
                    scaling='weak', vs_baseline=None,
                    dtype='f64' if args.precision == 'fp64' else 'f32+f64-refine', data='synthetic (analytic field)',
                    config=dict(workload=args.workload, grid=f'{n}x{n}', nu=nu, dt=dt,
                                precision=args.precision, parallelism='replicas',
                                timing='host wall clock around one synchronous K-step call',
                                l2='working set (fields and FFT scratch) near the L2 size; not flushed'),
                    roofline=None, cpu_baseline=cpu,
                    e2e=dict(value=cells * steps_total / e2e_s, unit='cell-updates/s',
                             h2d_bytes_per_step=8 * 3 * cells / steps_total, d2h_bytes_per_step=8 * 4 * cells / steps_total),
                    clocks=clocks.summary(), gpu_launches=int(launches),
                    taylor_green=dict(end_time=w['end_time'], steps=steps_total, errors=info,
                                      errors_fp64=info64))
        print(json.dumps(line), flush=True)


def run_ours_gmres(args, w, rank, world):
    """GMRES pressure path (pressure_solver='iterative'): K steps with the rectangle-preconditioned
    FGMRES, the same K steps with the learned network attached (trained on the solves of the
    first record_steps steps of the same case), and the direct FFT/Schur path from the same
    state; iterations per solve, time per step and the force-coefficient differences."""
    import torch
    pkg = load_package()
    learned = pkg.learned
    kw = {k: w[k] for k in ('nx', 'ny', 'Lx', 'Ly', 'D', 'xc', 'yc', 'nu')}
    dt, K = w['dt'], args.steps
    cells = w['nx'] * w['ny']

    def case(solver):
        s = pkg.MAC_CylinderFlow(boundary='ghost_cell', time_scheme='ab2_cn', verbose=False, precision=args.precision, pressure_solver=solver, **kw)
        seeded_state(s, w)
        return s

    def timed(s, n):
        its, solves = [], []
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for k in range(n):
            rc, d = s.step_raw(dt, 1, first_index=k + w['record_steps'])
            pkg._lib.check(rc, s._h)
            its.append(int(d[0].pressure_iterations))
            solves.append(int(d[0].pressure_solve_count))
            s.time = d[0].time
        torch.cuda.synchronize()
        el = time.perf_counter() - t0
        return el * 1e3 / n, its, solves, float(d[0].cd), float(d[0].cl)

    plain = case('iterative')
    rhs, sol = learned.record_pressure_pairs(plain, w['record_steps'], dt)
    x, y, mask = learned.training_set(plain, rhs, sol)
    weights = learned.UNetWeights(seed=1)
    t0 = time.perf_counter()
    hist = learned.train(weights, x, y, mask, epochs=w['epochs'], lr=2e-3, batch=4)
    train_s = time.perf_counter() - t0
    # the learned case repeats the recorded steps, then runs the timed steps with the network
    net_case = case('iterative')
    net_case.solve(n_steps=w['record_steps'], dt=dt, perturb_transient=False, save_artifacts=False, verbose=False)
    direct = case('direct')
    direct.solve(n_steps=w['record_steps'], dt=dt, perturb_transient=False, save_artifacts=False, verbose=False)
    launches0 = pkg._lib.lib.gm_kernel_launches()
    with ClockSampler(int(os.environ.get('LOCAL_RANK', 0))) as clocks:
        ms_plain, its_plain, n_plain, cd_plain, cl_plain = timed(plain, K)
    launches = pkg._lib.lib.gm_kernel_launches() - launches0
    # the same steps with the FGMRES control loop on the host (one read-back per Arnoldi step)
    os.environ['GHOSTMAC_GMRES_HOST'] = '1'
    ms_host, its_host, n_host, _, _ = timed(plain, K)
    os.environ.pop('GHOSTMAC_GMRES_HOST', None)
    pc = learned.LearnedPreconditioner(net_case, weights)
    ms_net, its_net, n_net, cd_net, cl_net = timed(net_case, K)
    pc.detach()
    ms_dir, _, _, cd_dir, cl_dir = timed(direct, K)
    if rank == 0:
        per = lambda its, ns: float(np.sum(its) / max(np.sum(ns), 1))
        line = dict(metric=METRIC, value=cells * world / (ms_plain * 1e-3), unit='cell-updates/s', n_gpus=world,
                    steps=K, warmup=w['record_steps'], ms_per_step=ms_plain, higher_is_better=True, scaling='weak',
                    vs_baseline=None, dtype='f64' if args.precision == 'fp64' else 'f32+f64-refine',
                    data='synthetic', config=dict(workload=args.workload, grid=f"{w['nx']}x{w['ny']}", dt=dt,
                                                  precision=args.precision, parallelism='replicas',
                                                  pressure='FGMRES(50), rectangle-preconditioned',
                                                  timing='host wall clock around each synchronous step'),
                    roofline=None, cpu_baseline=None,
                    e2e=dict(value=cells * world / (ms_plain * 1e-3), unit='cell-updates/s',
                             h2d_bytes_per_step=0, d2h_bytes_per_step=int(C.sizeof(pkg._lib.StepDiag))),
                    clocks=clocks.summary(), gpu_launches=int(launches),
                    gmres=dict(iterations_per_solve_plain=per(its_plain, n_plain),
                               iterations_per_solve_learned=per(its_net, n_net),
                               ms_per_step_plain=ms_plain, ms_per_step_learned=ms_net, ms_per_step_direct=ms_dir,
                               ms_per_step_plain_host_control=ms_host,
                               iterations_per_solve_plain_host_control=per(its_host, n_host),
                               control='device (graph: restart cycles as a WHILE node, Arnoldi steps as IF nodes)',
                               cd_rel_diff_plain_vs_direct=abs(cd_plain - cd_dir) / abs(cd_dir),
                               cd_rel_diff_learned_vs_direct=abs(cd_net - cd_dir) / abs(cd_dir),
                               cl_abs_diff_learned_vs_plain=abs(cl_net - cl_plain),
                               training_pairs=int(x.shape[0]), training_epochs=w['epochs'], training_s=train_s,
                               training_loss_ratio=hist[-1] / hist[0]))
        print(json.dumps(line), flush=True)


def tg_summary(pkg, w, steps):
    """Config 2 beside the single case: the periodic Taylor-Green step at 1024^2 in the FP32
    mode (K steps, one synchronous call) and its error norms at t = 1 in both precisions."""
    tg = pkg.taylor_green
    n, nu, dt = w['n'], w['nu'], w['dt']
    case = tg.TaylorGreen(n, nu, 'fp32')
    q0, p0 = tg.exact(n, nu, 0.0)
    case.set_state(q0, p0)
    case.step(dt, 3)
    t0 = time.perf_counter()
    case.step(dt, steps)
    ms = (time.perf_counter() - t0) * 1e3 / steps
    case.close()
    info32 = tg.run(n, dt, w['end_time'], nu, 'fp32')[0]
    info64 = tg.run(n, dt, w['end_time'], nu, 'fp64')[0]
    norms = lambda i: dict(velocity_l2=i['velocity']['l2'], velocity_linf=i['velocity']['linf'],
                           pressure_l2=i['pressure']['l2'], max_divergence=i['max_divergence'])
    return dict(workload='taylor_green_1024', value=n * n / (ms * 1e-3), unit='cell-updates/s', ms_per_step=ms,
                steps=steps, errors_at_t1_fp32=norms(info32), errors_at_t1_fp64=norms(info64))


def gmres_summary(pkg, w, steps):
    """Config 5 beside the single case: the 1024x512 case with pressure_solver='iterative'
    (FGMRES with device control, FP32 preconditioner) against the direct path from the same
    state; the learned network is left to its own workload (it trains for about 30 s)."""
    import torch
    kw = {k: w[k] for k in ('nx', 'ny', 'Lx', 'Ly', 'D', 'xc', 'yc', 'nu')}
    dt = w['dt']
    out = dict(workload='gmres_1024x512_re150', steps=steps)
    for solver in ('iterative', 'direct'):
        s = pkg.MAC_CylinderFlow(boundary='ghost_cell', time_scheme='ab2_cn', verbose=False, precision='fp32', pressure_solver=solver, **kw)
        seeded_state(s, w)
        s._push()
        its, nsol = 0, 0
        for k in range(3):
            rc, d = s.step_raw(dt, 1, first_index=k)
            pkg._lib.check(rc, s._h)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for k in range(steps):
            rc, d = s.step_raw(dt, 1, first_index=3 + k)
            pkg._lib.check(rc, s._h)
            its += int(d[0].pressure_iterations)
            nsol += int(d[0].pressure_solve_count)
        torch.cuda.synchronize()
        ms = (time.perf_counter() - t0) * 1e3 / steps
        out[solver] = dict(ms_per_step=ms, cell_updates_per_s=w['nx'] * w['ny'] / (ms * 1e-3),
                           max_divergence=float(d[0].max_divergence))
        if solver == 'iterative':
            out[solver]['krylov_iterations_per_solve'] = its / max(nsol, 1)
        del s
    return out


def cutcell_summary(pkg, w, steps):
    """The cut-cell AB2/CN path (boundary='cut_cell') on the 800x820 grid beside the ghost-cell
    headline: K steps after three warm-up steps (one call, the host reads each step's
    diagnostics), with the CN GMRES iterations and the step gates."""
    import torch
    kw = {k: w[k] for k in ('nx', 'ny', 'Lx', 'Ly', 'D', 'xc', 'yc', 'nu')}
    dt = w['dt']
    t0 = time.perf_counter()
    os.environ['GHOSTMAC_PHASE_TIMING'] = '1'  # nine event records inside each step graph
    try:
        s = pkg.MAC_CylinderFlow(boundary='cut_cell', time_scheme='ab2_cn', verbose=False, **kw)
    finally:
        os.environ.pop('GHOSTMAC_PHASE_TIMING', None)
    setup_s = time.perf_counter() - t0
    seeded_state(s, w)
    s._push()
    rc, d = s.step_raw(dt, 3, start_time=0.0)
    pkg.cutcell._check(rc, s._h)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    rc, d = s.step_raw(dt, steps, start_time=3 * dt)
    torch.cuda.synchronize()
    ms = (time.perf_counter() - t0) * 1e3 / steps
    pkg.cutcell._check(rc, s._h)
    its = [int(d[k].momentum_iterations) for k in range(steps)]
    ph = np.zeros(8)
    pkg.cutcell._check(pkg._lib.lib.gm_cc_phase_timing(s._h, pkg._lib.ptr(ph)), s._h)
    names = ('advection', 'startup_or_ab2_and_cn_rhs', 'cn_gmres', 'cn_residual_check', 'projection_1',
             'cn_action_and_defect', 'projection_2', 'outputs_and_forces')
    out = dict(workload='cutcell_800x820_re100', grid=f"{w['nx']}x{w['ny']}", precision='fp64', steps=steps,
               ms_per_step=ms, value=w['nx'] * w['ny'] / (ms * 1e-3), unit='cell-updates/s',
               cn_gmres_iterations_per_step=float(np.mean(its)), pressure_solves_per_step=int(d[steps - 1].pressure_solves),
               max_divergence=max(float(d[k].max_divergence) for k in range(steps)),
               cd=float(d[steps - 1].cd), cl=float(d[steps - 1].cl), setup_s=setup_s,
               schur_rank=int(s.cc.pressure_inverse_info['rank']),
               last_step_phase_ms=dict(zip(names, (float(x) for x in ph))))
    del s
    return out


def batch_summary(pkg, L, w, steps, warmup):
    """The 64-case sweep (config 4) timed beside the single-case workload: K batch steps of the
    FP32 mode and of the plain FP64 mode, each one call (one graph launch per step), the cases'
    state (about 1 GB) larger than L2.  Returns the summary the bench line carries."""
    import torch
    dt = w['dt']
    out = dict(workload='sweep64_batch', steps=steps)
    for prec in ('fp32', 'fp64'):
        t0 = time.perf_counter()
        cases, _ = sweep_cases(pkg, w, prec)
        setup_s = time.perf_counter() - t0
        cells = sum(c.nx * c.ny for c in cases)
        batch = pkg.CylinderBatch(cases)
        for c in cases:
            c._push()
        k = 0
        for _ in range(max(warmup, 3)):
            rc, diag, done = batch.step_raw(dt, 1, first_index=k)
            batch._check(rc)
            k += 1
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        rc, diag, done = batch.step_raw(dt, steps, first_index=k)
        torch.cuda.synchronize()
        ms = (time.perf_counter() - t0) * 1e3 / steps
        batch._check(rc)
        divs = [diag[i].max_divergence for i in range(len(cases) * steps)]
        assert max(divs) < 1e-10
        shapes, probe = batch.launch_shapes()
        out[prec] = dict(value=cells / (ms * 1e-3), unit='cell-updates/s', ms_per_step=ms, cases=len(cases),
                         cells_per_step=cells, max_divergence=max(divs), setup_s=setup_s,
                         launch_shapes=list(shapes), shape_probe_ms=[x for x in probe if x != -1.0][:6])
        batch.close()
        del batch, cases
    out['speedup_fp32_vs_plain_fp64'] = out['fp64']['ms_per_step'] / out['fp32']['ms_per_step']
    return out


def run_ours_batch(args, w, rank, world):
    """Batched sweep: all cases advance together, one graph launch per step."""
    import torch
    pkg = load_package()
    L = pkg._lib
    dev = int(os.environ.get('LOCAL_RANK', 0))
    torch.cuda.set_device(dev)
    dt = w['dt']
    t0 = time.perf_counter()
    cases, params = sweep_cases(pkg, w, args.precision)
    setup_s = time.perf_counter() - t0
    cells = sum(c.nx * c.ny for c in cases)
    batch = pkg.CylinderBatch(cases)
    for c in cases:
        c._push()

    def step(b, k, n=1):
        rc, diag, done = b.step_raw(dt, n, first_index=k)
        b._check(rc)
        for i, c in enumerate(b.cases):
            c.time = diag[i * n + n - 1].time
        return [diag[i * n + j] for i in range(len(b.cases)) for j in range(n)]

    def timed(b, k0):
        # K steps in one call: one graph launch per step, one status readback at the end; the
        # cases' state (about 1 GB) is far larger than L2, so no flush is needed between steps
        torch.cuda.synchronize()
        t_0 = time.perf_counter()
        d = step(b, k0, args.steps)
        return (time.perf_counter() - t_0) * 1e3 / args.steps, d

    for k in range(max(args.warmup, 3)):
        step(batch, k)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    launches0 = L.lib.gm_kernel_launches()
    with ClockSampler(dev) as clocks:
        step_ms, d = timed(batch, max(args.warmup, 3))
    divs = [x.max_divergence for x in d]
    sweeps = [x.pressure_refinement_iterations + x.momentum_refinement_iterations for x in d]
    launches = L.lib.gm_kernel_launches() - launches0
    assert max(divs) < 1e-10
    step_ms = replica_step_ms(step_ms, world)
    value = cells * world / (step_ms * 1e-3)
    # dominant kernel class (per-class event timing of one launch-by-launch batch step)
    per_class = {}
    os.environ['GHOSTMAC_HOST_REFINE'] = '1'
    L.lib.gm_kernel_timing(0, 1, None, None, None)
    step(batch, 0)
    for cls in KERNEL_CLASSES:
        tot, cnt, by = C.c_double(), C.c_int64(), C.c_double()
        L.lib.gm_kernel_timing(cls, 0, C.byref(tot), C.byref(cnt), C.byref(by))
        per_class[cls] = (tot.value, cnt.value, by.value)
    L.lib.gm_kernel_timing(0, 0, None, None, None)
    os.environ.pop('GHOSTMAC_HOST_REFINE', None)
    dominant = max(per_class, key=lambda c: per_class[c][0])
    tot, cnt, by = per_class[dominant]
    bytes_per_launch = by / max(cnt, 1)
    mean_ms = tot / max(cnt, 1)
    peak, peak_kind = peaks()
    achieved = by / max(tot * 1e-3, 1e-12) / 1e9
    compare = None
    if args.precision == 'fp32' and not args.no_compare:
        c64, _ = sweep_cases(pkg, w, 'fp64')
        b64 = pkg.CylinderBatch(c64)
        for c in c64:
            c._push()
        for k in range(max(args.warmup, 3)):
            step(b64, k)
        ms64, _ = timed(b64, max(args.warmup, 3))
        compare = dict(plain_fp64_value=cells / (ms64 * 1e-3), plain_fp64_ms_per_step=ms64,
                       speedup_vs_plain_fp64=ms64 / step_ms)
        b64.close()
        del c64
    # end to end through CylinderBatch.solve with host arrays (push + step + pull of every case)
    e2e_steps = max(1, min(args.steps, 5))
    torch.cuda.synchronize()
    t_0 = time.perf_counter()
    for _ in range(e2e_steps):
        batch.solve(1, dt=dt)
    e2e_s = (time.perf_counter() - t_0) / e2e_steps
    state_bytes = sum(8 * (c.ny * (c.nx + 1) + (c.ny + 1) * c.nx + c.nx * c.ny) for c in cases)
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        workers = os.cpu_count() or 1
        rate, done, ncell, el = oracle_batch_rate(w, 20.0, workers)
        cpu = dict(value=rate, unit='cell-updates/s', cores=workers, kind='port',
                   sample=f'one AB2/CN step (after the start-up step) of each of the first {done} cases '
                          f'({ncell} cells, {el:.1f} s)')
    if rank == 0:
        grids = {}
        for c in cases:
            grids[f'{c.nx}x{c.ny}'] = grids.get(f'{c.nx}x{c.ny}', 0) + 1
        line = dict(metric=METRIC, value=value, unit='cell-updates/s', n_gpus=world, steps=args.steps,
                    warmup=args.warmup, ms_per_step=step_ms, higher_is_better=True, scaling='weak',
                    vs_baseline=None, dtype='f64' if args.precision == 'fp64' else 'f32+f64-refine', data='synthetic',
                    config=dict(workload=args.workload, cases=len(cases), grids=grids, cells_per_step=cells, dt=dt,
                                precision='fp64 plain' if args.precision == 'fp64' else 'fp32 inverses/stencils, fp64 refinement',
                                cases_per_gpu=len(cases), parallelism='replicas', setup_s=setup_s,
                                l2='working set (all cases, about 1 GB) larger than L2; K steps timed on the host '
                                   'around one batch call (one graph launch per step, one status readback)',
                                pressure='DCT/DST fast inverse + boundary Schur (direct)'),
                    roofline=dict(bound='hbm', achieved=achieved, peak=peak, unit='GB/s', frac=achieved / peak,
                                  traffic=None, kernel=KERNEL_CLASSES[dominant], peak_source=peak_kind,
                                  launches_timed=int(cnt), mean_launch_ms=mean_ms, bytes_per_launch=bytes_per_launch),
                    step_roofline=dict(algorithmic_bytes_per_cell_update=880,
                                       achieved_gbs=880.0 * cells / (step_ms * 1e-3) / 1e9),
                    cpu_baseline=cpu,
                    e2e=dict(value=cells / e2e_s, unit='cell-updates/s', h2d_bytes_per_step=state_bytes,
                             d2h_bytes_per_step=state_bytes + len(cases) * C.sizeof(L.StepDiag)),
                    clocks=clocks.summary(), gpu_launches=int(launches), max_divergence=max(divs),
                    refinement_sweeps_per_case_step=float(np.mean(sweeps)),
                    kernel_class_ms_per_step={KERNEL_CLASSES[c]: v[0] for c, v in per_class.items() if v[1]},
                    comparison=compare)
        print(json.dumps(line), flush=True)
    batch.close()


def profile_step(args, w):
    """One single-case step launch by launch (every kernel a separate launch, the refinement
    sweeps gated on the device) inside the NVTX range "one_step", after the warm-up steps."""
    os.environ['GHOSTMAC_NO_GRAPHS'] = '1'
    import torch
    pkg = load_package()
    kw = {k: w[k] for k in ('nx', 'ny', 'Lx', 'Ly', 'D', 'xc', 'yc', 'nu')}
    s = pkg.MAC_CylinderFlow(boundary='ghost_cell', time_scheme='ab2_cn', verbose=False, precision=args.precision, **kw)
    seeded_state(s, w)
    s._push()
    for k in range(args.warmup):
        rc, d = s.step_raw(w['dt'], 1, first_index=k)
        pkg._lib.check(rc, s._h)
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_push('one_step')
    rc, d = s.step_raw(w['dt'], 1, first_index=args.warmup)
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_pop()
    pkg._lib.check(rc, s._h)
    print(json.dumps(dict(profile_step=args.workload, precision=args.precision, max_divergence=d[0].max_divergence,
                          pressure_sweeps=int(d[0].pressure_refinement_iterations))), flush=True)


def profile_cutcell_ops(args, w):
    """Profiling driver of the cut-cell path: its step graph holds conditional nodes, whose kernel
    nodes ncu does not profile, so the operator calls that launch the same kernels one by one run
    inside the NVTX range "one_step": one viscous and one advective momentum evaluation and one
    projection of the seeded state."""
    import torch
    pkg = load_package()
    kw = {k: w[k] for k in ('nx', 'ny', 'Lx', 'Ly', 'D', 'xc', 'yc', 'nu')}
    s = pkg.MAC_CylinderFlow(boundary='cut_cell', time_scheme='ab2_cn', verbose=False, **kw)
    seeded_state(s, w)
    q = s.cc.pack(s.u, s.v)
    for _ in range(args.warmup):
        s.cc.compute_momentum_rhs(s.u, s.v, s.nu, s.rho, include_advection=False)
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_push('one_step')
    s.cc.compute_momentum_rhs(s.u, s.v, s.nu, s.rho, include_advection=False)
    s.cc.compute_momentum_rhs(s.u, s.v, 0.0, s.rho, include_advection=True)
    s.cc.project(q, w['dt'])
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_pop()
    print(json.dumps(dict(profile_ops=args.workload)), flush=True)


def run_ours_cutcell(args, w, rank, world):
    """The cut-cell path alone: the cutcell_summary figures as one line (1 GPU)."""
    import torch
    pkg = load_package()
    torch.zeros(1, device='cuda')
    # at most 60 timed steps: on this workload the reference's own loop (and this one, at the
    # same step) raises the CN momentum gate at step 71 (residual 2.1e-10 over the 1e-10 budget)
    out = cutcell_summary(pkg, w, max(1, min(args.steps, 60)))
    if rank == 0:
        line = dict(metric='cell-updates/s at div<1e-10 (cut-cell AB2/CN)', value=out['value'], unit='cell-updates/s',
                    n_gpus=world, steps=out['steps'], warmup=3, ms_per_step=out['ms_per_step'],
                    higher_is_better=True, scaling='weak', vs_baseline=None, dtype='f64', data='synthetic',
                    config=dict(workload=args.workload, grid=out['grid'], dt=w['dt'], boundary='cut_cell'),
                    cutcell=out)
        print(json.dumps(line), flush=True)


def run_ours_legacy(args, w, rank, world):
    """A legacy loop alone (1 GPU): K steps of MAC_CylinderFlow(time_scheme='legacy') after W
    warm-up steps, one solve() call, wall clock between two device synchronisations (each step
    is a few library calls from the host and reads the forces back)."""
    import torch
    pkg = load_package()
    torch.zeros(1, device='cuda')
    kw = {k: w[k] for k in ('nx', 'ny', 'Lx', 'Ly', 'D', 'xc', 'yc', 'nu')}
    t0 = time.perf_counter()
    s = pkg.MAC_CylinderFlow(boundary=w['boundary'], time_scheme='legacy', transport='centered', verbose=False, **kw)
    setup_s = time.perf_counter() - t0
    s.solve(n_steps=args.warmup, dt=w['dt'], perturb_transient=False, save_artifacts=False, verbose=False)
    steps = max(1, min(args.steps, 500))
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_push('legacy_steps')  # for ncu --nvtx-include "legacy_steps/"
    t0 = time.perf_counter()
    s.solve(n_steps=steps, dt=w['dt'], perturb_transient=False, save_artifacts=False, verbose=False)
    torch.cuda.synchronize()
    el = time.perf_counter() - t0
    torch.cuda.nvtx.range_pop()
    ms = el * 1e3 / steps
    max_div = s.divergence_stats()[0]
    if rank == 0:
        extra = dict(ghost_faces=s.ghost_counts()) if w['boundary'] == 'ghost_cell' else {}
        line = dict(metric=f"cell-updates/s (legacy {w['boundary']} loop)", value=w['nx'] * w['ny'] / (ms * 1e-3),
                    unit='cell-updates/s', n_gpus=world, steps=steps, warmup=args.warmup, ms_per_step=ms,
                    higher_is_better=True, scaling='weak', vs_baseline=None, dtype='f64',
                    data='synthetic (uniform inflow start)',
                    config=dict(workload=args.workload, grid=f"{w['nx']}x{w['ny']}", dt=w['dt'],
                                boundary=w['boundary'], time_scheme='legacy', transport='centered'),
                    legacy=dict(setup_s=setup_s, max_divergence=max_div, cd=s.last_step_diagnostics['cd'],
                                cl=s.last_step_diagnostics['cl'],
                                pressure_residual_linf=s.last_step_diagnostics.get(
                                    'pressure_residual_linf', s.last_step_diagnostics.get('residual_linf')), **extra))
        print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument('--gpus', type=int, default=1)
    ap.add_argument('--steps', type=int, default=200)
    ap.add_argument('--warmup', type=int, default=3)
    ap.add_argument('--impl', choices=('ours', 'reference'), default='ours')
    ap.add_argument('--workload', choices=sorted(WORKLOADS) + sorted(BATCH_WORKLOADS) + sorted(TG_WORKLOADS) +
                    sorted(GMRES_WORKLOADS) + sorted(CUTCELL_WORKLOADS) + sorted(LEGACY_WORKLOADS),
                    default=DEFAULT_WORKLOAD)
    ap.add_argument('--no-cpu', action='store_true', help='skip the CPU baseline leg')
    ap.add_argument('--no-compare', action='store_true', help='skip timing the plain FP64 step beside the FP32 mode')
    ap.add_argument('--no-batch', action='store_true', help='skip timing the 64-case sweep beside the single case')
    ap.add_argument('--no-extra', action='store_true',
                    help='skip the Taylor-Green and GMRES summaries beside the single case')
    ap.add_argument('--precision', choices=('fp64', 'fp32'), default='fp32',
                    help='fp64: plain FP64 method; fp32: FP32 inverses and stencils with FP64 refinement')
    ap.add_argument('--profile-step', action='store_true',
                    help='profiling driver: W warm-up steps, then one launch-by-launch step inside the NVTX range '
                         '"one_step" (for ncu --nvtx-include "one_step/"), no timing')
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    w = (WORKLOADS.get(args.workload) or BATCH_WORKLOADS.get(args.workload) or TG_WORKLOADS.get(args.workload) or
         GMRES_WORKLOADS.get(args.workload) or CUTCELL_WORKLOADS.get(args.workload) or
         LEGACY_WORKLOADS[args.workload])
    world = int(os.environ.get('WORLD_SIZE', 1))
    rank = int(os.environ.get('RANK', 0))
    if args.impl == 'reference':
        run_reference(args, w, rank)
        return
    if args.profile_step:
        if args.workload in CUTCELL_WORKLOADS:
            profile_cutcell_ops(args, w)
        else:
            profile_step(args, w)
        return
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(int(os.environ.get('LOCAL_RANK', 0)))
        dist.init_process_group('nccl')
    if args.workload in BATCH_WORKLOADS:
        run_ours_batch(args, w, rank, world)
    elif args.workload in TG_WORKLOADS:
        run_ours_tg(args, w, rank, world)
    elif args.workload in GMRES_WORKLOADS:
        run_ours_gmres(args, w, rank, world)
    elif args.workload in CUTCELL_WORKLOADS:
        run_ours_cutcell(args, w, rank, world)
    elif args.workload in LEGACY_WORKLOADS:
        run_ours_legacy(args, w, rank, world)
    else:
        run_ours(args, w, rank, world)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == '__main__':
    main()
