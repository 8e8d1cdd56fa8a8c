"""One explicit ghost-cell validation case on the GPU, with pressure telemetry and mean-wake
samples: the runner contract of validation/run_ghost_validation.py:19-102.

``run(config_path, output, restart=None)`` reads a case file (JSON: ``kind`` steady, periodic
or diagnostic; ``dt``, ``end_time``, ``sample_start``, optional ``profile_stride``, and the
``solver`` keywords of MAC_CylinderFlow), writes into a new directory:

* ``manifest.json`` -- the case, the restart file and its SHA-256, the run metadata and the
  SHA-256 of this runner, of the observables and of the analysis module;
* ``history.jsonl`` -- one JSON row per step: the step diagnostics, the step number, the
  front-minus-rear stagnation pressure ``delta_p`` and the wall time;
* ``centerline.bin`` / ``.json`` -- the CylinderSamples file;
* ``checkpoint.npz`` -- written every 45 s of wall time, at the end and after a failure;
* ``summary.json`` -- progress while running (atomically replaced), then the window
  statistics of C_D, C_L and delta_p, the periodic metrics of a periodic case (which needs 5
  complete cycles), and the run maxima of the divergence, CFL number and pressure residual;
* ``mean_observables.json`` -- the window means of the samples.

Restarting from a checkpoint requires the same solver configuration and a run that still
covers the whole sample window, as in the reference.  The pressure telemetry and the gates
are those of the library's step; the files follow the reference's layout so its campaign
tooling reads them unchanged.
"""
from __future__ import annotations

import argparse
import hashlib
import inspect
import json
import os
import time
from pathlib import Path

import numpy as np

from .analysis import periodic_metrics, window_statistics
from .ghost import MAC_CylinderFlow
from .observables import CylinderSamples, mean_observables

_HERE = Path(__file__).resolve().parent
CHECKPOINT_SECONDS = 45.0


def _sha256(path):
    return hashlib.sha256(Path(path).read_bytes()).hexdigest()


def MAC_configuration(options):
    """The full constructor configuration the options select (defaults filled in, verbose off),
    the form MAC_CylinderFlow.configuration takes."""
    bound = inspect.signature(MAC_CylinderFlow).bind(**options)
    bound.apply_defaults()
    config = dict(bound.arguments)
    config['verbose'] = False
    return config


def _check_case(case):
    dt, end, left = case['dt'], case['end_time'], case['sample_start']
    solver = case['solver']
    if (not np.isfinite([dt, end, left]).all() or dt <= 0 or not 0 <= left < end
            or case['kind'] not in ('steady', 'periodic', 'diagnostic')
            or solver.get('boundary') != 'ghost_cell' or solver.get('time_scheme') != 'ab2_cn'):
        raise ValueError('Invalid explicit Ghost validation case')
    return dt, end, left


def run(config_path, output, restart=None):
    case = json.loads(Path(config_path).read_text(encoding='utf-8'))
    dt, end, left = _check_case(case)
    output = Path(output)
    output.mkdir(parents=True, exist_ok=False)
    s = MAC_CylinderFlow.from_checkpoint(restart) if restart else MAC_CylinderFlow(**case['solver'])
    if s.configuration != MAC_configuration(case['solver']):
        raise ValueError('Restart/configuration mismatch')
    steps = round((end - s.time) / dt)
    if steps <= 0 or abs(s.time + steps * dt - end) > 1e-9 or left < s.time:
        raise ValueError('Window/end must be covered by this run at its declared timestep')
    initial_time = s.time
    samples = CylinderSamples(s, output / 'centerline.bin', stride=case.get('profile_stride', 10))
    samples.record(force=True)
    started = time.perf_counter()
    last_checkpoint = started
    count = 0
    maxima = dict(max_divergence=0., cfl=0., pressure_residual_linf=0.)
    manifest = dict(case=case, initial_time=initial_time, restart=str(restart) if restart else None,
                    restart_sha256=_sha256(restart) if restart else None,
                    metadata=s.metadata(dt, steps, perturb_transient=False),
                    runner_sha256=_sha256(__file__), observables_sha256=_sha256(_HERE / 'observables.py'),
                    analysis_sha256=_sha256(_HERE / 'analysis.py'), ram_stop_guard=False, ready_for_paper1=False)
    (output / 'manifest.json').write_text(json.dumps(manifest, indent=2), encoding='utf-8')

    def status(value):
        tmp = output / 'summary.tmp'
        tmp.write_text(json.dumps(value, indent=2, allow_nan=False), encoding='utf-8')
        os.replace(tmp, output / 'summary.json')

    with (output / 'history.jsonl').open('x', encoding='utf-8') as history:
        def observe(state, diagnostics):
            nonlocal last_checkpoint, count
            count += 1
            p = samples.pressures()
            row = dict(diagnostics, step=count, delta_p=float(p[0] - p[1]),
                       wall_seconds=time.perf_counter() - started)
            history.write(json.dumps(row, allow_nan=False) + '\n')
            for key in maxima:
                maxima[key] = max(maxima[key], float(row[key]))
            samples.record(pressures=p)
            if time.perf_counter() - last_checkpoint > CHECKPOINT_SECONDS:
                samples.flush()
                history.flush()
                state.save_checkpoint(output / 'checkpoint.npz', overwrite=True)
                last_checkpoint = time.perf_counter()
                status(dict(completed=False, steps=count, time=state.time,
                            seconds=time.perf_counter() - started, **maxima))
        try:
            s.solve(n_steps=steps, dt=dt, perturb_transient=False, save_artifacts=False, verbose=False,
                    step_callback=observe)
            samples.record(force=True)
            samples.close()
            history.flush()
            s.save_checkpoint(output / 'checkpoint.npz', overwrite=True)
        except BaseException as error:
            samples.close()
            history.flush()
            s.save_checkpoint(output / 'checkpoint.npz', overwrite=True)
            failed = dict(s.last_step_diagnostics)
            if failed.get('time') == s.time:
                for key in maxima:
                    if key in failed:
                        maxima[key] = max(maxima[key], float(failed[key]))
            status(dict(completed=False, steps=count, time=s.time, error=f'{type(error).__name__}: {error}',
                        last_step_diagnostics=failed, seconds=time.perf_counter() - started, **maxima))
            raise
    rows = [json.loads(line) for line in (output / 'history.jsonl').read_text(encoding='utf-8').splitlines()]
    t = np.array([r['time'] for r in rows])
    cd = np.array([r['cd'] for r in rows])
    cl = np.array([r['cl'] for r in rows])
    dp = np.array([r['delta_p'] for r in rows])
    window = [max(left, float(t[0])), float(t[-1])]
    periodic = None
    if case['kind'] == 'periodic':
        periodic = periodic_metrics(t, cd, cl, left, D=s.D, U_ref=s.U_ref)
        if periodic['cycles'] < 5:
            status(dict(completed=True, accepted=False, ready_for_paper1=False, steps=count,
                        reason='Insufficient complete cycles; no periodic mean-wake claim', **maxima))
            return
        window = [periodic['sample_start'], periodic['sample_end']]
    stats = window_statistics(t, np.column_stack((cd, cl, dp)), *window)
    mean = mean_observables(output / 'centerline.bin', *window)
    (output / 'mean_observables.json').write_text(json.dumps(mean, indent=2, allow_nan=False), encoding='utf-8')
    if periodic:
        periodic = {k: (None if isinstance(v, float) and not np.isfinite(v) else v) for k, v in periodic.items()}
    status(dict(completed=True, ready_for_paper1=False, steps=count, time=s.time,
                seconds=time.perf_counter() - started, statistics=stats, periodic=periodic,
                mean_flow_available=True, benchmark_accepted=False,
                acceptance_note='Reference-specific force, pressure, Lr, stationarity and domain checks are separate.',
                sample_window=window, **maxima))


def main(argv=None):
    ap = argparse.ArgumentParser(description='Run one explicit ghost-cell validation case on the GPU')
    ap.add_argument('config')
    ap.add_argument('output')
    ap.add_argument('--restart')
    args = ap.parse_args(argv)
    run(args.config, args.output, args.restart)


if __name__ == '__main__':
    main()
