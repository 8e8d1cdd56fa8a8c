"""The FP32 mode converts between FP64 and FP32 with integer operations (kernels.cuh:
f64_to_f32i / f32_to_f64i) instead of the FP64-pipe cvt instructions.  The same functions are
__host__ __device__; this test builds tests/cvt_check.cu for the host with nvcc and checks
4.1 million values, including the edge cases (zeros, the FP32 normal range boundary, overflow,
Inf, NaN, exact halfway points)."""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def test_integer_conversions_round_like_ieee(tmp_path):
    nvcc = shutil.which('nvcc') or ('/usr/local/cuda/bin/nvcc' if Path('/usr/local/cuda/bin/nvcc').exists() else None)
    if nvcc is None:
        pytest.skip('nvcc not available')
    exe = tmp_path / 'cvt_check'
    subprocess.run([nvcc, '-std=c++17', '-I', str(ROOT / 'cfd-cylinder-flow-ghost-cell_gb300' / 'csrc'),
                    '-o', str(exe), str(ROOT / 'tests' / 'cvt_check.cu')], check=True, capture_output=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    assert 'bad 0' in out.stdout
