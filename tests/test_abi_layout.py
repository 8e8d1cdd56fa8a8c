"""The ctypes structures of _lib.py against the C structs of include/ghostmac.h: a small C
program compiled with the host compiler prints sizeof and the offset of every field the ctypes
side declares, and each must equal the ctypes layout (a field missing from the C struct fails
the compile)."""
import ctypes as C
import shutil
import subprocess
from pathlib import Path

import pytest

from conftest import load_module

ROOT = Path(__file__).resolve().parents[1]
PAIRS = {
    'Config': 'gm_config', 'Sizes': 'gm_sizes', 'StepDiag': 'gm_step_diag', 'SolveInfo': 'gm_solve_info',
    'Csr': 'gm_csr', 'CcFaces': 'gm_cc_faces', 'CcConfig': 'gm_cc_config', 'CcStepDiag': 'gm_cc_step_diag',
    'LegacyState': 'gm_legacy_state', 'LegacyStepDiag': 'gm_legacy_step_diag',
}


def test_structures_match_the_header(tmp_path):
    cc = shutil.which('gcc') or shutil.which('cc')
    if cc is None:
        pytest.skip('no host C compiler')
    L = load_module('_lib')
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "include/ghostmac.h"', 'int main(void) {']
    expect = []
    for py, cname in PAIRS.items():
        cls = getattr(L, py)
        lines.append(f'  printf("%zu\\n", sizeof({cname}));')
        expect.append(C.sizeof(cls))
        for field in cls._fields_:
            name = field[0]
            lines.append(f'  printf("%zu\\n", offsetof({cname}, {name}));')
            expect.append(getattr(cls, name).offset)
    lines += ['  return 0;', '}']
    src = tmp_path / 'layout.c'
    src.write_text('\n'.join(lines) + '\n')
    exe = tmp_path / 'layout'
    subprocess.run([cc, '-std=c11', '-I', str(ROOT), '-o', str(exe), str(src)], check=True)
    got = [int(x) for x in subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()]
    assert got == expect
