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


def test_new_entry_points_reject_bad_arguments_without_a_device():
    """The legacy and ghost-cell entry points validate their arguments before any CUDA call:
    null handles, negative sizes and an empty ghost table give GM_EVALUE or GM_OK on any host."""
    L = load_module('_lib')
    lib = L.lib
    st = L.LegacyState()
    diag = (L.LegacyStepDiag * 1)()
    assert lib.gm_poisson_legacy_step(None, C.byref(st), 0.002, 1, diag, None) == L.GM_EVALUE
    assert lib.gm_cc_legacy_step(None, 0.002, 1, 0.0, 1, None) == L.GM_EVALUE
    assert lib.gm_mac_ghost_apply(None, 10, -1, None, None, None, None, None, None, 1, 0.0, None) == L.GM_EVALUE
    assert lib.gm_mac_ghost_apply(None, 10, 0, None, None, None, None, None, None, 0, 0.0, None) == L.GM_OK
    out = (C.c_double * 4)()
    assert lib.gm_mac_ghost_forces(None, None, None, 8, 8, 0.1, 0.1, 0.4, 0.4, 0.1, 360, 0.01, out, None) == \
        L.GM_EVALUE
    assert lib.gm_mac_ghost_correct(None, None, None, None, None, None, None, 8, 8, 0.1, 0.1, 0.002, 1.0, 0,
                                    None) == L.GM_EVALUE
