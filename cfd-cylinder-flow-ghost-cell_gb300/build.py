"""Build libghostmac.so in place for sm_103a (GB300).

    python cfd-cylinder-flow-ghost-cell_gb300/build.py

The host setup (geometry.cpp) is compiled by g++ with -ffp-contract=off so that
classification and stencil indices come from plain IEEE operations; the CUDA
translation units are compiled by nvcc for sm_103a only.  Objects build in
parallel into _build/ next to this file.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
SRC = HERE / 'csrc'
OUT = HERE / 'libghostmac.so'
BUILD = HERE / '_build'
ARCH = ['-gencode', 'arch=compute_103a,code=sm_103a']


def _nvcc() -> str:
    for cand in (shutil.which('nvcc'), '/usr/local/cuda/bin/nvcc'):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError('nvcc not found')


def sources_newer_than(target: Path) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    deps = list(SRC.glob('*')) + [HERE.parent / 'include' / 'ghostmac.h', Path(__file__)]
    return any(p.stat().st_mtime > t for p in deps if p.is_file())


def build(force: bool = False, verbose: bool = False) -> Path:
    if not force and not sources_newer_than(OUT):
        return OUT
    nvcc = _nvcc()
    BUILD.mkdir(exist_ok=True)
    inc = ['-I', str(SRC), '-I', str(HERE.parent / 'include')]
    jobs = [
        (['g++', '-O2', '-std=c++17', '-fPIC', '-ffp-contract=off', *inc, '-c', str(SRC / 'geometry.cpp'),
          '-o', str(BUILD / 'geometry.o')]),
        ([nvcc, *ARCH, '-O3', '-std=c++17', '-lineinfo', '-Xcompiler', '-fPIC', *inc, '-c', str(SRC / 'kernels.cu'),
          '-o', str(BUILD / 'kernels.o')]),
        ([nvcc, *ARCH, '-O3', '-std=c++17', '-lineinfo', '-Xcompiler', '-fPIC', *inc, '-c', str(SRC / 'ghostmac.cu'),
          '-o', str(BUILD / 'ghostmac.o')]),
        ([nvcc, *ARCH, '-O3', '-std=c++17', '-lineinfo', '-Xcompiler', '-fPIC', *inc, '-c', str(SRC / 'noalloc.cu'),
          '-o', str(BUILD / 'noalloc.o')]),
        ([nvcc, *ARCH, '-O3', '-std=c++17', '-lineinfo', '-Xcompiler', '-fPIC', *inc, '-c', str(SRC / 'periodic.cu'),
          '-o', str(BUILD / 'periodic.o')]),
        ([nvcc, *ARCH, '-O3', '-std=c++17', '-lineinfo', '-Xcompiler', '-fPIC', *inc, '-c', str(SRC / 'unet.cu'),
          '-o', str(BUILD / 'unet.o')]),
        ([nvcc, *ARCH, '-O3', '-std=c++17', '-lineinfo', '-Xcompiler', '-fPIC', *inc, '-c', str(SRC / 'rowgemm.cu'),
          '-o', str(BUILD / 'rowgemm.o')]),
        ([nvcc, *ARCH, '-O3', '-std=c++17', '-lineinfo', '-Xcompiler', '-fPIC', *inc, '-c', str(SRC / 'modal.cu'),
          '-o', str(BUILD / 'modal.o')]),
        ([nvcc, *ARCH, '-O3', '-std=c++17', '-lineinfo', '-Xcompiler', '-fPIC', *inc, '-c', str(SRC / 'cutcell.cu'),
          '-o', str(BUILD / 'cutcell.o')]),
        # the legacy MAC kernels repeat the reference's arithmetic bit for bit: no FMA contraction
        ([nvcc, *ARCH, '-O3', '-std=c++17', '-lineinfo', '-fmad=false', '-Xcompiler', '-fPIC', *inc, '-c',
          str(SRC / 'legacy.cu'), '-o', str(BUILD / 'legacy.o')]),
    ]
    procs = [subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True) for cmd in jobs]
    failed = []
    for cmd, p in zip(jobs, procs):
        out, _ = p.communicate()
        if verbose and out:
            print(out)
        if p.returncode:
            failed.append((' '.join(cmd), out))
    if failed:
        raise RuntimeError('build failed:\n' + '\n'.join(f'{c}\n{o}' for c, o in failed))
    tmp = OUT.with_suffix('.so.tmp')
    link = [nvcc, *ARCH, '-shared', '-o', str(tmp), str(BUILD / 'geometry.o'), str(BUILD / 'kernels.o'),
            str(BUILD / 'ghostmac.o'), str(BUILD / 'noalloc.o'), str(BUILD / 'periodic.o'),
            str(BUILD / 'unet.o'), str(BUILD / 'rowgemm.o'), str(BUILD / 'legacy.o'), str(BUILD / 'modal.o'),
            str(BUILD / 'cutcell.o'), '-lcudart']
    r = subprocess.run(link, capture_output=True, text=True)
    if r.returncode:
        raise RuntimeError('link failed:\n' + r.stdout + r.stderr)
    os.replace(tmp, OUT)
    return OUT


if __name__ == '__main__':
    print(build(force='--force' in sys.argv, verbose=True))
