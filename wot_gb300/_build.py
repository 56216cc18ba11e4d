"""Build libwotg.so in-tree with nvcc for sm_103a.

Each ``csrc/*.cu`` is compiled to an object in parallel, then linked into
``wot_gb300/libwotg.so`` (static CUDA runtime, so the library loads without a
GPU or a toolkit on the library path). Rebuilds only when a source or header is
newer than the library.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, 'csrc')
BUILD = os.path.join(PKG, '_build')
LIB = os.path.join(PKG, 'libwotg.so')
ARCH = ['-gencode', 'arch=compute_103a,code=sm_103a']
NVCC_FLAGS = ['-O3', '-lineinfo', '-std=c++17', '-Xcompiler', '-fPIC', '--expt-relaxed-constexpr']


def nvcc() -> str:
    for cand in (os.environ.get('NVCC'), shutil.which('nvcc'), '/usr/local/cuda/bin/nvcc'):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError('nvcc not found: the CUDA toolkit is required to build libwotg')


def _sources():
    return sorted(glob.glob(os.path.join(CSRC, '*.cu')))


def _deps():
    return (_sources() + glob.glob(os.path.join(CSRC, '*.cuh'))
            + glob.glob(os.path.join(ROOT, 'include', '*.h')) + [os.path.abspath(__file__)])


def up_to_date() -> bool:
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(p) <= t for p in _deps())


def build(force: bool = False, verbose: bool = False, extra_flags=()) -> str:
    """Compile every CUDA source and link libwotg.so; returns its path."""
    if not force and up_to_date():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    cc = nvcc()
    objs = []

    def compile_one(src):
        obj = os.path.join(BUILD, os.path.basename(src).replace('.cu', '.o'))
        cmd = [cc, *ARCH, *NVCC_FLAGS, *extra_flags, '-I', os.path.join(ROOT, 'include'),
               '-c', src, '-o', obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError('nvcc failed on %s:\n%s\n%s' % (src, ' '.join(cmd), r.stderr))
        if verbose and r.stderr:
            print(r.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=max(1, min(8, os.cpu_count() or 1))) as ex:
        objs = list(ex.map(compile_one, _sources()))
    tmp = LIB + '.tmp'
    cmd = [cc, *ARCH, '-shared', '-o', tmp, *objs]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError('nvcc link failed:\n%s\n%s' % (' '.join(cmd), r.stderr))
    os.replace(tmp, LIB)
    return LIB


if __name__ == '__main__':
    import sys
    print(build(force='--force' in sys.argv, verbose=True,
                extra_flags=['-Xptxas', '-v'] if '--ptxas' in sys.argv else []))
