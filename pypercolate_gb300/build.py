"""Builds libnzgb300.so in-tree with nvcc for sm_103a (GB300).

Each .cu translation unit compiles in parallel; the objects are linked into
one shared library next to this file (``_lib/libnzgb300.so``).
"""
import concurrent.futures
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, 'csrc')
OUT_DIR = os.path.join(HERE, '_lib')
LIB = os.path.join(OUT_DIR, 'libnzgb300.so')
SOURCES = ['nz_uf.cu', 'nz_lattice.cu', 'nz_canonical.cu', 'nz_conv_tc.cu', 'nz_api.cu', 'nz_noalloc.cu',
           'nz_mix.cu', 'nz_mlp.cu']
ARCH = ['-gencode', 'arch=compute_103a,code=sm_103a']
FLAGS = ['-O3', '-lineinfo', '-std=c++17', '-Xcompiler', '-fPIC', '-Xcompiler', '-Wall',
         '-Xcompiler', '-Wno-unknown-pragmas',
         '--expt-relaxed-constexpr']


def nvcc():
    exe = shutil.which('nvcc')
    if exe is None:
        cand = '/usr/local/cuda/bin/nvcc'
        if os.path.exists(cand):
            return cand
        raise RuntimeError('nvcc not found')
    return exe


def _deps():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files.append(os.path.join(os.path.dirname(HERE), 'include', 'nz_gb300.h'))
    files.append(os.path.abspath(__file__))
    return files


def up_to_date():
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(f) <= t for f in _deps())


def build(force=False, verbose=False, extra_flags=()):
    if not force and up_to_date():
        return LIB
    os.makedirs(os.path.join(OUT_DIR, 'obj'), exist_ok=True)
    cc = nvcc()

    def compile_one(src):
        obj = os.path.join(OUT_DIR, 'obj', src.replace('.cu', '.o'))
        cmd = [cc, *ARCH, *FLAGS, *extra_flags, '-c', os.path.join(CSRC, src), '-o', obj]
        if verbose:
            print(' '.join(cmd), flush=True)
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError('nvcc failed on %s:\n%s%s' % (src, res.stdout, res.stderr))
        if verbose and (res.stdout or res.stderr):
            print(res.stdout + res.stderr)
        return obj

    with concurrent.futures.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIB + '.tmp'
    cmd = [cc, *ARCH, '-shared', '-o', tmp, *objs, '-lcudart']
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError('link failed:\n%s%s' % (res.stdout, res.stderr))
    os.replace(tmp, LIB)
    return LIB


if __name__ == '__main__':
    print(build(force='--force' in sys.argv, verbose=True,
                extra_flags=['-Xptxas', '-v'] if '--ptxas' in sys.argv else []))
