"""In-tree build of the CUDA library ``kymatio_gb300/_lib/libkymatio_gb300.so``.

Every translation unit under ``kymatio_gb300/csrc`` is compiled in parallel
for sm_103a with nvcc, then linked into one shared library with a plain C
ABI (declared in ``include/kymatio_gb300.h``).  The library links the static
CUDA runtime and no torch symbols, so any host language can load it.

    python -m kymatio_gb300.build          # build if sources are newer
    python -m kymatio_gb300.build --force  # rebuild
"""
import argparse
import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, 'csrc')
OUT_DIR = os.path.join(PKG, '_lib')
LIB = os.path.join(OUT_DIR, 'libkymatio_gb300.so')
BUILD_DIR = os.path.join(PKG, '_build')

ARCH = ['-gencode', 'arch=compute_103a,code=sm_103a']
NVCC_FLAGS = ['-O3', '-lineinfo', '-std=c++17', '-Xcompiler', '-fPIC', '-Xcompiler', '-O2',
              '--expt-relaxed-constexpr', '-I' + os.path.join(ROOT, 'include')]


def nvcc_path():
    for cand in (os.environ.get('NVCC'), shutil.which('nvcc'), '/usr/local/cuda/bin/nvcc'):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError('nvcc not found: the CUDA toolkit is required to build kymatio_gb300')


def _sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith('.cu'))


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(('.cuh', '.h'))]
    hs.append(os.path.join(ROOT, 'include', 'kymatio_gb300.h'))
    return hs


def _digest(src):
    h = hashlib.sha1()
    for p in [src] + sorted(_headers()):
        with open(p, 'rb') as f:
            h.update(f.read())
    h.update(' '.join(ARCH + NVCC_FLAGS).encode())
    return h.hexdigest()[:16]


def _compile(src, force, verbose):
    obj = os.path.join(BUILD_DIR, os.path.basename(src)[:-3] + '.' + _digest(src) + '.o')
    if os.path.exists(obj) and not force:
        return obj
    cmd = [nvcc_path()] + ARCH + NVCC_FLAGS + ['-c', src, '-o', obj]
    if verbose:
        cmd.insert(1, '-Xptxas=-v')
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError('nvcc failed for %s:\n%s\n%s' % (src, r.stdout, r.stderr))
    if verbose:
        sys.stderr.write(r.stderr)
    return obj


def build(force=False, verbose=False, jobs=None):
    """Compile all sources (in parallel) and link the shared library."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    os.makedirs(OUT_DIR, exist_ok=True)
    srcs = _sources()
    jobs = jobs or min(len(srcs), os.cpu_count() or 4)
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        objs = list(ex.map(lambda s: _compile(s, force, verbose), srcs))
    keep = set(objs)
    for f in os.listdir(BUILD_DIR):  # drop objects of older source versions
        p = os.path.join(BUILD_DIR, f)
        if f.endswith('.o') and p not in keep:
            os.remove(p)
    stamp = hashlib.sha1(''.join(objs).encode()).hexdigest()[:16]
    stamp_file = LIB + '.stamp'
    if (not force and os.path.exists(LIB) and os.path.exists(stamp_file)
            and open(stamp_file).read() == stamp):
        return LIB
    tmp = LIB + '.tmp'
    cmd = [nvcc_path()] + ARCH + ['-shared', '-o', tmp] + objs
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError('link failed:\n%s\n%s' % (r.stdout, r.stderr))
    os.replace(tmp, LIB)
    with open(stamp_file, 'w') as f:
        f.write(stamp)
    return LIB


if __name__ == '__main__':
    ap = argparse.ArgumentParser()
    ap.add_argument('--force', action='store_true')
    ap.add_argument('--verbose', action='store_true')
    a = ap.parse_args()
    print(build(force=a.force, verbose=a.verbose))
