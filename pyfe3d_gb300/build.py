"""Build the CUDA library ``libfe3d_gb300.so`` in-tree for sm_103a.

Every translation unit in ``csrc/`` is compiled in parallel with nvcc and
linked into one shared library with a plain C ABI (``include/fe3d_gb300.h``)
that the Python layer loads with ctypes.

    python -m pyfe3d_gb300.build
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, 'csrc')
INCLUDE = os.path.join(ROOT, 'include')
OBJDIR = os.path.join(HERE, '_build')
LIB = os.path.join(HERE, 'libfe3d_gb300.so')
ARCH = ['-gencode', 'arch=compute_103a,code=sm_103a']
NVCC_FLAGS = ['-O3', '-lineinfo', '-std=c++17', '-Xcompiler', '-fPIC', '--expt-relaxed-constexpr',
              '-I' + INCLUDE, '-I' + CSRC]


def nvcc():
    exe = shutil.which('nvcc')
    if exe is None:
        cand = '/usr/local/cuda/bin/nvcc'
        if os.path.exists(cand):
            return cand
        raise RuntimeError('nvcc not found')
    return exe


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith('.cu'))


def _compile(src, verbose):
    obj = os.path.join(OBJDIR, os.path.basename(src)[:-3] + '.o')
    deps = [src] + [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(('.cuh', '.h'))]
    deps.append(os.path.join(INCLUDE, 'fe3d_gb300.h'))
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(d) for d in deps):
        return obj, ''
    cmd = [nvcc()] + ARCH + NVCC_FLAGS + ['-c', src, '-o', obj]
    if verbose:
        cmd.insert(1, '-Xptxas=-v')
    out = subprocess.run(cmd, capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError('nvcc failed for %s:\n%s%s' % (src, out.stdout, out.stderr))
    return obj, out.stdout + out.stderr


def build(verbose=False, force=False):
    """Compile csrc/*.cu and link libfe3d_gb300.so; returns the library path."""
    os.makedirs(OBJDIR, exist_ok=True)
    if force:
        for f in os.listdir(OBJDIR):
            os.remove(os.path.join(OBJDIR, f))
    srcs = sources()
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        results = list(ex.map(lambda s: _compile(s, verbose), srcs))
    objs = [r[0] for r in results]
    if verbose:
        for _, log in results:
            if log:
                print(log)
    if (not os.path.exists(LIB)) or max(os.path.getmtime(o) for o in objs) > os.path.getmtime(LIB):
        cmd = [nvcc()] + ARCH + ['-shared', '-o', LIB] + objs + ['-lcudart']
        out = subprocess.run(cmd, capture_output=True, text=True)
        if out.returncode != 0:
            raise RuntimeError('link failed:\n' + out.stdout + out.stderr)
    return LIB


if __name__ == '__main__':
    print(build(verbose='-v' in sys.argv, force='-f' in sys.argv))
