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


CY_DIR = os.path.join(HERE, 'cy')
CY_CPP = os.path.join(OBJDIR, 'fe3d_cy.cpp')


def build_cython():
    """The Cython binding of the C ABI (``pyfe3d_gb300.fe3d_cy``): Cython -> C++
    where Cython is installed (the generated C++ is kept in the build folder),
    then g++ against the Python headers and libfe3d_gb300.so.  Returns the
    module path, or None when neither Cython nor generated C++ is there."""
    import sysconfig
    pyx = os.path.join(CY_DIR, 'fe3d_cy.pyx')
    os.makedirs(OBJDIR, exist_ok=True)
    try:
        import Cython  # noqa: F401
        have_cython = True
    except ImportError:
        have_cython = False
    deps = [pyx, os.path.join(CY_DIR, 'fe3d_gb300.pxd')]
    if have_cython and (not os.path.exists(CY_CPP) or
                        os.path.getmtime(CY_CPP) < max(os.path.getmtime(d) for d in deps)):
        cmd = [sys.executable, '-m', 'cython', '--cplus', '-3', '-I', CY_DIR, pyx, '-o', CY_CPP]
        out = subprocess.run(cmd, capture_output=True, text=True)
        if out.returncode != 0:
            raise RuntimeError('cython failed:\n' + out.stdout + out.stderr)
    if not os.path.exists(CY_CPP):
        return None
    mod = os.path.join(HERE, 'fe3d_cy' + (sysconfig.get_config_var('EXT_SUFFIX') or '.so'))
    if os.path.exists(mod) and os.path.getmtime(mod) >= max(os.path.getmtime(CY_CPP), os.path.getmtime(LIB)):
        return mod
    cmd = ['g++', '-O2', '-fPIC', '-shared', '-I' + sysconfig.get_paths()['include'], '-I' + INCLUDE,
           CY_CPP, '-L' + HERE, '-lfe3d_gb300', '-Wl,-rpath,$ORIGIN', '-o', mod]
    out = subprocess.run(cmd, capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError('g++ failed for the Cython binding:\n' + out.stdout + out.stderr)
    return mod


if __name__ == '__main__':
    print(build(verbose='-v' in sys.argv, force='-f' in sys.argv))
    print(build_cython())
