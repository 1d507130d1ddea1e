"""Build the reference implementation's element modules as the CPU reference.

Test and benchmark infrastructure only (the library never imports it).

The reference (pyfe3d, Cython compiled to C++) is built from its own
sources: its Quad4, BeamC, ShellProp and BeamProp modules
(pyfe3d/quad4.pyx, beamc.pyx, shellprop.pyx, beamprop.pyx) are translated
to C++ with Cython (C++ mode, language level 3, the `linetrace` directive of
the reference's setup.py) and compiled with g++ -O2 -fopenmp, as its setup.py
does.  Everything is written under oracle/_ref/:

    oracle/_ref/src/pyfe3d/<module>.cpp   generated C++ (needs the reference
                                         sources and Cython: done where the
                                         reference is available)
    oracle/_ref/pyfe3d/<module><ext>      compiled extension modules
    oracle/_ref/pyfe3d/__init__.py        a minimal package file written here
                                         (DOF, INT, DOUBLE and the classes)

The generated C++ needs only g++ and the Python headers, so a machine
without the reference sources or Cython compiles the sources generated
elsewhere (`python oracle/build_ref.py compile`).

    python oracle/build_ref.py [generate|compile|all] [--ref PATH]

`generate` reads the reference from --ref, PYFE3D_REF or, when neither is
given, the checkout this recipe was written against (DEFAULT_REF).
"""
import argparse
import concurrent.futures as cf
import os
import subprocess
import sys
import sysconfig

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, '_ref')
SRC = os.path.join(OUT, 'src', 'pyfe3d')
PKG = os.path.join(OUT, 'pyfe3d')
MODULES = ('beamprop', 'shellprop', 'beamc', 'quad4')
DEFAULT_REF = '/root/reference'

INIT = '''"""The reference's element modules built by oracle/build_ref.py (CPU reference)."""
import ctypes

import numpy as np

from .quad4 import Quad4, Quad4Data, Quad4Probe
from .beamc import BeamC, BeamCData, BeamCProbe
from .shellprop import ShellProp
from .beamprop import BeamProp

DOF = 6
INT = np.int64 if ctypes.sizeof(ctypes.c_long) == 8 else np.int32
DOUBLE = np.float64
'''


def generate(ref):
    """Cython -> C++ for the path's modules of the reference checkout `ref`."""
    src_dir = os.path.join(ref, 'pyfe3d')
    os.makedirs(SRC, exist_ok=True)
    for m in MODULES:
        pyx = os.path.join(src_dir, m + '.pyx')
        out = os.path.join(SRC, m + '.cpp')
        if os.path.exists(out) and os.path.getmtime(out) >= os.path.getmtime(pyx):
            continue
        cmd = [sys.executable, '-m', 'cython', '--cplus', '-3', '-X', 'linetrace=True', pyx, '-o', out]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError('cython failed for %s:\n%s%s' % (m, r.stdout, r.stderr))
    os.makedirs(PKG, exist_ok=True)
    with open(os.path.join(PKG, '__init__.py'), 'w') as fh:
        fh.write(INIT)


def _compile_one(m):
    src = os.path.join(SRC, m + '.cpp')
    ext = sysconfig.get_config_var('EXT_SUFFIX') or '.so'
    out = os.path.join(PKG, m + ext)
    if os.path.exists(out) and os.path.getmtime(out) >= os.path.getmtime(src):
        return out
    inc = sysconfig.get_paths()['include']
    cmd = ['g++', '-O2', '-fPIC', '-shared', '-fopenmp', '-I' + inc, src, '-o', out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError('g++ failed for %s:\n%s%s' % (m, r.stdout, r.stderr))
    return out


def have_sources():
    return all(os.path.exists(os.path.join(SRC, m + '.cpp')) for m in MODULES)


def compile_all():
    """Compile the generated C++ (in parallel); returns the module paths."""
    if not have_sources():
        raise RuntimeError('no generated reference sources under %s' % SRC)
    os.makedirs(PKG, exist_ok=True)
    if not os.path.exists(os.path.join(PKG, '__init__.py')):
        with open(os.path.join(PKG, '__init__.py'), 'w') as fh:
            fh.write(INIT)
    with cf.ThreadPoolExecutor(max_workers=len(MODULES)) as ex:
        return list(ex.map(_compile_one, MODULES))


def build(ref=None):
    """Generate (when the reference sources are reachable) and compile; a
    no-op without generated sources.  Returns True when the modules exist."""
    ref = ref or os.environ.get('PYFE3D_REF') or DEFAULT_REF
    if os.path.isdir(os.path.join(ref, 'pyfe3d')):
        try:
            import Cython  # noqa: F401
            generate(ref)
        except ImportError:
            pass
    if not have_sources():
        return False
    compile_all()
    return True


def load():
    """The compiled reference package (pyfe3d), or None when not built."""
    if not os.path.isdir(PKG):
        return None
    if OUT not in sys.path:
        sys.path.insert(0, OUT)
    try:
        import pyfe3d
    except ImportError:
        return None
    if not os.path.dirname(os.path.abspath(pyfe3d.__file__)) == PKG:
        return None
    return pyfe3d


if __name__ == '__main__':
    ap = argparse.ArgumentParser()
    ap.add_argument('what', nargs='?', default='all', choices=['generate', 'compile', 'all'])
    ap.add_argument('--ref', default=os.environ.get('PYFE3D_REF') or DEFAULT_REF)
    a = ap.parse_args()
    if a.what in ('generate', 'all'):
        generate(a.ref)
    if a.what in ('compile', 'all'):
        print('\n'.join(compile_all()))
