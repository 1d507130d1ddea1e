"""The C-ABI library loads and exports every symbol its header declares (no GPU)."""
import ctypes
import os
import re

from conftest import ROOT


def header_functions():
    names = []
    for f in os.listdir(os.path.join(ROOT, 'include')):
        if f.endswith('.h'):
            src = open(os.path.join(ROOT, 'include', f)).read()
            src = re.sub(r'/\*.*?\*/', '', src, flags=re.S)
            names += re.findall(r'^\s*(?:const\s+)?[a-z_0-9]+\s*\**\s*(fe3d_[a-z0-9_]+)\s*\(', src, re.M)
    return sorted(set(names))


def test_library_exports_header_symbols():
    from pyfe3d_gb300 import build
    path = build.build()
    lib = ctypes.CDLL(path)
    names = header_functions()
    assert len(names) >= 15
    for n in names:
        assert hasattr(lib, n), n


def test_python_signatures_cover_header():
    from pyfe3d_gb300 import _lib
    declared = set(_lib.declared_symbols())
    missing = [n for n in header_functions() if n not in declared and n != 'fe3d_error_string']
    assert not missing, missing


def test_version_and_error_strings():
    from pyfe3d_gb300 import _lib
    lib = _lib.load()
    assert lib.fe3d_version() >= 1
    lib.fe3d_error_string.restype = ctypes.c_char_p
    assert lib.fe3d_error_string(-1) == b'invalid argument'


def test_argument_errors_before_launch():
    """Invalid arguments are rejected on the host, before any device work."""
    from pyfe3d_gb300 import _lib
    lib = _lib.load()
    assert lib.fe3d_quad4_kc0(-1, None, None, None, 0, None, 0, None, None, None, None, None, 0,
                              None, None, None, None, 0, 0, None, None) == -1
    # probe mode without its inputs
    assert lib.fe3d_quad4_kc0(4, ctypes.c_void_p(8), ctypes.c_void_p(8), None, 0, None, 0, None,
                              None, None, None, ctypes.c_void_p(8), 1, None, ctypes.c_void_p(8),
                              ctypes.c_void_p(8), ctypes.c_void_p(8), 10, 0, None, None) == -1
    assert lib.fe3d_quad4_m(1, ctypes.c_void_p(8), ctypes.c_void_p(8), ctypes.c_void_p(8), 3, None,
                            None, None, ctypes.c_void_p(8), 1, None, ctypes.c_void_p(8),
                            ctypes.c_void_p(8), ctypes.c_void_p(8), 480, 7, None, None) == -1
    assert lib.fe3d_beamc_m(1, ctypes.c_void_p(8), ctypes.c_void_p(8), ctypes.c_void_p(8),
                            ctypes.c_void_p(8), ctypes.c_void_p(8), 1, None, ctypes.c_void_p(8),
                            ctypes.c_void_p(8), ctypes.c_void_p(8), 144, 5, None, None) == -1
    # zero elements is a no-op
    assert lib.fe3d_quad4_frame(0, None, None, 0, None, 0, None, None, None, None, None, None) == 0


def test_reduced_shell_argument_errors_before_launch():
    """Tria3R / Quad4R entry points reject bad arguments on the host."""
    from pyfe3d_gb300 import _lib
    lib = _lib.load()
    v = ctypes.c_void_p(8)
    for fn in (lib.fe3d_tria3r_kc0, lib.fe3d_quad4r_kc0):
        # negative count, missing arrays, probe mode without its inputs
        assert fn(-1, None, None, None, 0, None, 0, None, None, None, None, None, 0, None, None, 0, None, 0,
                  None, None, None, 0, 0, None, None) == -1
        assert fn(3, v, v, None, 0, None, 0, None, None, None, None, v, 1, None, v, 0, v, 0, v, v, v, 10, 0,
                  None, None) == -1
        # bad stride of the per-element parameters
        assert fn(3, v, v, v, 9, None, 0, None, None, None, None, v, 1, None, v, 7, v, 0, v, v, v, 10, 0,
                  None, None) == -1
        assert fn(0, None, None, None, 0, None, 0, None, None, None, None, None, 0, None, None, 0, None, 0,
                  None, None, None, 0, 0, None, None) == 0
    assert lib.fe3d_tria3r_m(1, v, v, v, 9, None, None, v, 1, None, v, v, v, 270, 3, None, None) == -1
    assert lib.fe3d_tria3r_kg_given_stress(1, v, v, v, 9, None, None, None, v, 2, v, v, v, 81, 0, None,
                                           None) == -1
    assert lib.fe3d_tria3r_finte(1, v, v, v, v, v, v, v, 1, None, v, 0, v, 0, None, 0, None, None, None) == -1
    assert lib.fe3d_tria3r_frame(0, None, None, 0, None, 0, None, None, None, None, None, None) == 0
