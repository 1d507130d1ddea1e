"""ctypes front end of the CPU oracle (test infrastructure only).

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` use this module, as the checker.  The product package
``pyfe3d_gb300`` never imports it.

Each wrapper takes numpy arrays, follows the per-element sequence of the
reference (rotation -> probe -> matrix) and writes COO triplets exactly
where ``pyfe3d`` would (``init_k`` offsets, ``+=`` on values).
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, 'build', 'libfe3d_oracle.so')
Q4P_STRIDE = 28
BCP_STRIDE = 16

_lib = None


def build(quiet=True):
    """Compile the oracle shared library with its Makefile."""
    out = subprocess.run(['make', '-C', HERE], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError('oracle build failed:\n' + out.stdout + out.stderr)
    if not quiet:
        print(out.stdout)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        _lib = ctypes.CDLL(LIB_PATH)
        _lib.orc_num_threads.restype = ctypes.c_int
    return _lib


def _p(a):
    if a is None:
        return None
    return a.ctypes.data_as(ctypes.c_void_p)


def _d(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _i(a):
    return np.ascontiguousarray(a, dtype=np.int64)


def set_threads(n):
    lib().orc_set_threads(ctypes.c_int(int(n)))


def num_threads():
    return int(lib().orc_num_threads())


# ---------------------------------------------------------------- Quad4
def q4_rotation(x, c, xmat=None, m=None):
    R = np.zeros(9)
    m = np.array([1., 0., 0., 1.]) if m is None else _d(m).copy()
    lib().orc_q4_rotation(_p(_d(x)), _p(_i(c)), _p(None if xmat is None else _d(xmat)),
                          _p(R), _p(m))
    return R, m


def q4_probe_xe(x, c, R):
    xe = np.zeros(12)
    area = ctypes.c_double(0.)
    lib().orc_q4_probe_xe(_p(_d(x)), _p(_i(c)), _p(_d(R)), _p(xe), ctypes.byref(area))
    return xe, area.value


def q4_probe_ue(u, c, R):
    ue = np.zeros(24)
    lib().orc_q4_probe_ue(_p(_d(u)), _p(_i(c)), _p(_d(R)), _p(ue))
    return ue


def q4_kc0(R, m, xe, area, P, c, init_k, Kr, Kc, Kv, values_only=0):
    lib().orc_q4_kc0(_p(_d(R)), _p(_d(m)), _p(_d(xe)), ctypes.c_double(area), _p(_d(P)),
                     _p(_i(c)), ctypes.c_int64(init_k), _p(Kr), _p(Kc), _p(Kv),
                     ctypes.c_int(values_only))


def q4_kc0_local(m, xe, area, P):
    Ke = np.zeros(576)
    lib().orc_q4_kc0_local(_p(_d(m)), _p(_d(xe)), ctypes.c_double(area), _p(_d(P)), _p(Ke))
    return Ke.reshape(24, 24)


def q4_fint(R, m, xe, area, P, c, ue, fint):
    lib().orc_q4_fint(_p(_d(R)), _p(_d(m)), _p(_d(xe)), ctypes.c_double(area), _p(_d(P)),
                      _p(_i(c)), _p(_d(ue)), _p(fint))


def q4_finte(m, xe, area, P, ue):
    fe = np.zeros(24)
    lib().orc_q4_finte(_p(_d(m)), _p(_d(xe)), ctypes.c_double(area), _p(_d(P)), _p(_d(ue)), _p(fe))
    return fe


def q4_kg_given_stress(R, xe, N, c, init_k, Kr, Kc, Kv):
    lib().orc_q4_kg_given_stress(_p(_d(R)), _p(_d(xe)), ctypes.c_double(N[0]), ctypes.c_double(N[1]),
                                 ctypes.c_double(N[2]), _p(_i(c)), ctypes.c_int64(init_k), _p(Kr), _p(Kc),
                                 _p(Kv))


def bc_fint(R, L, P, c, ue, fint=None):
    """Local finte (returned) and, with fint, fint[c + .] += R finte."""
    fe = np.zeros(12)
    lib().orc_bc_fint(_p(_d(R)), ctypes.c_double(L), _p(_d(P)), _p(_i(c)), _p(_d(ue)), _p(fe),
                      None if fint is None else _p(fint))
    return fe


def q4_kg(R, m, xe, ue, P, c, init_k, Kr, Kc, Kv):
    lib().orc_q4_kg(_p(_d(R)), _p(_d(m)), _p(_d(xe)), _p(_d(ue)), _p(_d(P)), _p(_i(c)),
                    ctypes.c_int64(init_k), _p(Kr), _p(Kc), _p(Kv))


def q4_m(R, xe, area, P, c, init_k, Kr, Kc, Kv, mtype=0):
    lib().orc_q4_m(_p(_d(R)), _p(_d(xe)), ctypes.c_double(area), _p(_d(P)), _p(_i(c)),
                   ctypes.c_int64(init_k), _p(Kr), _p(Kc), _p(Kv), ctypes.c_int(mtype))


def _pid(pid, props, E, stride):
    """Element -> record map; a single record is shared by every element."""
    if pid is None and np.asarray(props).size // stride < E:
        return np.zeros(E, dtype=np.int32)
    return None if pid is None else np.ascontiguousarray(pid, dtype=np.int32)


def q4_kc0_batch(cdof, init_k, x, props, pid=None, xmat=None, Kr=None, Kc=None, Kv=None,
                 values_only=0):
    cdof = _i(cdof)
    init_k = _i(init_k)
    E = init_k.shape[0]
    n = int(init_k.max()) + 576 if E else 0
    Kr = np.zeros(n, np.int64) if Kr is None else Kr
    Kc = np.zeros(n, np.int64) if Kc is None else Kc
    Kv = np.zeros(n) if Kv is None else Kv
    pid = _pid(pid, props, E, Q4P_STRIDE)
    lib().orc_q4_kc0_batch(ctypes.c_int64(E), _p(cdof), _p(init_k), _p(_d(x)),
                           _p(None if xmat is None else _d(xmat)), _p(_d(props)), _p(pid),
                           _p(Kr), _p(Kc), _p(Kv), ctypes.c_int(values_only))
    return Kr, Kc, Kv


def q4_kg_batch(cdof, init_k, x, u, props, pid=None, xmat=None):
    cdof = _i(cdof)
    init_k = _i(init_k)
    E = init_k.shape[0]
    n = int(init_k.max()) + 144 if E else 0
    Kr = np.zeros(n, np.int64)
    Kc = np.zeros(n, np.int64)
    Kv = np.zeros(n)
    pid = _pid(pid, props, E, Q4P_STRIDE)
    lib().orc_q4_kg_batch(ctypes.c_int64(E), _p(cdof), _p(init_k), _p(_d(x)),
                          _p(None if xmat is None else _d(xmat)), _p(_d(u)), _p(_d(props)),
                          _p(pid), _p(Kr), _p(Kc), _p(Kv))
    return Kr, Kc, Kv


def q4_m_batch(cdof, init_k, x, props, pid=None, mtype=0):
    cdof = _i(cdof)
    init_k = _i(init_k)
    E = init_k.shape[0]
    n = int(init_k.max()) + 480 if E else 0
    Kr = np.zeros(n, np.int64)
    Kc = np.zeros(n, np.int64)
    Kv = np.zeros(n)
    pid = _pid(pid, props, E, Q4P_STRIDE)
    lib().orc_q4_m_batch(ctypes.c_int64(E), _p(cdof), _p(init_k), _p(_d(x)), _p(_d(props)),
                         _p(pid), _p(Kr), _p(Kc), _p(Kv), ctypes.c_int(mtype))
    return Kr, Kc, Kv


# ---------------------------------------------------------------- BeamC
def bc_rotation(x, c, vxy):
    R = np.zeros(9)
    lib().orc_bc_rotation(_p(_d(x)), _p(_i(c)), _p(_d(vxy)), _p(R))
    return R


def bc_probe_xe(x, c, R):
    xe = np.zeros(6)
    L = ctypes.c_double(0.)
    lib().orc_bc_probe_xe(_p(_d(x)), _p(_i(c)), _p(_d(R)), _p(xe), ctypes.byref(L))
    return xe, L.value


def bc_probe_ue(u, c, R):
    ue = np.zeros(12)
    lib().orc_bc_probe_ue(_p(_d(u)), _p(_i(c)), _p(_d(R)), _p(ue))
    return ue


def bc_kc0(R, L, P, c, init_k, Kr, Kc, Kv, values_only=0):
    lib().orc_bc_kc0(_p(_d(R)), ctypes.c_double(L), _p(_d(P)), _p(_i(c)),
                     ctypes.c_int64(init_k), _p(Kr), _p(Kc), _p(Kv), ctypes.c_int(values_only))


def bc_kg(R, L, P, ue, c, init_k, Kr, Kc, Kv, values_only=0):
    lib().orc_bc_kg(_p(_d(R)), ctypes.c_double(L), _p(_d(P)), _p(_d(ue)), _p(_i(c)),
                    ctypes.c_int64(init_k), _p(Kr), _p(Kc), _p(Kv), ctypes.c_int(values_only))


def bc_m(R, L, P, c, init_k, Kr, Kc, Kv, mtype=0):
    lib().orc_bc_m(_p(_d(R)), ctypes.c_double(L), _p(_d(P)), _p(_i(c)),
                   ctypes.c_int64(init_k), _p(Kr), _p(Kc), _p(Kv), ctypes.c_int(mtype))


def bc_kc0_batch(cdof, init_k, x, vxy, props, pid=None, values_only=0):
    cdof = _i(cdof)
    init_k = _i(init_k)
    E = init_k.shape[0]
    n = int(init_k.max()) + 144 if E else 0
    Kr = np.zeros(n, np.int64)
    Kc = np.zeros(n, np.int64)
    Kv = np.zeros(n)
    pid = _pid(pid, props, E, BCP_STRIDE)
    lib().orc_bc_kc0_batch(ctypes.c_int64(E), _p(cdof), _p(init_k), _p(_d(x)), _p(_d(vxy)),
                           _p(_d(props)), _p(pid), _p(Kr), _p(Kc), _p(Kv),
                           ctypes.c_int(values_only))
    return Kr, Kc, Kv


def _bc_elements(cdof, x, vxy, props, pid):
    """Per-element frame, length and property record, in element order."""
    cdof = _i(cdof).reshape(-1, 2)
    vxy = _d(vxy).reshape(-1, 3)
    props = _d(props).reshape(-1, BCP_STRIDE)
    E = cdof.shape[0]
    pid = np.zeros(E, np.int32) if pid is None else np.asarray(pid)
    for e in range(E):
        R = bc_rotation(x, cdof[e], vxy[e] if vxy.shape[0] > 1 else vxy[0])
        _, L = bc_probe_xe(x, cdof[e], R)
        yield e, cdof[e], R, L, props[pid[e]]


def bc_kg_batch(cdof, init_k, x, u, vxy, props, pid=None, Kr=None, Kc=None, Kv=None, values_only=0):
    """BeamC update_probe_ue + update_KG over every element (beamc.pyx:234-284,
    1392-2179) into the given arrays (new zeroed ones when omitted)."""
    init_k = _i(init_k)
    n = int(init_k.max()) + 144 if init_k.size else 0
    Kr = np.zeros(n, np.int64) if Kr is None else Kr
    Kc = np.zeros(n, np.int64) if Kc is None else Kc
    Kv = np.zeros(n) if Kv is None else Kv
    for e, c, R, L, P in _bc_elements(cdof, x, vxy, props, pid):
        ue = bc_probe_ue(u, c, R)
        bc_kg(R, L, P, ue, c, int(init_k[e]), Kr, Kc, Kv, values_only)
    return Kr, Kc, Kv


def bc_m_batch(cdof, init_k, x, vxy, props, pid=None, Kr=None, Kc=None, Kv=None, mtype=0):
    """BeamC update_M over every element (beamc.pyx:2181-3152)."""
    init_k = _i(init_k)
    n = int(init_k.max()) + 144 if init_k.size else 0
    Kr = np.zeros(n, np.int64) if Kr is None else Kr
    Kc = np.zeros(n, np.int64) if Kc is None else Kc
    Kv = np.zeros(n) if Kv is None else Kv
    for e, c, R, L, P in _bc_elements(cdof, x, vxy, props, pid):
        bc_m(R, L, P, c, int(init_k[e]), Kr, Kc, Kv, mtype)
    return Kr, Kc, Kv


# ------------------------------------------------- Tria3R / Quad4R
def t3_rotation(x, c, xmat=None, m=None):
    R = np.zeros(9)
    m = np.array([1., 0., 0., 1.]) if m is None else _d(m).copy()
    lib().orc_t3_rotation(_p(_d(x)), _p(_i(c)), _p(None if xmat is None else _d(xmat)),
                          _p(R), _p(m))
    return R, m


def t3_probe_xe(x, c, R):
    xe = np.zeros(9)
    area = ctypes.c_double(0.)
    lib().orc_t3_probe_xe(_p(_d(x)), _p(_i(c)), _p(_d(R)), _p(xe), ctypes.byref(area))
    return xe, area.value


def t3_probe_ue(u, c, R):
    ue = np.zeros(18)
    lib().orc_t3_probe_ue(_p(_d(u)), _p(_i(c)), _p(_d(R)), _p(ue))
    return ue


def t3_kc0_local(m, xe, area, P, k6rot=100., alpha=0.7):
    Ke = np.zeros(324)
    lib().orc_t3_kc0_local(_p(_d(m)), _p(_d(xe)), ctypes.c_double(area), _p(_d(P)),
                           ctypes.c_double(k6rot), ctypes.c_double(alpha), _p(Ke))
    return Ke.reshape(18, 18)


def t3_kc0(R, m, xe, area, P, c, init_k, Kr, Kc, Kv, k6rot=100., alpha=0.7, values_only=0):
    lib().orc_t3_kc0(_p(_d(R)), _p(_d(m)), _p(_d(xe)), ctypes.c_double(area), _p(_d(P)),
                     ctypes.c_double(k6rot), ctypes.c_double(alpha), _p(_i(c)), ctypes.c_int64(init_k),
                     _p(Kr), _p(Kc), _p(Kv), ctypes.c_int(values_only))


def t3_finte(m, xe, area, P, ue, k6rot=100., alpha=0.7):
    fe = np.zeros(18)
    lib().orc_t3_finte(_p(_d(m)), _p(_d(xe)), ctypes.c_double(area), _p(_d(P)), ctypes.c_double(k6rot),
                       ctypes.c_double(alpha), _p(_d(ue)), _p(fe))
    return fe


def t3_fint(R, m, xe, area, P, c, ue, fint, k6rot=100., alpha=0.7):
    lib().orc_t3_fint(_p(_d(R)), _p(_d(m)), _p(_d(xe)), ctypes.c_double(area), _p(_d(P)),
                      ctypes.c_double(k6rot), ctypes.c_double(alpha), _p(_i(c)), _p(_d(ue)), _p(fint))


def t3_kg(R, m, xe, area, ue, P, c, init_k, Kr, Kc, Kv, values_only=0):
    lib().orc_t3_kg(_p(_d(R)), _p(_d(m)), _p(_d(xe)), ctypes.c_double(area), _p(_d(ue)), _p(_d(P)),
                    _p(_i(c)), ctypes.c_int64(init_k), _p(Kr), _p(Kc), _p(Kv), ctypes.c_int(values_only))


def t3_kg_given_stress(R, xe, area, N, c, init_k, Kr, Kc, Kv, values_only=0):
    lib().orc_t3_kg_given_stress(_p(_d(R)), _p(_d(xe)), ctypes.c_double(area), ctypes.c_double(N[0]),
                                 ctypes.c_double(N[1]), ctypes.c_double(N[2]), _p(_i(c)),
                                 ctypes.c_int64(init_k), _p(Kr), _p(Kc), _p(Kv), ctypes.c_int(values_only))


def t3_m(R, area, P, c, init_k, Kr, Kc, Kv, mtype=0):
    lib().orc_t3_m(_p(_d(R)), ctypes.c_double(area), _p(_d(P)), _p(_i(c)), ctypes.c_int64(init_k),
                   _p(Kr), _p(Kc), _p(Kv), ctypes.c_int(mtype))


def q4r_kc0_local(m, xe, area, P, k6rot=100., hg=(1., 1., 1., 1., 1.)):
    Ke = np.zeros(576)
    lib().orc_q4r_kc0_local(_p(_d(m)), _p(_d(xe)), ctypes.c_double(area), _p(_d(P)),
                            ctypes.c_double(k6rot), _p(_d(hg)), _p(Ke))
    return Ke.reshape(24, 24)


def q4r_kc0(R, m, xe, area, P, c, init_k, Kr, Kc, Kv, k6rot=100., hg=(1., 1., 1., 1., 1.),
            values_only=0):
    lib().orc_q4r_kc0(_p(_d(R)), _p(_d(m)), _p(_d(xe)), ctypes.c_double(area), _p(_d(P)),
                      ctypes.c_double(k6rot), _p(_d(hg)), _p(_i(c)), ctypes.c_int64(init_k),
                      _p(Kr), _p(Kc), _p(Kv), ctypes.c_int(values_only))


def q4r_finte(m, xe, area, P, ue, k6rot=100., hg=(1., 1., 1., 1., 1.)):
    fe = np.zeros(24)
    lib().orc_q4r_finte(_p(_d(m)), _p(_d(xe)), ctypes.c_double(area), _p(_d(P)), ctypes.c_double(k6rot),
                        _p(_d(hg)), _p(_d(ue)), _p(fe))
    return fe


def q4r_fint(R, m, xe, area, P, c, ue, fint, k6rot=100., hg=(1., 1., 1., 1., 1.)):
    lib().orc_q4r_fint(_p(_d(R)), _p(_d(m)), _p(_d(xe)), ctypes.c_double(area), _p(_d(P)),
                       ctypes.c_double(k6rot), _p(_d(hg)), _p(_i(c)), _p(_d(ue)), _p(fint))


def _per_elem(v, E, width=1):
    v = np.asarray(v, dtype=np.float64)
    if v.size == width:
        v = np.tile(v.reshape(-1), E)
    return np.ascontiguousarray(v.reshape(-1))


def t3_kc0_batch(cdof, init_k, x, props, pid=None, xmat=None, k6rot=100., alpha=0.7, values_only=0):
    cdof = _i(cdof)
    init_k = _i(init_k)
    E = init_k.shape[0]
    n = int(init_k.max()) + 324 if E else 0
    Kr, Kc, Kv = np.zeros(n, np.int64), np.zeros(n, np.int64), np.zeros(n)
    pid = _pid(pid, props, E, Q4P_STRIDE)
    lib().orc_t3_kc0_batch(ctypes.c_int64(E), _p(cdof), _p(init_k), _p(_d(x)),
                           _p(None if xmat is None else _d(xmat)), _p(_d(props)), _p(pid),
                           _p(_per_elem(k6rot, E)), _p(_per_elem(alpha, E)), _p(Kr), _p(Kc), _p(Kv),
                           ctypes.c_int(values_only))
    return Kr, Kc, Kv


def q4r_kc0_batch(cdof, init_k, x, props, pid=None, xmat=None, k6rot=100., hg=(1., 1., 1., 1., 1.),
                  values_only=0):
    cdof = _i(cdof)
    init_k = _i(init_k)
    E = init_k.shape[0]
    n = int(init_k.max()) + 576 if E else 0
    Kr, Kc, Kv = np.zeros(n, np.int64), np.zeros(n, np.int64), np.zeros(n)
    pid = _pid(pid, props, E, Q4P_STRIDE)
    lib().orc_q4r_kc0_batch(ctypes.c_int64(E), _p(cdof), _p(init_k), _p(_d(x)),
                            _p(None if xmat is None else _d(xmat)), _p(_d(props)), _p(pid),
                            _p(_per_elem(k6rot, E)), _p(_per_elem(hg, E, 5)), _p(Kr), _p(Kc), _p(Kv),
                            ctypes.c_int(values_only))
    return Kr, Kc, Kv


# ------------------------------------------------- property records
SHELL_FIELDS = ('A11', 'A12', 'A16', 'A22', 'A26', 'A66', 'B11', 'B12', 'B16', 'B22',
                'B26', 'B66', 'D11', 'D12', 'D16', 'D22', 'D26', 'D66', 'E44', 'E45',
                'E55', 'scf_k13', 'scf_k23', 'h', 'intrho', 'intrhoz', 'intrhoz2')
BEAM_FIELDS = ('A', 'E', 'G', 'Iyy', 'Izz', 'Iyz', 'J', 'Ay', 'Az', 'intrho', 'intrhoy',
               'intrhoz', 'intrhoy2', 'intrhoz2', 'intrhoyz')


def shell_record(prop):
    """Flatten any object exposing ShellProp attributes into a 28-double record."""
    rec = np.zeros(Q4P_STRIDE)
    for i, f in enumerate(SHELL_FIELDS):
        rec[i] = float(getattr(prop, f))
    return rec


def beam_record(prop):
    rec = np.zeros(BCP_STRIDE)
    for i, f in enumerate(BEAM_FIELDS):
        rec[i] = float(getattr(prop, f))
    return rec
