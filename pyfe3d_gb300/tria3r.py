"""Tria3R element with the API of ``pyfe3d.tria3r`` (pyfe3d/tria3r.pyx:128-7723).

Every method computes on the GPU through ``libfe3d_gb300.so``; the object only
holds the element state (offsets, frame, probe buffers).  For whole meshes
use :mod:`pyfe3d_gb300.batch` (``tria3r_update_KC0`` and friends), which
runs the same kernels over all elements in one launch.
"""
import numpy as np

from . import _lib
from ._elem import CooTarget, dev, gather, host
from .shellprop import shell_record

DOF = 6
NUM_NODES = 3
_LOCAL_C = np.array([0, 6, 12], dtype=np.int64)


class Tria3RData:
    """Sparse sizes per element (tria3r.pyx:128-151)."""

    def __init__(self):
        self.KC0_SPARSE_SIZE = 324
        self.KG_SPARSE_SIZE = 81
        self.M_SPARSE_SIZE = 270


class Tria3RProbe:
    """Per-probe buffers shared by the elements using it (tria3r.pyx:154-193)."""

    def __init__(self):
        self.xe = np.zeros(NUM_NODES * DOF // 2, dtype=np.float64)
        self.ue = np.zeros(NUM_NODES * DOF, dtype=np.float64)
        self.finte = np.zeros(NUM_NODES * DOF, dtype=np.float64)


class Tria3R:
    """Triangular shell with reduced integration (tria3r.pyx:196-292)."""

    def __init__(self, p):
        self.probe = p
        self.eid = -1
        self.pid = -1
        self.n1 = self.n2 = self.n3 = -1
        self.c1 = self.c2 = self.c3 = -1
        self.init_k_KC0 = 0
        self.init_k_KG = 0
        self.init_k_M = 0
        self.area = 0.
        self.K6ROT = 100.
        self.alpha_shear_locking = 0.7
        self.r11 = self.r12 = self.r13 = 0.
        self.r21 = self.r22 = self.r23 = 0.
        self.r31 = self.r32 = self.r33 = 0.
        self.m11 = 1.
        self.m12 = 0.
        self.m21 = 0.
        self.m22 = 1.

    # -- state <-> device -------------------------------------------------
    def _c(self):
        return np.array([self.c1, self.c2, self.c3], dtype=np.int64)

    def _R(self):
        return np.array([self.r11, self.r12, self.r13, self.r21, self.r22, self.r23,
                         self.r31, self.r32, self.r33])

    def _set_R(self, R):
        (self.r11, self.r12, self.r13, self.r21, self.r22, self.r23,
         self.r31, self.r32, self.r33) = (float(v) for v in R)

    def _m(self):
        return np.array([self.m11, self.m12, self.m21, self.m22])

    def _coords(self, x):
        c = self._c()
        if (c < 0).any():
            raise ValueError('Tria3R DOF offsets c1..c3 are not set')
        idx = (c // 2)[:, None] + np.arange(3)[None, :]
        return dev(gather(x, idx.ravel()))

    def _probe_inputs(self):
        return (dev(self._R()), dev(self._m()), dev(np.asarray(self.probe.xe, dtype=np.float64)),
                dev(np.array([self.area])))

    def _scalars(self):
        return dev(np.array([self.K6ROT])), dev(np.array([self.alpha_shear_locking]))

    # -- frame and probes -------------------------------------------------
    def update_rotation_matrix(self, x, xmati=0., xmatj=0., xmatk=0.):
        """Element frame and material-direction cosines (tria3r.pyx:294-423)."""
        lib = _lib.load()
        xs = self._coords(x)
        R = dev(np.zeros(9))
        m = dev(self._m())
        xmat = dev(np.array([xmati, xmatj, xmatk], dtype=np.float64))
        err = _lib.err_word()
        rc = lib.fe3d_tria3r_frame(1, _lib.keep(dev(_LOCAL_C, np.int64)), _lib.ptr(xs), 9, _lib.ptr(xmat), 0,
                                   _lib.ptr(R), _lib.ptr(m), None, None, _lib.ptr(err), _lib.stream_ptr())
        _lib.check(rc, 'Tria3R.update_rotation_matrix', err)
        self._set_R(host(R))
        self.m11, self.m12, self.m21, self.m22 = (float(v) for v in host(m))

    def update_probe_xe(self, x):
        """Local nodal coordinates and area (tria3r.pyx:480-547)."""
        lib = _lib.load()
        xs = self._coords(x)
        xe = dev(np.zeros(9))
        area = dev(np.zeros(1))
        err = _lib.err_word()
        rc = lib.fe3d_tria3r_probe_xe(1, _lib.keep(dev(_LOCAL_C, np.int64)), _lib.ptr(xs), 9,
                                      _lib.keep(dev(self._R())), _lib.ptr(xe), _lib.ptr(area), _lib.ptr(err),
                                      _lib.stream_ptr())
        _lib.check(rc, 'Tria3R.update_probe_xe', err)
        self.probe.xe[:] = host(xe)
        self.area = float(host(area)[0])

    def update_area(self):
        """Area of the local coordinates held by the probe (tria3r.pyx:530-547)."""
        lib = _lib.load()
        xe = np.asarray(self.probe.xe, dtype=np.float64)
        area = dev(np.zeros(1))
        err = _lib.err_word()
        rc = lib.fe3d_tria3r_probe_xe(1, _lib.keep(dev(_LOCAL_C, np.int64)), _lib.keep(dev(xe)), 9,
                                      _lib.keep(dev(np.eye(3).ravel())), None, _lib.ptr(area), _lib.ptr(err),
                                      _lib.stream_ptr())
        _lib.check(rc, 'Tria3R.update_area', err)
        self.area = float(host(area)[0])

    def update_probe_ue(self, u):
        """Local element displacements R^T u (tria3r.pyx:426-477)."""
        lib = _lib.load()
        c = self._c()
        idx = (c[:, None] + np.arange(6)[None, :]).ravel()
        us = dev(gather(u, idx))
        ue = dev(np.zeros(18))
        err = _lib.err_word()
        rc = lib.fe3d_tria3r_probe_ue(1, _lib.keep(dev(_LOCAL_C, np.int64)), _lib.ptr(us), 18,
                                      _lib.keep(dev(self._R())), _lib.ptr(ue), _lib.ptr(err), _lib.stream_ptr())
        _lib.check(rc, 'Tria3R.update_probe_ue', err)
        self.probe.ue[:] = host(ue)

    # -- structural matrices ----------------------------------------------
    def update_KC0(self, KC0r, KC0c, KC0v, prop, update_KC0v_only=0):
        """Constitutive stiffness triplets at init_k_KC0 (tria3r.pyx:950-2960)."""
        lib = _lib.load()
        tgt = CooTarget(KC0r, KC0c, KC0v, self.init_k_KC0, 324, update_KC0v_only == 0)
        R, m, xe, area = self._probe_inputs()
        k6, al = self._scalars()
        P = dev(shell_record(prop))
        err = _lib.err_word()
        rc = lib.fe3d_tria3r_kc0(1, _lib.keep(dev(self._c(), np.int64)), _lib.ptr(tgt.init_k), None, 0, None, 0,
                                 _lib.ptr(R), _lib.ptr(m), _lib.ptr(xe), _lib.ptr(area), _lib.ptr(P), 1, None,
                                 _lib.ptr(k6), 0, _lib.ptr(al), 0, _lib.ptr(tgt.r), _lib.ptr(tgt.c),
                                 _lib.ptr(tgt.v), tgt.nk, int(update_KC0v_only != 0), _lib.ptr(err),
                                 _lib.stream_ptr())
        _lib.check(rc, 'Tria3R.update_KC0', err)
        tgt.finish()

    def update_probe_finte(self, prop):
        """probe.finte = KC0e probe.ue in the element frame (tria3r.pyx:549-947)."""
        lib = _lib.load()
        R, m, xe, area = self._probe_inputs()
        k6, al = self._scalars()
        ue = dev(np.asarray(self.probe.ue, dtype=np.float64))
        P = dev(shell_record(prop))
        fe = dev(np.zeros(18))
        err = _lib.err_word()
        rc = lib.fe3d_tria3r_finte(1, _lib.keep(dev(_LOCAL_C, np.int64)), _lib.ptr(R), _lib.ptr(m), _lib.ptr(xe),
                                   _lib.ptr(area), _lib.ptr(ue), _lib.ptr(P), 1, None, _lib.ptr(k6), 0,
                                   _lib.ptr(al), 0, None, 0, _lib.ptr(fe), _lib.ptr(err), _lib.stream_ptr())
        _lib.check(rc, 'Tria3R.update_probe_finte', err)
        self.probe.finte[:] = host(fe)

    def update_fint(self, fint, prop):
        """Internal forces R (KC0e ue) added at c1..c3; probe.finte is
        updated too (tria3r.pyx:2975-3017)."""
        lib = _lib.load()
        R, m, xe, area = self._probe_inputs()
        k6, al = self._scalars()
        ue = dev(np.asarray(self.probe.ue, dtype=np.float64))
        P = dev(shell_record(prop))
        c = self._c()
        idx = (c[:, None] + np.arange(6)[None, :]).ravel()
        # the element's 18 entries of fint are gathered, accumulated by the
        # kernel on the device and scattered back (assignment only)
        f = dev(gather(fint, idx))
        fe = dev(np.zeros(18))
        err = _lib.err_word()
        rc = lib.fe3d_tria3r_finte(1, _lib.keep(dev(_LOCAL_C, np.int64)), _lib.ptr(R), _lib.ptr(m), _lib.ptr(xe),
                                   _lib.ptr(area), _lib.ptr(ue), _lib.ptr(P), 1, None, _lib.ptr(k6), 0,
                                   _lib.ptr(al), 0, _lib.ptr(f), 18, _lib.ptr(fe), _lib.ptr(err),
                                   _lib.stream_ptr())
        _lib.check(rc, 'Tria3R.update_fint', err)
        self.probe.finte[:] = host(fe)
        if _lib.is_cuda_tensor(fint):
            torch = _lib.torch_mod()
            fint[torch.as_tensor(idx, device=fint.device)] = f
        else:
            fint[idx] = host(f)

    def update_KG(self, KGr, KGc, KGv, prop, update_KGv_only=0):
        """Geometric stiffness from probe.ue (tria3r.pyx:3020-3574)."""
        lib = _lib.load()
        tgt = CooTarget(KGr, KGc, KGv, self.init_k_KG, 81, update_KGv_only == 0)
        R, m, xe, area = self._probe_inputs()
        ue = dev(np.asarray(self.probe.ue, dtype=np.float64))
        P = dev(shell_record(prop))
        err = _lib.err_word()
        rc = lib.fe3d_tria3r_kg(1, _lib.keep(dev(self._c(), np.int64)), _lib.ptr(tgt.init_k), None, 0, None, 0,
                                None, 0, _lib.ptr(R), _lib.ptr(m), _lib.ptr(xe), _lib.ptr(area), _lib.ptr(ue),
                                _lib.ptr(P), 1, None, _lib.ptr(tgt.r), _lib.ptr(tgt.c), _lib.ptr(tgt.v), tgt.nk,
                                int(update_KGv_only != 0), _lib.ptr(err), _lib.stream_ptr())
        _lib.check(rc, 'Tria3R.update_KG', err)
        tgt.finish()

    def update_KG_given_stress(self, Nxx, Nyy, Nxy, KGr, KGc, KGv, update_KGv_only=0):
        """Geometric stiffness of a constant stress state (tria3r.pyx:3576-4061)."""
        lib = _lib.load()
        tgt = CooTarget(KGr, KGc, KGv, self.init_k_KG, 81, update_KGv_only == 0)
        R, _, xe, area = self._probe_inputs()
        ns = dev(np.array([Nxx, Nyy, Nxy], dtype=np.float64))
        err = _lib.err_word()
        rc = lib.fe3d_tria3r_kg_given_stress(1, _lib.keep(dev(self._c(), np.int64)), _lib.ptr(tgt.init_k), None,
                                             0, _lib.ptr(R), _lib.ptr(xe), _lib.ptr(area), _lib.ptr(ns), 0,
                                             _lib.ptr(tgt.r), _lib.ptr(tgt.c), _lib.ptr(tgt.v), tgt.nk,
                                             int(update_KGv_only != 0), _lib.ptr(err), _lib.stream_ptr())
        _lib.check(rc, 'Tria3R.update_KG_given_stress', err)
        tgt.finish()

    def update_M(self, Mr, Mc, Mv, prop, mtype=0):
        """Mass matrix triplets, mtype 0/1/2 (tria3r.pyx:4063-7723)."""
        if mtype not in (0, 1, 2):
            raise ValueError('mtype must be 0, 1 or 2')
        lib = _lib.load()
        size = 162 if mtype == 2 else 270
        tgt = CooTarget(Mr, Mc, Mv, self.init_k_M, size, True)
        R, _, _, area = self._probe_inputs()
        P = dev(shell_record(prop))
        err = _lib.err_word()
        rc = lib.fe3d_tria3r_m(1, _lib.keep(dev(self._c(), np.int64)), _lib.ptr(tgt.init_k), None, 0,
                               _lib.ptr(R), _lib.ptr(area), _lib.ptr(P), 1, None, _lib.ptr(tgt.r),
                               _lib.ptr(tgt.c), _lib.ptr(tgt.v), tgt.nk, int(mtype), _lib.ptr(err),
                               _lib.stream_ptr())
        _lib.check(rc, 'Tria3R.update_M', err)
        tgt.finish()
