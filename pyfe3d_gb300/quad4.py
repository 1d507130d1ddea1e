"""Quad4 element with the API of ``pyfe3d.quad4`` (pyfe3d/quad4.pyx:132-3081).

Every method computes on the GPU through ``libfe3d_gb300.so``; the object only
holds the element state (offsets, frame, probe buffers).  Calling a GPU kernel
per element is correct but latency-bound: for whole meshes use
:mod:`pyfe3d_gb300.batch`, which runs the same kernels over all elements in
one launch.
"""
import numpy as np

from . import _lib
from ._elem import CooTarget, dev, gather, host
from .shellprop import shell_record

DOF = 6
NUM_NODES = 4
_LOCAL_C = np.array([0, 6, 12, 18], dtype=np.int64)


class Quad4Data:
    """Sparse sizes per element (quad4.pyx:142-180)."""

    def __init__(self):
        self.KC0_SPARSE_SIZE = 576
        self.KG_SPARSE_SIZE = 144
        self.M_SPARSE_SIZE = 480
        self.KA_BETA_SPARSE_SIZE = 144
        self.KA_GAMMA_SPARSE_SIZE = 144
        self.CA_SPARSE_SIZE = 144


class Quad4Probe:
    """Per-probe buffers shared by the elements using it (quad4.pyx:183-271)."""

    def __init__(self):
        self.xe = np.zeros(NUM_NODES * DOF // 2, dtype=np.float64)
        self.ue = np.zeros(NUM_NODES * DOF, dtype=np.float64)
        self.finte = np.zeros(NUM_NODES * DOF, dtype=np.float64)


class Quad4:
    """Quadrilateral shell element with mixed integration (quad4.pyx:398-489)."""

    def __init__(self, p):
        self.probe = p
        self.eid = -1
        self.pid = -1
        self.n1 = self.n2 = self.n3 = self.n4 = -1
        self.c1 = self.c2 = self.c3 = self.c4 = -1
        self.init_k_KC0 = 0
        self.init_k_KG = 0
        self.init_k_M = 0
        self.init_k_KA_beta = 0
        self.init_k_KA_gamma = 0
        self.init_k_CA = 0
        self.area = 0.
        self.K6ROT = 100.
        self.r11 = self.r12 = self.r13 = 0.
        self.r21 = self.r22 = self.r23 = 0.
        self.r31 = self.r32 = self.r33 = 0.
        self.m11 = 1.
        self.m12 = 0.
        self.m21 = 0.
        self.m22 = 1.

    # -- state <-> device -------------------------------------------------
    def _c(self):
        return np.array([self.c1, self.c2, self.c3, self.c4], dtype=np.int64)

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
            raise ValueError('Quad4 DOF offsets c1..c4 are not set')
        idx = (c // 2)[:, None] + np.arange(3)[None, :]
        return dev(gather(x, idx.ravel()))

    # -- frame and probes -------------------------------------------------
    def update_rotation_matrix(self, x, xmati=0., xmatj=0., xmatk=0.):
        """Element frame and material-direction cosines (quad4.pyx:491-624)."""
        lib = _lib.load()
        xs = self._coords(x)
        R = dev(np.zeros(9))
        m = dev(self._m())
        xmat = dev(np.array([xmati, xmatj, xmatk], dtype=np.float64))
        err = _lib.err_word()
        rc = lib.fe3d_quad4_frame(1, _lib.keep(dev(_LOCAL_C, np.int64)), _lib.ptr(xs), 12,
                                  _lib.ptr(xmat), 0, _lib.ptr(R), _lib.ptr(m), None, None,
                                  _lib.ptr(err), _lib.stream_ptr())
        _lib.check(rc, 'Quad4.update_rotation_matrix', err)
        self._set_R(host(R))
        self.m11, self.m12, self.m21, self.m22 = (float(v) for v in host(m))

    def update_probe_xe(self, x):
        """Local nodal coordinates and area (quad4.pyx:682-752)."""
        lib = _lib.load()
        xs = self._coords(x)
        xe = dev(np.zeros(12))
        area = dev(np.zeros(1))
        err = _lib.err_word()
        rc = lib.fe3d_quad4_probe_xe(1, _lib.keep(dev(_LOCAL_C, np.int64)), _lib.ptr(xs), 12,
                                     _lib.keep(dev(self._R())), _lib.ptr(xe), _lib.ptr(area),
                                     _lib.ptr(err), _lib.stream_ptr())
        _lib.check(rc, 'Quad4.update_probe_xe', err)
        self.probe.xe[:] = host(xe)
        self.area = float(host(area)[0])

    def update_area(self):
        """Shoelace area of the local coordinates held by the probe (quad4.pyx:733-752)."""
        lib = _lib.load()
        xe = np.asarray(self.probe.xe, dtype=np.float64)
        R = np.eye(3).ravel()
        area = dev(np.zeros(1))
        err = _lib.err_word()
        rc = lib.fe3d_quad4_probe_xe(1, _lib.keep(dev(_LOCAL_C, np.int64)), _lib.keep(dev(xe)), 12,
                                     _lib.keep(dev(R)), None, _lib.ptr(area), _lib.ptr(err),
                                     _lib.stream_ptr())
        _lib.check(rc, 'Quad4.update_area', err)
        self.area = float(host(area)[0])

    def update_probe_ue(self, u):
        """Local element displacements R^T u (quad4.pyx:627-679)."""
        lib = _lib.load()
        c = self._c()
        idx = (c[:, None] + np.arange(6)[None, :]).ravel()
        us = dev(gather(u, idx))
        ue = dev(np.zeros(24))
        err = _lib.err_word()
        rc = lib.fe3d_quad4_probe_ue(1, _lib.keep(dev(_LOCAL_C, np.int64)), _lib.ptr(us), 24,
                                     _lib.keep(dev(self._R())), _lib.ptr(ue), _lib.ptr(err),
                                     _lib.stream_ptr())
        _lib.check(rc, 'Quad4.update_probe_ue', err)
        self.probe.ue[:] = host(ue)

    # -- structural matrices ----------------------------------------------
    def _probe_inputs(self):
        return (dev(self._R()), dev(self._m()), dev(np.asarray(self.probe.xe, dtype=np.float64)),
                dev(np.array([self.area])))

    def update_KC0(self, KC0r, KC0c, KC0v, prop, update_KC0v_only=0):
        """Constitutive stiffness triplets at init_k_KC0 (quad4.pyx:1204-1313)."""
        lib = _lib.load()
        tgt = CooTarget(KC0r, KC0c, KC0v, self.init_k_KC0, 576, update_KC0v_only == 0)
        R, m, xe, area = self._probe_inputs()
        P = dev(shell_record(prop))
        err = _lib.err_word()
        rc = lib.fe3d_quad4_kc0(1, _lib.keep(dev(self._c(), np.int64)), _lib.ptr(tgt.init_k),
                                None, 0, None, 0, _lib.ptr(R), _lib.ptr(m), _lib.ptr(xe),
                                _lib.ptr(area), _lib.ptr(P), 1, None, _lib.ptr(tgt.r),
                                _lib.ptr(tgt.c), _lib.ptr(tgt.v), tgt.nk, int(update_KC0v_only != 0),
                                _lib.ptr(err), _lib.stream_ptr())
        _lib.check(rc, 'Quad4.update_KC0', err)
        tgt.finish()

    def update_KG(self, KGr, KGc, KGv, prop):
        """Geometric stiffness from probe.ue (quad4.pyx:1365-2257)."""
        lib = _lib.load()
        tgt = CooTarget(KGr, KGc, KGv, self.init_k_KG, 144, True)
        R, m, xe, _ = self._probe_inputs()
        ue = dev(np.asarray(self.probe.ue, dtype=np.float64))
        P = dev(shell_record(prop))
        err = _lib.err_word()
        rc = lib.fe3d_quad4_kg(1, _lib.keep(dev(self._c(), np.int64)), _lib.ptr(tgt.init_k),
                               None, 0, None, 0, None, 0, _lib.ptr(R), _lib.ptr(m), _lib.ptr(xe),
                               _lib.ptr(ue), _lib.ptr(P), 1, None, _lib.ptr(tgt.r), _lib.ptr(tgt.c),
                               _lib.ptr(tgt.v), tgt.nk, _lib.ptr(err), _lib.stream_ptr())
        _lib.check(rc, 'Quad4.update_KG', err)
        tgt.finish()

    def update_KG_given_stress(self, Nxx, Nyy, Nxy, KGr, KGc, KGv):
        """Geometric stiffness of a constant stress state (Nxx, Nyy, Nxy) at
        init_k_KG (quad4.pyx:2259-3081); needs the frame and probe.xe."""
        lib = _lib.load()
        tgt = CooTarget(KGr, KGc, KGv, self.init_k_KG, 144, True)
        R, _, xe, _ = self._probe_inputs()
        ns = dev(np.array([Nxx, Nyy, Nxy], dtype=np.float64))
        err = _lib.err_word()
        rc = lib.fe3d_quad4_kg_given_stress(1, _lib.keep(dev(self._c(), np.int64)), _lib.ptr(tgt.init_k),
                                            None, 0, None, 0, _lib.ptr(R), _lib.ptr(xe), _lib.ptr(ns), 0,
                                            _lib.ptr(tgt.r), _lib.ptr(tgt.c), _lib.ptr(tgt.v), tgt.nk,
                                            _lib.ptr(err), _lib.stream_ptr())
        _lib.check(rc, 'Quad4.update_KG_given_stress', err)
        tgt.finish()

    def update_probe_finte(self, prop):
        """probe.finte = KC0e probe.ue in the element frame (quad4.pyx:1174-1201)."""
        lib = _lib.load()
        R, m, xe, area = self._probe_inputs()
        ue = dev(np.asarray(self.probe.ue, dtype=np.float64))
        P = dev(shell_record(prop))
        fe = dev(np.zeros(24))
        err = _lib.err_word()
        rc = lib.fe3d_quad4_finte(1, _lib.keep(dev(_LOCAL_C, np.int64)), _lib.ptr(R), _lib.ptr(m),
                                  _lib.ptr(xe), _lib.ptr(area), _lib.ptr(ue), _lib.ptr(P), 1, None, None, 0,
                                  _lib.ptr(fe), _lib.ptr(err), _lib.stream_ptr())
        _lib.check(rc, 'Quad4.update_probe_finte', err)
        self.probe.finte[:] = host(fe)

    def update_M(self, Mr, Mc, Mv, prop, mtype=0):
        """Mass matrix triplets, mtype 0/1/2 (quad4.pyx:3083-9489)."""
        if mtype not in (0, 1, 2):
            raise ValueError('mtype must be 0, 1 or 2')
        lib = _lib.load()
        size = 288 if mtype == 2 else 480
        tgt = CooTarget(Mr, Mc, Mv, self.init_k_M, size, True)
        R, _, xe, area = self._probe_inputs()
        P = dev(shell_record(prop))
        err = _lib.err_word()
        rc = lib.fe3d_quad4_m(1, _lib.keep(dev(self._c(), np.int64)), _lib.ptr(tgt.init_k), None, 0,
                              _lib.ptr(R), _lib.ptr(xe), _lib.ptr(area), _lib.ptr(P), 1, None,
                              _lib.ptr(tgt.r), _lib.ptr(tgt.c), _lib.ptr(tgt.v), tgt.nk, int(mtype),
                              _lib.ptr(err), _lib.stream_ptr())
        _lib.check(rc, 'Quad4.update_M', err)
        tgt.finish()

    def update_fint(self, fint, prop):
        """Internal forces R (KC0e ue) added at c1..c4 (quad4.pyx:1316-1362)."""
        lib = _lib.load()
        R, m, xe, area = self._probe_inputs()
        ue = dev(np.asarray(self.probe.ue, dtype=np.float64))
        P = dev(shell_record(prop))
        c = self._c()
        idx = (c[:, None] + np.arange(6)[None, :]).ravel()
        # the element's 24 entries of fint are gathered, accumulated by the
        # kernel on the device and scattered back (assignment only)
        f = dev(gather(fint, idx))
        err = _lib.err_word()
        rc = lib.fe3d_quad4_fint(1, _lib.keep(dev(_LOCAL_C, np.int64)), _lib.ptr(R), _lib.ptr(m),
                                 _lib.ptr(xe), _lib.ptr(area), _lib.ptr(ue), _lib.ptr(P), 1, None,
                                 _lib.ptr(f), 24, _lib.ptr(err), _lib.stream_ptr())
        _lib.check(rc, 'Quad4.update_fint', err)
        if _lib.is_cuda_tensor(fint):
            torch = _lib.torch_mod()
            fint[torch.as_tensor(idx, device=fint.device)] = f
        else:
            fint[idx] = host(f)
