"""BeamC element with the API of ``pyfe3d.beamc`` (pyfe3d/beamc.pyx:19-3152).

Every method computes on the GPU through ``libfe3d_gb300.so``; see
:mod:`pyfe3d_gb300.batch` for whole-mesh launches.
"""
import numpy as np

from . import _lib
from ._elem import CooTarget, dev, gather, host
from .shellprop import beam_record

DOF = 6
NUM_NODES = 2
_LOCAL_C = np.array([0, 6], dtype=np.int64)


class BeamCData:
    """Sparse sizes per element (beamc.pyx:23-46)."""

    def __init__(self):
        self.KC0_SPARSE_SIZE = 144
        self.KG_SPARSE_SIZE = 144
        self.M_SPARSE_SIZE = 144


class BeamCProbe:
    """Per-probe buffers (beamc.pyx:49-86)."""

    def __init__(self):
        self.xe = np.zeros(NUM_NODES * DOF // 2, dtype=np.float64)
        self.ue = np.zeros(NUM_NODES * DOF, dtype=np.float64)
        self.finte = np.zeros(NUM_NODES * DOF, dtype=np.float64)


class BeamC:
    """Timoshenko 3D beam with consistent shape functions (beamc.pyx:89-156)."""

    def __init__(self, p):
        self.probe = p
        self.eid = -1
        self.pid = -1
        self.n1 = self.n2 = -1
        self.c1 = self.c2 = -1
        self.init_k_KC0 = 0
        self.init_k_KG = 0
        self.init_k_M = 0
        self.length = 0.
        self.vxyi = self.vxyj = self.vxyk = 0.
        self.r11 = self.r12 = self.r13 = 0.
        self.r21 = self.r22 = self.r23 = 0.
        self.r31 = self.r32 = self.r33 = 0.

    def _c(self):
        return np.array([self.c1, self.c2], dtype=np.int64)

    def _R(self):
        return np.array([self.r11, self.r12, self.r13, self.r21, self.r22, self.r23,
                         self.r31, self.r32, self.r33])

    def _coords(self, x):
        c = self._c()
        if (c < 0).any():
            raise ValueError('BeamC DOF offsets c1, c2 are not set')
        idx = (c // 2)[:, None] + np.arange(3)[None, :]
        return dev(gather(x, idx.ravel()))

    def update_rotation_matrix(self, vxyi, vxyj, vxyk, x):
        """Beam frame from the axis and the vector vxy (beamc.pyx:158-231)."""
        lib = _lib.load()
        self.vxyi, self.vxyj, self.vxyk = float(vxyi), float(vxyj), float(vxyk)
        xs = self._coords(x)
        vxy = dev(np.array([vxyi, vxyj, vxyk], dtype=np.float64))
        R = dev(np.zeros(9))
        err = _lib.err_word()
        rc = lib.fe3d_beamc_frame(1, _lib.keep(dev(_LOCAL_C, np.int64)), _lib.ptr(xs), 6,
                                  _lib.ptr(vxy), 0, _lib.ptr(R), None, None, _lib.ptr(err),
                                  _lib.stream_ptr())
        _lib.check(rc, 'BeamC.update_rotation_matrix', err)
        (self.r11, self.r12, self.r13, self.r21, self.r22, self.r23,
         self.r31, self.r32, self.r33) = (float(v) for v in host(R))

    def update_probe_xe(self, x):
        """Local coordinates and length (beamc.pyx:287-349)."""
        lib = _lib.load()
        xs = self._coords(x)
        xe = dev(np.zeros(6))
        L = dev(np.zeros(1))
        err = _lib.err_word()
        rc = lib.fe3d_beamc_probe_xe(1, _lib.keep(dev(_LOCAL_C, np.int64)), _lib.ptr(xs), 6,
                                     _lib.keep(dev(self._R())), _lib.ptr(xe), _lib.ptr(L),
                                     _lib.ptr(err), _lib.stream_ptr())
        _lib.check(rc, 'BeamC.update_probe_xe', err)
        self.probe.xe[:] = host(xe)
        self.length = float(host(L)[0])

    def update_length(self):
        """Length from the local coordinates held by the probe (beamc.pyx:336-349)."""
        lib = _lib.load()
        L = dev(np.zeros(1))
        err = _lib.err_word()
        rc = lib.fe3d_beamc_probe_xe(1, _lib.keep(dev(_LOCAL_C, np.int64)),
                                     _lib.keep(dev(np.asarray(self.probe.xe, dtype=np.float64))), 6,
                                     _lib.keep(dev(np.eye(3).ravel())), None, _lib.ptr(L),
                                     _lib.ptr(err), _lib.stream_ptr())
        _lib.check(rc, 'BeamC.update_length', err)
        self.length = float(host(L)[0])

    def update_probe_ue(self, u):
        """Local displacements R^T u (beamc.pyx:234-284)."""
        lib = _lib.load()
        c = self._c()
        idx = (c[:, None] + np.arange(6)[None, :]).ravel()
        us = dev(gather(u, idx))
        ue = dev(np.zeros(12))
        err = _lib.err_word()
        rc = lib.fe3d_beamc_probe_ue(1, _lib.keep(dev(_LOCAL_C, np.int64)), _lib.ptr(us), 12,
                                     _lib.keep(dev(self._R())), _lib.ptr(ue), _lib.ptr(err),
                                     _lib.stream_ptr())
        _lib.check(rc, 'BeamC.update_probe_ue', err)
        self.probe.ue[:] = host(ue)

    def _common(self):
        return dev(self._R()), dev(np.array([self.length]))

    def update_KC0(self, KC0r, KC0c, KC0v, prop, update_KC0v_only=0):
        """Constitutive stiffness (beamc.pyx:489-1352)."""
        lib = _lib.load()
        tgt = CooTarget(KC0r, KC0c, KC0v, self.init_k_KC0, 144, update_KC0v_only == 0)
        R, L = self._common()
        P = dev(beam_record(prop))
        err = _lib.err_word()
        rc = lib.fe3d_beamc_kc0(1, _lib.keep(dev(self._c(), np.int64)), _lib.ptr(tgt.init_k),
                                _lib.ptr(R), _lib.ptr(L), _lib.ptr(P), 1, None, _lib.ptr(tgt.r),
                                _lib.ptr(tgt.c), _lib.ptr(tgt.v), tgt.nk, int(update_KC0v_only != 0),
                                _lib.ptr(err), _lib.stream_ptr())
        _lib.check(rc, 'BeamC.update_KC0', err)
        tgt.finish()

    def update_KG(self, KGr, KGc, KGv, prop, update_KGv_only=0):
        """Geometric stiffness from probe.ue; indices written when the flag is 0
        (beamc.pyx:1392-2179, following the code at :1451)."""
        lib = _lib.load()
        tgt = CooTarget(KGr, KGc, KGv, self.init_k_KG, 144, update_KGv_only == 0)
        R, L = self._common()
        ue = dev(np.asarray(self.probe.ue, dtype=np.float64))
        P = dev(beam_record(prop))
        err = _lib.err_word()
        rc = lib.fe3d_beamc_kg(1, _lib.keep(dev(self._c(), np.int64)), _lib.ptr(tgt.init_k),
                               _lib.ptr(R), _lib.ptr(L), _lib.ptr(ue), _lib.ptr(P), 1, None,
                               _lib.ptr(tgt.r), _lib.ptr(tgt.c), _lib.ptr(tgt.v), tgt.nk,
                               int(update_KGv_only != 0), _lib.ptr(err), _lib.stream_ptr())
        _lib.check(rc, 'BeamC.update_KG', err)
        tgt.finish()

    def update_probe_finte(self, prop):
        """probe.finte = KC0e probe.ue in the element frame (beamc.pyx:352-486)."""
        self._finte(None, prop)

    def update_fint(self, fint, prop):
        """Internal forces R finte added at c1, c2 (beamc.pyx:1354-1390);
        probe.finte is updated as in the reference."""
        self._finte(fint, prop)

    def _finte(self, fint, prop):
        lib = _lib.load()
        R, L = self._common()
        ue = dev(np.asarray(self.probe.ue, dtype=np.float64))
        P = dev(beam_record(prop))
        fe = dev(np.zeros(12))
        f = None
        if fint is not None:
            c = self._c()
            idx = (c[:, None] + np.arange(6)[None, :]).ravel()
            # the element's 12 entries are gathered, accumulated on the device
            # and written back
            f = dev(gather(fint, idx))
        err = _lib.err_word()
        # local offsets into the gathered 12 entries
        rc = lib.fe3d_beamc_fint(1, _lib.keep(dev(np.array([0, 6]), np.int64)), _lib.ptr(R), _lib.ptr(L),
                                 _lib.ptr(ue), _lib.ptr(P), 1, None, _lib.ptr(f), 12, _lib.ptr(fe),
                                 _lib.ptr(err), _lib.stream_ptr())
        _lib.check(rc, 'BeamC.update_fint', err)
        self.probe.finte[:] = host(fe)
        if f is not None:
            if _lib.is_cuda_tensor(fint):
                torch = _lib.torch_mod()
                fint[torch.as_tensor(idx, device=fint.device)] = f
            else:
                fint[idx] = host(f)

    def update_M(self, Mr, Mc, Mv, prop, mtype=0):
        """Mass matrix, mtype 0 consistent / 1 lumped (beamc.pyx:2181-3152)."""
        if mtype not in (0, 1):
            raise ValueError('mtype must be 0 or 1')
        lib = _lib.load()
        size = 144 if mtype == 0 else 36
        tgt = CooTarget(Mr, Mc, Mv, self.init_k_M, size, True)
        R, L = self._common()
        P = dev(beam_record(prop))
        err = _lib.err_word()
        rc = lib.fe3d_beamc_m(1, _lib.keep(dev(self._c(), np.int64)), _lib.ptr(tgt.init_k),
                              _lib.ptr(R), _lib.ptr(L), _lib.ptr(P), 1, None, _lib.ptr(tgt.r),
                              _lib.ptr(tgt.c), _lib.ptr(tgt.v), tgt.nk, int(mtype), _lib.ptr(err),
                              _lib.stream_ptr())
        _lib.check(rc, 'BeamC.update_M', err)
        tgt.finish()
