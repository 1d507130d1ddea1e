"""Quad4R element with the API of ``pyfe3d.quad4r`` (pyfe3d/quad4r.pyx:108-15199).

Quad4R shares Quad4's frame, probes, geometric stiffness and mass
(quad4r.pyx:286-548, 4681-12788 restate quad4.pyx:491-752, 1365-9489); its
own parts are the reduced-integration KC0 with hourglass control and the
internal forces, computed by the ``fe3d_quad4r_*`` kernels.  For whole meshes
use :mod:`pyfe3d_gb300.batch` (``quad4r_update_KC0`` and friends).
"""
import numpy as np

from . import _lib
from ._elem import CooTarget, dev, gather, host
from .quad4 import DOF, NUM_NODES, Quad4, _LOCAL_C
from .shellprop import shell_record


class Quad4RData:
    """Sparse sizes per element (quad4r.pyx:108-146)."""

    def __init__(self):
        self.KC0_SPARSE_SIZE = 576
        self.KG_SPARSE_SIZE = 144
        self.M_SPARSE_SIZE = 480
        self.KA_BETA_SPARSE_SIZE = 144
        self.KA_GAMMA_SPARSE_SIZE = 144
        self.CA_SPARSE_SIZE = 144


class Quad4RProbe:
    """Per-probe buffers shared by the elements using it (quad4r.pyx:149-190)."""

    def __init__(self):
        self.xe = np.zeros(NUM_NODES * DOF // 2, dtype=np.float64)
        self.ue = np.zeros(NUM_NODES * DOF, dtype=np.float64)
        self.finte = np.zeros(NUM_NODES * DOF, dtype=np.float64)


class Quad4R(Quad4):
    """Quadrilateral shell with reduced integration and hourglass control
    (quad4r.pyx:193-284)."""

    def _hg(self, hgfactor_u, hgfactor_v, hgfactor_w, hgfactor_rx, hgfactor_ry):
        return dev(np.array([hgfactor_u, hgfactor_v, hgfactor_w, hgfactor_rx, hgfactor_ry], dtype=np.float64))

    def update_KC0(self, KC0r, KC0c, KC0v, prop, update_KC0v_only=0, hgfactor_u=1., hgfactor_v=1.,
                   hgfactor_w=1., hgfactor_rx=1., hgfactor_ry=1.):
        """Constitutive stiffness triplets at init_k_KC0 (quad4r.pyx:1145-4618)."""
        lib = _lib.load()
        tgt = CooTarget(KC0r, KC0c, KC0v, self.init_k_KC0, 576, update_KC0v_only == 0)
        R, m, xe, area = self._probe_inputs()
        k6 = dev(np.array([self.K6ROT]))
        hg = self._hg(hgfactor_u, hgfactor_v, hgfactor_w, hgfactor_rx, hgfactor_ry)
        P = dev(shell_record(prop))
        err = _lib.err_word()
        rc = lib.fe3d_quad4r_kc0(1, _lib.keep(dev(self._c(), np.int64)), _lib.ptr(tgt.init_k), None, 0, None, 0,
                                 _lib.ptr(R), _lib.ptr(m), _lib.ptr(xe), _lib.ptr(area), _lib.ptr(P), 1, None,
                                 _lib.ptr(k6), 0, _lib.ptr(hg), 0, _lib.ptr(tgt.r), _lib.ptr(tgt.c),
                                 _lib.ptr(tgt.v), tgt.nk, int(update_KC0v_only != 0), _lib.ptr(err),
                                 _lib.stream_ptr())
        _lib.check(rc, 'Quad4R.update_KC0', err)
        tgt.finish()

    def _finte(self, prop, fint, hgs, what):
        lib = _lib.load()
        R, m, xe, area = self._probe_inputs()
        k6 = dev(np.array([self.K6ROT]))
        hg = self._hg(*hgs)
        ue = dev(np.asarray(self.probe.ue, dtype=np.float64))
        P = dev(shell_record(prop))
        fe = dev(np.zeros(24))
        f = idx = None
        if fint is not None:
            c = self._c()
            idx = (c[:, None] + np.arange(6)[None, :]).ravel()
            f = dev(gather(fint, idx))
        err = _lib.err_word()
        rc = lib.fe3d_quad4r_finte(1, _lib.keep(dev(_LOCAL_C, np.int64)), _lib.ptr(R), _lib.ptr(m), _lib.ptr(xe),
                                   _lib.ptr(area), _lib.ptr(ue), _lib.ptr(P), 1, None, _lib.ptr(k6), 0,
                                   _lib.ptr(hg), 0, _lib.ptr(f), 24 if f is not None else 0, _lib.ptr(fe),
                                   _lib.ptr(err), _lib.stream_ptr())
        _lib.check(rc, what, err)
        self.probe.finte[:] = host(fe)
        if fint is not None:
            if _lib.is_cuda_tensor(fint):
                torch = _lib.torch_mod()
                fint[torch.as_tensor(idx, device=fint.device)] = f
            else:
                fint[idx] = host(f)

    def update_probe_finte(self, prop, hgfactor_u=1., hgfactor_v=1., hgfactor_w=1., hgfactor_rx=1.,
                           hgfactor_ry=1.):
        """probe.finte = KC0e probe.ue in the element frame (quad4r.pyx:549-1143)."""
        self._finte(prop, None, (hgfactor_u, hgfactor_v, hgfactor_w, hgfactor_rx, hgfactor_ry),
                    'Quad4R.update_probe_finte')

    def update_fint(self, fint, prop, hgfactor_u=1., hgfactor_v=1., hgfactor_w=1., hgfactor_rx=1.,
                    hgfactor_ry=1.):
        """Internal forces R (KC0e ue) added at c1..c4 (quad4r.pyx:4620-4679)."""
        self._finte(prop, fint, (hgfactor_u, hgfactor_v, hgfactor_w, hgfactor_rx, hgfactor_ry),
                    'Quad4R.update_fint')

    def update_KG(self, KGr, KGc, KGv, prop, update_KGv_only=0):
        """Geometric stiffness from probe.ue (quad4r.pyx:4681-5572, the Quad4 matrix)."""
        lib = _lib.load()
        write = update_KGv_only == 0
        tgt = CooTarget(KGr, KGc, KGv, self.init_k_KG, 144, write)
        R, m, xe, _ = self._probe_inputs()
        ue = dev(np.asarray(self.probe.ue, dtype=np.float64))
        P = dev(shell_record(prop))
        err = _lib.err_word()
        rc = lib.fe3d_quad4_kg(1, _lib.keep(dev(self._c(), np.int64)), _lib.ptr(tgt.init_k),
                               None, 0, None, 0, None, 0, _lib.ptr(R), _lib.ptr(m), _lib.ptr(xe),
                               _lib.ptr(ue), _lib.ptr(P), 1, None, _lib.ptr(tgt.r) if write else None,
                               _lib.ptr(tgt.c) if write else None, _lib.ptr(tgt.v), tgt.nk, _lib.ptr(err),
                               _lib.stream_ptr())
        _lib.check(rc, 'Quad4R.update_KG', err)
        tgt.finish()

    def update_KG_given_stress(self, Nxx, Nyy, Nxy, KGr, KGc, KGv, update_KGv_only=0):
        """Geometric stiffness of a constant stress state (quad4r.pyx:5574-6396)."""
        lib = _lib.load()
        write = update_KGv_only == 0
        tgt = CooTarget(KGr, KGc, KGv, self.init_k_KG, 144, write)
        R, _, xe, _ = self._probe_inputs()
        ns = dev(np.array([Nxx, Nyy, Nxy], dtype=np.float64))
        err = _lib.err_word()
        rc = lib.fe3d_quad4_kg_given_stress(1, _lib.keep(dev(self._c(), np.int64)), _lib.ptr(tgt.init_k),
                                            None, 0, None, 0, _lib.ptr(R), _lib.ptr(xe), _lib.ptr(ns), 0,
                                            _lib.ptr(tgt.r) if write else None, _lib.ptr(tgt.c) if write else None,
                                            _lib.ptr(tgt.v), tgt.nk, _lib.ptr(err), _lib.stream_ptr())
        _lib.check(rc, 'Quad4R.update_KG_given_stress', err)
        tgt.finish()
