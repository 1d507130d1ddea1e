"""Whole-mesh element updates: one kernel launch for all elements.

These functions do what a loop of ``Quad4``/``BeamC`` method calls does in
the reference (frame -> probe -> matrix per element, pyfe3d tests such as
tests/test_quad4_static_point_load.py:53-78), over structure-of-arrays
element data:

  cdof    int64 (E, 4) / (E, 2)  DOF offsets c1..c4 (6 x node position)
  init_k  int64 (E,)             first sparse slot of each element
  props   float64 (P, 28)/(P,16) property records (see shellprop.shell_record)
  pid     int32 (E,) or None     record index per element (None: record e)

Inputs may be numpy arrays or CUDA tensors.  COO outputs that are CUDA
tensors are updated in place (zero copy); numpy outputs are copied to the
device, updated and copied back, as the reference's ``+=`` semantics need
their current values.
"""
import ctypes

import numpy as np

from . import _lib
from .shellprop import BEAM_PROP_STRIDE, SHELL_PROP_STRIDE


def _dev(a, dtype):
    return None if a is None else _lib.to_device(a, dtype)


def _props(props, stride):
    P = _dev(props, np.float64)
    if P.dim() == 1:
        P = P.reshape(1, -1)
    if P.shape[1] != stride:
        raise ValueError('property records must have %d columns, got %d' % (stride, P.shape[1]))
    return P.contiguous()


def _pid(pid, P, E):
    """Element -> record map; with pid None a single record is shared by all
    elements, otherwise record e belongs to element e."""
    if pid is None:
        if P.shape[0] == 1 and E > 1:
            torch = _lib.torch_mod()
            return torch.zeros(E, dtype=torch.int32, device=P.device)
        return None
    return _dev(pid, np.int32)


class _Out:
    """COO output arrays on the device (in place when already CUDA tensors)."""

    def __init__(self, Kr, Kc, Kv, need_idx):
        torch = _lib.torch_mod()
        self.host = not _lib.is_cuda_tensor(Kv)
        self.src = (Kr, Kc, Kv)
        self.need_idx = need_idx
        self.torch_host = isinstance(Kv, torch.Tensor) and not Kv.is_cuda
        if self.torch_host:
            # CPU tensors (pinned for asynchronous copies)
            dev = _lib.device()
            for t, dt in ((Kv, torch.float64), (Kr, torch.int64), (Kc, torch.int64)):
                if t is not None and (t.dtype != dt or not t.is_contiguous()):
                    raise TypeError('COO tensors must be contiguous int64/float64 tensors')
            self.v = Kv.to(dev, non_blocking=True)
            if need_idx:
                # slots no element writes keep the caller's indices
                self.r = Kr.to(dev, non_blocking=True)
                self.c = Kc.to(dev, non_blocking=True)
            else:
                self.r = self.c = None
        elif self.host:
            if not (isinstance(Kv, np.ndarray) and Kv.dtype == np.float64 and Kv.flags.c_contiguous):
                raise TypeError('value array must be a contiguous float64 numpy array or CUDA tensor')
            self.v = _lib.to_device(Kv, np.float64)
            if need_idx:
                for a in (Kr, Kc):
                    if not (isinstance(a, np.ndarray) and a.dtype == np.int64):
                        raise TypeError('row/column arrays must be int64')
                self.r = torch.empty(len(Kr), dtype=torch.int64, device=self.v.device)
                self.c = torch.empty(len(Kc), dtype=torch.int64, device=self.v.device)
                self.r.copy_(torch.from_numpy(Kr))
                self.c.copy_(torch.from_numpy(Kc))
            else:
                self.r = self.c = None
        else:
            for t, dt in ((Kv, torch.float64), (Kr, torch.int64), (Kc, torch.int64)):
                if t is None:
                    continue
                if t.dtype != dt or not t.is_contiguous():
                    raise TypeError('COO tensors must be contiguous int64/float64 CUDA tensors')
            self.v, self.r, self.c = Kv, Kr, Kc
        n = len(Kv)
        if need_idx and (len(Kr) < n or len(Kc) < n):
            raise ValueError('row/column arrays shorter than the value array')
        self.n = n

    def finish(self):
        if self.torch_host:
            Kr, Kc, Kv = self.src
            Kv.copy_(self.v, non_blocking=True)
            if self.need_idx:
                Kr.copy_(self.r, non_blocking=True)
                Kc.copy_(self.c, non_blocking=True)
            _lib.torch_mod().cuda.current_stream().synchronize()
        elif self.host:
            Kr, Kc, Kv = self.src
            Kv[:] = self.v.cpu().numpy()
            if self.need_idx:
                Kr[:] = self.r.cpu().numpy()
                Kc[:] = self.c.cpu().numpy()


def _check_init_k(init_k, size, n):
    if init_k.numel() and n < size:
        raise IndexError('sparse arrays shorter than one element block')


def quad4_frames(x, cdof, xmat=None, m=None, check=True):
    """update_rotation_matrix + update_probe_xe for all elements.

    Returns device tensors R (E, 9), m (E, 4), xe (E, 12), area (E,).
    """
    lib = _lib.load()
    torch = _lib.torch_mod()
    x = _dev(x, np.float64)
    cdof = _dev(cdof, np.int64).reshape(-1, 4).contiguous()
    E = cdof.shape[0]
    dev = x.device
    R = torch.empty((E, 9), dtype=torch.float64, device=dev)
    mm = (torch.tensor([1., 0., 0., 1.], dtype=torch.float64, device=dev).repeat(E, 1)
          if m is None else _dev(m, np.float64).reshape(E, 4).clone())
    xe = torch.empty((E, 12), dtype=torch.float64, device=dev)
    area = torch.empty(E, dtype=torch.float64, device=dev)
    xm, stride = _xmat(xmat, E)
    err = _lib.err_word()
    rc = lib.fe3d_quad4_frame(E, _lib.ptr(cdof), _lib.ptr(x), x.numel(), _lib.ptr(xm), stride,
                              _lib.ptr(R), _lib.ptr(mm), _lib.ptr(xe), _lib.ptr(area),
                              _lib.ptr(err), _lib.stream_ptr())
    _lib.check(rc, 'quad4_frames', err if check else None)
    return R, mm, xe, area


def _xmat(xmat, E):
    if xmat is None:
        return None, 0
    xm = _dev(xmat, np.float64)
    if xm.numel() == 3:
        return xm.reshape(3), 0
    if xm.numel() != 3 * E:
        raise ValueError('xmat must have 3 or 3*E entries')
    return xm.reshape(E, 3).contiguous(), 3


def _host_array(a, dtype):
    """Contiguous host view (numpy) of a numpy array or CPU tensor of dtype, else None."""
    torch = _lib.torch_mod()
    if isinstance(a, torch.Tensor):
        if a.is_cuda or a.dtype != {np.float64: torch.float64, np.int64: torch.int64,
                                    np.int32: torch.int32}[dtype] or not a.is_contiguous():
            return None
        return a.numpy()
    if isinstance(a, np.ndarray) and a.dtype == dtype and a.flags.c_contiguous:
        return a
    return None


def _quad4_kc0_host(KC0r, KC0c, KC0v, x, cdof, init_k, props, pid, values_only, check):
    """The pipelined host-buffer path (fe3d_quad4_kc0_host) when every array
    is in host memory with the reference's contiguous offsets; returns False
    to fall back to the device path."""
    lib = _lib.load()
    Kv = _host_array(KC0v, np.float64)
    Kr = None if values_only else _host_array(KC0r, np.int64)
    Kc = None if values_only else _host_array(KC0c, np.int64)
    if Kv is None or (not values_only and (Kr is None or Kc is None)):
        return False
    xh = _host_array(x, np.float64) if not isinstance(x, np.ndarray) else np.ascontiguousarray(x, np.float64)
    ch = _host_array(cdof, np.int64) if not isinstance(cdof, np.ndarray) else np.ascontiguousarray(cdof, np.int64)
    ih = _host_array(init_k, np.int64) if not isinstance(init_k, np.ndarray) else \
        np.ascontiguousarray(init_k, np.int64)
    Ph = _host_array(props, np.float64) if not isinstance(props, np.ndarray) else \
        np.ascontiguousarray(props, np.float64)
    if xh is None or ch is None or ih is None or Ph is None:
        return False
    Ph = Ph.reshape(-1, SHELL_PROP_STRIDE) if Ph.size % SHELL_PROP_STRIDE == 0 else None
    if Ph is None:
        return False
    E = ch.size // 4
    if ih.size != E or (not values_only and (len(Kr) < len(Kv) or len(Kc) < len(Kv))):
        return False
    if pid is None and Ph.shape[0] == 1 and E > 1:
        ph = np.zeros(E, dtype=np.int32)
    elif pid is None:
        ph = None
    else:
        ph = _host_array(pid, np.int32) if not isinstance(pid, np.ndarray) else np.ascontiguousarray(pid, np.int32)
        if ph is None:
            return False
    err = ctypes.c_int(0)
    ptr = lambda a: None if a is None else a.ctypes.data
    rc = lib.fe3d_quad4_kc0_host(E, ptr(ch), ptr(ih), ptr(xh), xh.size, ptr(Ph), Ph.shape[0], ptr(ph),
                                 ptr(Kr), ptr(Kc), ptr(Kv), Kv.size, int(values_only), 0, ctypes.byref(err),
                                 _lib.stream_ptr())
    if rc == -1:  # not the contiguous layout: the device path handles it
        return False
    _lib.check(rc, 'quad4_update_KC0')
    if check and err.value:
        raise _lib.Fe3dError('quad4_update_KC0: device reported error bits 0x%x (an offset outside the '
                             'caller\'s buffers)' % err.value)
    return True


def quad4_update_KC0(KC0r, KC0c, KC0v, x, cdof, init_k, props, pid=None, xmat=None,
                     update_KC0v_only=0, check=True):
    """Quad4.update_KC0 over all elements, frame computed on the fly.  Host
    arrays (numpy or CPU tensors, pinned for full speed) with the reference's
    contiguous offsets stream through the GPU in overlapped chunks."""
    lib = _lib.load()
    if xmat is None and not _lib.is_cuda_tensor(KC0v) and \
            _quad4_kc0_host(KC0r, KC0c, KC0v, x, cdof, init_k, props, pid, update_KC0v_only != 0, check):
        return
    x = _dev(x, np.float64)
    cdof = _dev(cdof, np.int64).reshape(-1, 4).contiguous()
    init_k = _dev(init_k, np.int64).reshape(-1).contiguous()
    E = cdof.shape[0]
    if init_k.numel() != E:
        raise ValueError('init_k must have one entry per element')
    P = _props(props, SHELL_PROP_STRIDE)
    pid = _pid(pid, P, cdof.shape[0])
    out = _Out(KC0r, KC0c, KC0v, update_KC0v_only == 0)
    xm, stride = _xmat(xmat, E)
    err = _lib.err_word()
    rc = lib.fe3d_quad4_kc0(E, _lib.ptr(cdof), _lib.ptr(init_k), _lib.ptr(x), x.numel(),
                            _lib.ptr(xm), stride, None, None, None, None, _lib.ptr(P), P.shape[0],
                            _lib.ptr(pid), _lib.ptr(out.r), _lib.ptr(out.c), _lib.ptr(out.v), out.n,
                            int(update_KC0v_only != 0), _lib.ptr(err), _lib.stream_ptr())
    _lib.check(rc, 'quad4_update_KC0', err if check else None)
    out.finish()


def quad4_update_KC0_csr(vals, fmap, x, props, pid=None, xmat=None, group=0, mode='assign', check=True):
    """Quad4.update_KC0 of group ``group`` of a :class:`~pyfe3d_gb300.solver.FusedMap`
    added straight into the reduced CSR values ``vals`` (no triplets): the
    fused replacement of update_KC0 + coo_matrix(...).tocsc() + K[bu][:, bu]
    (tests/test_quad4_static_point_load.py:74-99).  ``pid`` and ``xmat``
    follow the group's element order."""
    lib = _lib.load()
    if fmap.nn[group] != 4:
        raise ValueError('group %d is not a Quad4 group' % group)
    E = fmap.E[group]
    x = _dev(x, np.float64)
    P = _props(props, SHELL_PROP_STRIDE)
    pid = _pid(pid, P, E)
    xm, stride = _xmat(xmat, E)
    if not (_lib.is_cuda_tensor(vals) and vals.dtype == _lib.torch_mod().float64 and vals.is_contiguous()
            and vals.numel() == fmap.pattern.nnz):
        raise TypeError('vals must be a contiguous float64 CUDA tensor of the pattern\'s %d entries'
                        % fmap.pattern.nnz)
    err = _lib.err_word()
    rc = lib.fe3d_quad4_kc0_csr(fmap.handle, int(group), _lib.ptr(x), x.numel(), _lib.ptr(xm), stride, _lib.ptr(P),
                                P.shape[0], _lib.ptr(pid), _lib.ptr(vals), fmap.MODES[mode], _lib.ptr(err),
                                _lib.stream_ptr())
    _lib.check(rc, 'quad4_update_KC0_csr', err if check else None)
    return vals


def quad4_update_KG(KGr, KGc, KGv, x, u, cdof, init_k, props, pid=None, xmat=None, check=True):
    """Quad4.update_probe_ue + update_KG over all elements from the global u."""
    lib = _lib.load()
    x = _dev(x, np.float64)
    u = _dev(u, np.float64)
    cdof = _dev(cdof, np.int64).reshape(-1, 4).contiguous()
    init_k = _dev(init_k, np.int64).reshape(-1).contiguous()
    E = cdof.shape[0]
    P = _props(props, SHELL_PROP_STRIDE)
    pid = _pid(pid, P, cdof.shape[0])
    out = _Out(KGr, KGc, KGv, True)
    xm, stride = _xmat(xmat, E)
    err = _lib.err_word()
    rc = lib.fe3d_quad4_kg(E, _lib.ptr(cdof), _lib.ptr(init_k), _lib.ptr(x), x.numel(), _lib.ptr(xm),
                           stride, _lib.ptr(u), u.numel(), None, None, None, None, _lib.ptr(P),
                           P.shape[0], _lib.ptr(pid), _lib.ptr(out.r), _lib.ptr(out.c),
                           _lib.ptr(out.v), out.n, _lib.ptr(err), _lib.stream_ptr())
    _lib.check(rc, 'quad4_update_KG', err if check else None)
    out.finish()


def quad4_update_KG_given_stress(KGr, KGc, KGv, x, cdof, init_k, nstress, xmat=None, check=True):
    """Quad4.update_KG_given_stress over all elements: ``nstress`` holds
    (Nxx, Nyy, Nxy) per element, shape (E, 3), or one triplet for all."""
    lib = _lib.load()
    x = _dev(x, np.float64)
    cdof = _dev(cdof, np.int64).reshape(-1, 4).contiguous()
    init_k = _dev(init_k, np.int64).reshape(-1).contiguous()
    E = cdof.shape[0]
    ns = _dev(nstress, np.float64).reshape(-1).contiguous()
    if ns.numel() not in (3, 3 * E):
        raise ValueError('nstress must have 3 or 3*E entries')
    out = _Out(KGr, KGc, KGv, True)
    xm, stride = _xmat(xmat, E)
    err = _lib.err_word()
    rc = lib.fe3d_quad4_kg_given_stress(E, _lib.ptr(cdof), _lib.ptr(init_k), _lib.ptr(x), x.numel(),
                                        _lib.ptr(xm), stride, None, None, _lib.ptr(ns),
                                        3 if ns.numel() == 3 * E and E > 1 else 0, _lib.ptr(out.r),
                                        _lib.ptr(out.c), _lib.ptr(out.v), out.n, _lib.ptr(err),
                                        _lib.stream_ptr())
    _lib.check(rc, 'quad4_update_KG_given_stress', err if check else None)
    out.finish()


def quad4_update_fint(fint, x, u, cdof, props, pid=None, xmat=None, check=True):
    """Quad4.update_probe_ue + update_fint over all elements: fint += the
    internal forces R (KC0e ue) of every element (fint: numpy or CUDA)."""
    lib = _lib.load()
    torch = _lib.torch_mod()
    x = _dev(x, np.float64)
    u = _dev(u, np.float64)
    cdof = _dev(cdof, np.int64).reshape(-1, 4).contiguous()
    E = cdof.shape[0]
    R, m, xe, area = quad4_frames(x, cdof, xmat=xmat, check=check)
    ue = torch.empty((E, 24), dtype=torch.float64, device=u.device)
    err = _lib.err_word()
    rc = lib.fe3d_quad4_probe_ue(E, _lib.ptr(cdof), _lib.ptr(u), u.numel(), _lib.ptr(R), _lib.ptr(ue),
                                 _lib.ptr(err), _lib.stream_ptr())
    _lib.check(rc, 'quad4_probe_ue')
    P = _props(props, SHELL_PROP_STRIDE)
    pid = _pid(pid, P, E)
    f = fint if _lib.is_cuda_tensor(fint) else _dev(fint, np.float64)
    rc = lib.fe3d_quad4_fint(E, _lib.ptr(cdof), _lib.ptr(R), _lib.ptr(m), _lib.ptr(xe), _lib.ptr(area),
                             _lib.ptr(ue), _lib.ptr(P), P.shape[0], _lib.ptr(pid), _lib.ptr(f), f.numel(),
                             _lib.ptr(err), _lib.stream_ptr())
    _lib.check(rc, 'quad4_update_fint', err if check else None)
    if not _lib.is_cuda_tensor(fint):
        fint[:] = f.cpu().numpy()


def quad4_update_M(Mr, Mc, Mv, x, cdof, init_k, props, pid=None, mtype=0, check=True):
    """Quad4.update_M over all elements (mtype 0, 1 or 2)."""
    if mtype not in (0, 1, 2):
        raise ValueError('mtype must be 0, 1 or 2')
    lib = _lib.load()
    x = _dev(x, np.float64)
    cdof = _dev(cdof, np.int64).reshape(-1, 4).contiguous()
    init_k = _dev(init_k, np.int64).reshape(-1).contiguous()
    E = cdof.shape[0]
    P = _props(props, SHELL_PROP_STRIDE)
    pid = _pid(pid, P, cdof.shape[0])
    out = _Out(Mr, Mc, Mv, True)
    err = _lib.err_word()
    rc = lib.fe3d_quad4_m(E, _lib.ptr(cdof), _lib.ptr(init_k), _lib.ptr(x), x.numel(), None, None,
                          None, _lib.ptr(P), P.shape[0], _lib.ptr(pid), _lib.ptr(out.r),
                          _lib.ptr(out.c), _lib.ptr(out.v), out.n, int(mtype), _lib.ptr(err),
                          _lib.stream_ptr())
    _lib.check(rc, 'quad4_update_M', err if check else None)
    out.finish()


def beamc_frames(x, cdof, vxy, check=True):
    """BeamC update_rotation_matrix + update_probe_xe for all elements.

    Returns device tensors R (E, 9), xe (E, 6), length (E,)."""
    lib = _lib.load()
    torch = _lib.torch_mod()
    x = _dev(x, np.float64)
    cdof = _dev(cdof, np.int64).reshape(-1, 2).contiguous()
    E = cdof.shape[0]
    v = _dev(vxy, np.float64)
    stride = 0 if v.numel() == 3 else 3
    if stride == 3 and v.numel() != 3 * E:
        raise ValueError('vxy must have 3 or 3*E entries')
    R = torch.empty((E, 9), dtype=torch.float64, device=x.device)
    xe = torch.empty((E, 6), dtype=torch.float64, device=x.device)
    L = torch.empty(E, dtype=torch.float64, device=x.device)
    err = _lib.err_word()
    rc = lib.fe3d_beamc_frame(E, _lib.ptr(cdof), _lib.ptr(x), x.numel(), _lib.ptr(v), stride,
                              _lib.ptr(R), _lib.ptr(xe), _lib.ptr(L), _lib.ptr(err),
                              _lib.stream_ptr())
    _lib.check(rc, 'beamc_frames', err if check else None)
    return R, xe, L


def beamc_update_KC0(KC0r, KC0c, KC0v, x, cdof, init_k, vxy, props, pid=None,
                     update_KC0v_only=0, check=True):
    lib = _lib.load()
    R, _, L = beamc_frames(x, cdof, vxy, check)
    cdof = _dev(cdof, np.int64).reshape(-1, 2).contiguous()
    init_k = _dev(init_k, np.int64).reshape(-1).contiguous()
    P = _props(props, BEAM_PROP_STRIDE)
    pid = _pid(pid, P, cdof.shape[0])
    out = _Out(KC0r, KC0c, KC0v, update_KC0v_only == 0)
    err = _lib.err_word()
    rc = lib.fe3d_beamc_kc0(cdof.shape[0], _lib.ptr(cdof), _lib.ptr(init_k), _lib.ptr(R), _lib.ptr(L),
                            _lib.ptr(P), P.shape[0], _lib.ptr(pid), _lib.ptr(out.r), _lib.ptr(out.c),
                            _lib.ptr(out.v), out.n, int(update_KC0v_only != 0), _lib.ptr(err),
                            _lib.stream_ptr())
    _lib.check(rc, 'beamc_update_KC0', err if check else None)
    out.finish()


def beamc_update_KG(KGr, KGc, KGv, x, u, cdof, init_k, vxy, props, pid=None, update_KGv_only=0,
                    check=True):
    lib = _lib.load()
    torch = _lib.torch_mod()
    R, _, L = beamc_frames(x, cdof, vxy, check)
    cdof = _dev(cdof, np.int64).reshape(-1, 2).contiguous()
    E = cdof.shape[0]
    u = _dev(u, np.float64)
    ue = torch.empty((E, 12), dtype=torch.float64, device=u.device)
    err = _lib.err_word()
    rc = lib.fe3d_beamc_probe_ue(E, _lib.ptr(cdof), _lib.ptr(u), u.numel(), _lib.ptr(R), _lib.ptr(ue),
                                 _lib.ptr(err), _lib.stream_ptr())
    _lib.check(rc, 'beamc_probe_ue')
    init_k = _dev(init_k, np.int64).reshape(-1).contiguous()
    P = _props(props, BEAM_PROP_STRIDE)
    pid = _pid(pid, P, cdof.shape[0])
    out = _Out(KGr, KGc, KGv, update_KGv_only == 0)
    rc = lib.fe3d_beamc_kg(E, _lib.ptr(cdof), _lib.ptr(init_k), _lib.ptr(R), _lib.ptr(L), _lib.ptr(ue),
                           _lib.ptr(P), P.shape[0], _lib.ptr(pid), _lib.ptr(out.r), _lib.ptr(out.c),
                           _lib.ptr(out.v), out.n, int(update_KGv_only != 0), _lib.ptr(err),
                           _lib.stream_ptr())
    _lib.check(rc, 'beamc_update_KG', err if check else None)
    out.finish()


def beamc_update_fint(fint, x, u, cdof, vxy, props, pid=None, check=True):
    """BeamC.update_probe_ue + update_fint over all elements; returns the
    local internal forces finte (E, 12) as well."""
    lib = _lib.load()
    torch = _lib.torch_mod()
    R, _, L = beamc_frames(x, cdof, vxy, check)
    cdof = _dev(cdof, np.int64).reshape(-1, 2).contiguous()
    E = cdof.shape[0]
    u = _dev(u, np.float64)
    ue = torch.empty((E, 12), dtype=torch.float64, device=u.device)
    err = _lib.err_word()
    rc = lib.fe3d_beamc_probe_ue(E, _lib.ptr(cdof), _lib.ptr(u), u.numel(), _lib.ptr(R), _lib.ptr(ue),
                                 _lib.ptr(err), _lib.stream_ptr())
    _lib.check(rc, 'beamc_probe_ue')
    P = _props(props, BEAM_PROP_STRIDE)
    pid = _pid(pid, P, E)
    f = fint if _lib.is_cuda_tensor(fint) else _dev(fint, np.float64)
    finte = torch.empty((E, 12), dtype=torch.float64, device=u.device)
    rc = lib.fe3d_beamc_fint(E, _lib.ptr(cdof), _lib.ptr(R), _lib.ptr(L), _lib.ptr(ue), _lib.ptr(P),
                             P.shape[0], _lib.ptr(pid), _lib.ptr(f), f.numel(), _lib.ptr(finte), _lib.ptr(err),
                             _lib.stream_ptr())
    _lib.check(rc, 'beamc_update_fint', err if check else None)
    if not _lib.is_cuda_tensor(fint):
        fint[:] = f.cpu().numpy()
    return finte


def beamc_update_M(Mr, Mc, Mv, x, cdof, init_k, vxy, props, pid=None, mtype=0, check=True):
    if mtype not in (0, 1):
        raise ValueError('mtype must be 0 or 1')
    lib = _lib.load()
    R, _, L = beamc_frames(x, cdof, vxy, check)
    cdof = _dev(cdof, np.int64).reshape(-1, 2).contiguous()
    init_k = _dev(init_k, np.int64).reshape(-1).contiguous()
    P = _props(props, BEAM_PROP_STRIDE)
    pid = _pid(pid, P, cdof.shape[0])
    out = _Out(Mr, Mc, Mv, True)
    err = _lib.err_word()
    rc = lib.fe3d_beamc_m(cdof.shape[0], _lib.ptr(cdof), _lib.ptr(init_k), _lib.ptr(R), _lib.ptr(L),
                          _lib.ptr(P), P.shape[0], _lib.ptr(pid), _lib.ptr(out.r), _lib.ptr(out.c),
                          _lib.ptr(out.v), out.n, int(mtype), _lib.ptr(err), _lib.stream_ptr())
    _lib.check(rc, 'beamc_update_M', err if check else None)
    out.finish()


# --------------------------------------------------------- Tria3R / Quad4R
# Reduced-integration shells (pyfe3d/tria3r.pyx, pyfe3d/quad4r.pyx).  k6rot
# (K6ROT), alpha (Tria3R.alpha_shear_locking) and hg (Quad4R hourglass
# factors u, v, w, rx, ry) are one value / one 5-vector for all elements or
# one per element.  Quad4R's frame, probes, KG, KG of given stress and mass
# are the Quad4 ones (quad4r.pyx:286-548, 4681-12788): quad4r_update_KG and
# friends below are the Quad4 functions.

def _per_elem(v, E, width, name):
    t = _dev(np.asarray(v, dtype=np.float64) if not _lib.is_cuda_tensor(v) else v, np.float64).reshape(-1)
    if t.numel() == width:
        return t.contiguous(), 0
    if t.numel() != width * E:
        raise ValueError('%s must have %d or %d entries' % (name, width, width * E))
    return t.contiguous(), width


def tria3r_frames(x, cdof, xmat=None, m=None, check=True):
    """Tria3R update_rotation_matrix + update_probe_xe for all elements.

    Returns device tensors R (E, 9), m (E, 4), xe (E, 9), area (E,)."""
    lib = _lib.load()
    torch = _lib.torch_mod()
    x = _dev(x, np.float64)
    cdof = _dev(cdof, np.int64).reshape(-1, 3).contiguous()
    E = cdof.shape[0]
    dev = x.device
    R = torch.empty((E, 9), dtype=torch.float64, device=dev)
    mm = (torch.tensor([1., 0., 0., 1.], dtype=torch.float64, device=dev).repeat(E, 1)
          if m is None else _dev(m, np.float64).reshape(E, 4).clone())
    xe = torch.empty((E, 9), dtype=torch.float64, device=dev)
    area = torch.empty(E, dtype=torch.float64, device=dev)
    xm, stride = _xmat(xmat, E)
    err = _lib.err_word()
    rc = lib.fe3d_tria3r_frame(E, _lib.ptr(cdof), _lib.ptr(x), x.numel(), _lib.ptr(xm), stride,
                               _lib.ptr(R), _lib.ptr(mm), _lib.ptr(xe), _lib.ptr(area),
                               _lib.ptr(err), _lib.stream_ptr())
    _lib.check(rc, 'tria3r_frames', err if check else None)
    return R, mm, xe, area


def _reduced_kc0(fn, nn, size, KC0r, KC0c, KC0v, x, cdof, init_k, props, pid, xmat, k6rot, aux, aux_w,
                 update_KC0v_only, check, what):
    lib = _lib.load()
    x = _dev(x, np.float64)
    cdof = _dev(cdof, np.int64).reshape(-1, nn).contiguous()
    init_k = _dev(init_k, np.int64).reshape(-1).contiguous()
    E = cdof.shape[0]
    if init_k.numel() != E:
        raise ValueError('init_k must have one entry per element')
    P = _props(props, SHELL_PROP_STRIDE)
    pid = _pid(pid, P, E)
    k6, k6s = _per_elem(k6rot, E, 1, 'k6rot')
    ax, axs = _per_elem(aux, E, aux_w, 'alpha' if aux_w == 1 else 'hg')
    out = _Out(KC0r, KC0c, KC0v, update_KC0v_only == 0)
    xm, stride = _xmat(xmat, E)
    err = _lib.err_word()
    rc = fn(E, _lib.ptr(cdof), _lib.ptr(init_k), _lib.ptr(x), x.numel(), _lib.ptr(xm), stride,
            None, None, None, None, _lib.ptr(P), P.shape[0], _lib.ptr(pid), _lib.ptr(k6), k6s,
            _lib.ptr(ax), axs, _lib.ptr(out.r), _lib.ptr(out.c), _lib.ptr(out.v), out.n,
            int(update_KC0v_only != 0), _lib.ptr(err), _lib.stream_ptr())
    _lib.check(rc, what, err if check else None)
    out.finish()


def tria3r_update_KC0(KC0r, KC0c, KC0v, x, cdof, init_k, props, pid=None, xmat=None, k6rot=100.,
                      alpha=0.7, update_KC0v_only=0, check=True):
    """Tria3R.update_KC0 over all elements (324 slots each), frame computed
    on the fly (tria3r.pyx:294-547, 950-2960)."""
    _reduced_kc0(_lib.load().fe3d_tria3r_kc0, 3, 324, KC0r, KC0c, KC0v, x, cdof, init_k, props, pid, xmat,
                 k6rot, alpha, 1, update_KC0v_only, check, 'tria3r_update_KC0')


def quad4r_update_KC0(KC0r, KC0c, KC0v, x, cdof, init_k, props, pid=None, xmat=None, k6rot=100.,
                      hg=(1., 1., 1., 1., 1.), update_KC0v_only=0, check=True):
    """Quad4R.update_KC0 over all elements (576 slots each), frame computed
    on the fly (quad4r.pyx:286-548, 1145-4618)."""
    _reduced_kc0(_lib.load().fe3d_quad4r_kc0, 4, 576, KC0r, KC0c, KC0v, x, cdof, init_k, props, pid, xmat,
                 k6rot, hg, 5, update_KC0v_only, check, 'quad4r_update_KC0')


def _reduced_fint(nn, fint, x, u, cdof, props, pid, xmat, k6rot, aux, aux_w, check, what):
    lib = _lib.load()
    torch = _lib.torch_mod()
    x = _dev(x, np.float64)
    u = _dev(u, np.float64)
    cdof = _dev(cdof, np.int64).reshape(-1, nn).contiguous()
    E = cdof.shape[0]
    frames = tria3r_frames if nn == 3 else quad4_frames
    R, m, xe, area = frames(x, cdof, xmat=xmat, check=check)
    ue = torch.empty((E, 6 * nn), dtype=torch.float64, device=u.device)
    err = _lib.err_word()
    probe = lib.fe3d_tria3r_probe_ue if nn == 3 else lib.fe3d_quad4_probe_ue
    rc = probe(E, _lib.ptr(cdof), _lib.ptr(u), u.numel(), _lib.ptr(R), _lib.ptr(ue), _lib.ptr(err),
               _lib.stream_ptr())
    _lib.check(rc, what + ' (probe_ue)')
    P = _props(props, SHELL_PROP_STRIDE)
    pid = _pid(pid, P, E)
    k6, k6s = _per_elem(k6rot, E, 1, 'k6rot')
    ax, axs = _per_elem(aux, E, aux_w, 'alpha' if aux_w == 1 else 'hg')
    f = fint if _lib.is_cuda_tensor(fint) else _dev(fint, np.float64)
    finte = torch.empty((E, 6 * nn), dtype=torch.float64, device=u.device)
    fn = lib.fe3d_tria3r_finte if nn == 3 else lib.fe3d_quad4r_finte
    rc = fn(E, _lib.ptr(cdof), _lib.ptr(R), _lib.ptr(m), _lib.ptr(xe), _lib.ptr(area), _lib.ptr(ue),
            _lib.ptr(P), P.shape[0], _lib.ptr(pid), _lib.ptr(k6), k6s, _lib.ptr(ax), axs, _lib.ptr(f),
            f.numel(), _lib.ptr(finte), _lib.ptr(err), _lib.stream_ptr())
    _lib.check(rc, what, err if check else None)
    if not _lib.is_cuda_tensor(fint):
        fint[:] = f.cpu().numpy()
    return finte


def tria3r_update_fint(fint, x, u, cdof, props, pid=None, xmat=None, k6rot=100., alpha=0.7, check=True):
    """Tria3R.update_probe_ue + update_fint over all elements; returns the
    local internal forces finte (E, 18) as well (tria3r.pyx:549-947, 2975-3017)."""
    return _reduced_fint(3, fint, x, u, cdof, props, pid, xmat, k6rot, alpha, 1, check, 'tria3r_update_fint')


def quad4r_update_fint(fint, x, u, cdof, props, pid=None, xmat=None, k6rot=100., hg=(1., 1., 1., 1., 1.),
                       check=True):
    """Quad4R.update_probe_ue + update_fint over all elements; returns finte
    (E, 24) as well (quad4r.pyx:549-1143, 4620-4679)."""
    return _reduced_fint(4, fint, x, u, cdof, props, pid, xmat, k6rot, hg, 5, check, 'quad4r_update_fint')


def tria3r_update_KG(KGr, KGc, KGv, x, u, cdof, init_k, props, pid=None, xmat=None, update_KGv_only=0,
                     check=True):
    """Tria3R.update_probe_ue + update_KG over all elements from the global u
    (81 slots each, tria3r.pyx:3020-3574)."""
    lib = _lib.load()
    x = _dev(x, np.float64)
    u = _dev(u, np.float64)
    cdof = _dev(cdof, np.int64).reshape(-1, 3).contiguous()
    init_k = _dev(init_k, np.int64).reshape(-1).contiguous()
    E = cdof.shape[0]
    P = _props(props, SHELL_PROP_STRIDE)
    pid = _pid(pid, P, E)
    out = _Out(KGr, KGc, KGv, update_KGv_only == 0)
    xm, stride = _xmat(xmat, E)
    err = _lib.err_word()
    rc = lib.fe3d_tria3r_kg(E, _lib.ptr(cdof), _lib.ptr(init_k), _lib.ptr(x), x.numel(), _lib.ptr(xm), stride,
                            _lib.ptr(u), u.numel(), None, None, None, None, None, _lib.ptr(P), P.shape[0],
                            _lib.ptr(pid), _lib.ptr(out.r), _lib.ptr(out.c), _lib.ptr(out.v), out.n,
                            int(update_KGv_only != 0), _lib.ptr(err), _lib.stream_ptr())
    _lib.check(rc, 'tria3r_update_KG', err if check else None)
    out.finish()


def tria3r_update_KG_given_stress(KGr, KGc, KGv, x, cdof, init_k, nstress, update_KGv_only=0, check=True):
    """Tria3R.update_KG_given_stress over all elements: ``nstress`` holds
    (Nxx, Nyy, Nxy) per element, shape (E, 3), or one triplet for all."""
    lib = _lib.load()
    x = _dev(x, np.float64)
    cdof = _dev(cdof, np.int64).reshape(-1, 3).contiguous()
    init_k = _dev(init_k, np.int64).reshape(-1).contiguous()
    E = cdof.shape[0]
    ns = _dev(nstress, np.float64).reshape(-1).contiguous()
    if ns.numel() not in (3, 3 * E):
        raise ValueError('nstress must have 3 or 3*E entries')
    out = _Out(KGr, KGc, KGv, update_KGv_only == 0)
    err = _lib.err_word()
    rc = lib.fe3d_tria3r_kg_given_stress(E, _lib.ptr(cdof), _lib.ptr(init_k), _lib.ptr(x), x.numel(), None,
                                         None, None, _lib.ptr(ns), 3 if ns.numel() == 3 * E and E > 1 else 0,
                                         _lib.ptr(out.r), _lib.ptr(out.c), _lib.ptr(out.v), out.n,
                                         int(update_KGv_only != 0), _lib.ptr(err), _lib.stream_ptr())
    _lib.check(rc, 'tria3r_update_KG_given_stress', err if check else None)
    out.finish()


def tria3r_update_M(Mr, Mc, Mv, x, cdof, init_k, props, pid=None, mtype=0, check=True):
    """Tria3R.update_M over all elements (mtype 0/1: 270 slots, 2: 162)."""
    if mtype not in (0, 1, 2):
        raise ValueError('mtype must be 0, 1 or 2')
    lib = _lib.load()
    x = _dev(x, np.float64)
    cdof = _dev(cdof, np.int64).reshape(-1, 3).contiguous()
    init_k = _dev(init_k, np.int64).reshape(-1).contiguous()
    E = cdof.shape[0]
    P = _props(props, SHELL_PROP_STRIDE)
    pid = _pid(pid, P, E)
    out = _Out(Mr, Mc, Mv, True)
    err = _lib.err_word()
    rc = lib.fe3d_tria3r_m(E, _lib.ptr(cdof), _lib.ptr(init_k), _lib.ptr(x), x.numel(), None, None,
                           _lib.ptr(P), P.shape[0], _lib.ptr(pid), _lib.ptr(out.r), _lib.ptr(out.c),
                           _lib.ptr(out.v), out.n, int(mtype), _lib.ptr(err), _lib.stream_ptr())
    _lib.check(rc, 'tria3r_update_M', err if check else None)
    out.finish()


quad4r_frames = quad4_frames
quad4r_update_KG = quad4_update_KG
quad4r_update_KG_given_stress = quad4_update_KG_given_stress
quad4r_update_M = quad4_update_M
