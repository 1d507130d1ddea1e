"""Global assembly, boundary-condition elimination and the static solve.

Stands in for what the reference's users write around the element loop
(tests/test_quad4_static_point_load.py:80-102,
tests/test_beamc_static_point_load.py:83-109)::

    K = coo_matrix((KC0v, (KC0r, KC0c)), shape=(N, N)).tocsc()
    Kuu = K[bu, :][:, bu]
    u[bu] = spsolve(Kuu, fext[bu])

with a pattern built once on the GPU (:class:`CSRPattern`), a deterministic
numeric assembly per value update and a block-Jacobi PCG (:class:`Solver`).
"""
import ctypes

import numpy as np

from . import _lib
from ._lib import c_i64, c_int, c_vp


class SolveOpts(ctypes.Structure):
    _fields_ = [('tol', ctypes.c_double), ('maxiter', ctypes.c_int64), ('precision', ctypes.c_int),
                ('check_every', ctypes.c_int), ('replace_every', ctypes.c_int),
                ('flexible', ctypes.c_int), ('inner_tol', ctypes.c_double)]


class SolveStats(ctypes.Structure):
    _fields_ = [('status', ctypes.c_int), ('reserved', ctypes.c_int), ('iterations', ctypes.c_int64),
                ('replacements', ctypes.c_int64), ('relres', ctypes.c_double)]

    def as_dict(self):
        return {'status': {0: 'converged', 1: 'maxiter', 3: 'non-finite', 4: 'stagnated'}.get(self.status,
                                                                             str(self.status)),
                'iterations': int(self.iterations), 'replacements': int(self.replacements),
                'relres': float(self.relres)}


class CSRPattern:
    """Reduced CSR pattern of COO indices (built once, reused for every update).

    ``bk`` marks constrained DOFs (the reference tests' boolean mask); rows
    and columns of those DOFs are eliminated, duplicates summed.
    """

    def __init__(self, Kr, Kc, N, bk=None):
        lib = _lib.load()
        torch = _lib.torch_mod()
        r = _lib.to_device(Kr, np.int64)
        c = _lib.to_device(Kc, np.int64)
        if r.numel() != c.numel():
            raise ValueError('row and column arrays differ in length')
        self.N = int(N)
        fixed = None
        if bk is not None:
            bk = _lib.to_device(np.asarray(bk, dtype=np.uint8) if not _lib.is_cuda_tensor(bk) else bk.to(torch.uint8),
                                np.uint8)
            if bk.numel() != self.N:
                raise ValueError('bk must have N entries')
            fixed = bk
        h = c_vp()
        err = _lib.err_word()
        rc = lib.fe3d_pattern_build(_lib.ptr(r), _lib.ptr(c), r.numel(), self.N, _lib.ptr(fixed),
                                    ctypes.byref(h), _lib.ptr(err), _lib.stream_ptr())
        _lib.check(rc, 'fe3d_pattern_build', err)
        self._h = h
        nr, nz, ni = c_i64(), c_i64(), c_i64()
        lib.fe3d_pattern_info(h, ctypes.byref(nr), ctypes.byref(nz), ctypes.byref(ni))
        self.nrows, self.nnz, self.nnz_in = nr.value, nz.value, ni.value
        dev = r.device
        self.rowptr = torch.empty(self.nrows + 1, dtype=torch.int64, device=dev)
        self.colind = torch.empty(max(self.nnz, 1), dtype=torch.int32, device=dev)[:self.nnz]
        self.dof_of_row = torch.empty(max(self.nrows, 1), dtype=torch.int64, device=dev)[:self.nrows]
        rc = lib.fe3d_pattern_copy(h, _lib.ptr(self.rowptr), _lib.ptr(self.colind) if self.nnz else None,
                                   _lib.ptr(self.dof_of_row) if self.nrows else None, _lib.stream_ptr())
        _lib.check(rc, 'fe3d_pattern_copy')

    @property
    def handle(self):
        return self._h

    def __del__(self):
        h = getattr(self, '_h', None)
        if h is not None and _lib._lib is not None:
            try:
                _lib._lib.fe3d_pattern_free(h)
            except Exception:
                pass
            self._h = None

    def assemble(self, Kv, out=None):
        """Reduced CSR values of the COO values Kv (device tensor of length nnz)."""
        lib = _lib.load()
        torch = _lib.torch_mod()
        v = _lib.to_device(Kv, np.float64)
        if v.numel() != self.nnz_in:
            raise ValueError('value array length %d differs from the pattern (%d)' % (v.numel(), self.nnz_in))
        if out is None:
            out = torch.empty(max(self.nnz, 1), dtype=torch.float64, device=v.device)[:self.nnz]
        rc = lib.fe3d_assemble(self._h, _lib.ptr(v), _lib.ptr(out), _lib.stream_ptr())
        _lib.check(rc, 'fe3d_assemble')
        return out

    def spmv(self, vals, x, y=None):
        lib = _lib.load()
        torch = _lib.torch_mod()
        x = _lib.to_device(x, np.float64)
        if y is None:
            y = torch.empty(self.nrows, dtype=torch.float64, device=x.device)
        rc = lib.fe3d_spmv(self._h, _lib.ptr(vals), _lib.ptr(x), _lib.ptr(y), _lib.stream_ptr())
        _lib.check(rc, 'fe3d_spmv')
        return y

    def to_scipy(self, vals):
        """Host scipy CSR of the reduced matrix (for checks and interop)."""
        from scipy.sparse import csr_matrix
        return csr_matrix((vals.cpu().numpy(), self.colind.cpu().numpy(), self.rowptr.cpu().numpy()),
                          shape=(self.nrows, self.nrows))

    def reduce(self, f):
        """f[bu] of a full-length vector (device tensor)."""
        f = _lib.to_device(f, np.float64)
        return f[self.dof_of_row]

    def expand(self, ur):
        """Full-length vector with zeros at the constrained DOFs."""
        torch = _lib.torch_mod()
        u = torch.zeros(self.N, dtype=torch.float64, device=ur.device)
        u[self.dof_of_row] = ur
        return u


class ElemGroup(ctypes.Structure):
    """fe3d_elem_group: E elements of nn nodes, DOF offsets cdof [E, nn] on the device."""
    _fields_ = [('E', ctypes.c_int64), ('nn', ctypes.c_int), ('cdof', ctypes.c_void_p)]


def _groups(groups):
    """ctypes array of element groups from (cdof [E, nn]) arrays; returns it and
    the device tensors it points into (kept alive by the caller)."""
    torch = _lib.torch_mod()
    devs = []
    arr = (ElemGroup * len(groups))()
    for i, cd in enumerate(groups):
        t = _lib.to_device(cd, np.int64)
        if t.dim() != 2:
            raise ValueError('element DOF offsets must be [E, nodes per element]')
        t = t.contiguous()
        devs.append(t)
        arr[i].E = t.shape[0]
        arr[i].nn = t.shape[1]
        arr[i].cdof = t.data_ptr() if t.numel() else None
    del torch
    return arr, devs


class ElementPattern(CSRPattern):
    """The reduced CSR pattern of one or more element groups, built from their
    connectivity (no COO triplets): ``groups`` is a list of DOF-offset arrays
    [E, nodes per element] (the elements' c1..c4 or c1, c2), in the order
    their matrices will be added.  Equal to :class:`CSRPattern` of the groups'
    KC0 triplets.  Values come from :class:`FusedMap` (no ``assemble``)."""

    def __init__(self, groups, N, bk=None):
        lib = _lib.load()
        torch = _lib.torch_mod()
        self.N = int(N)
        arr, self._group_tensors = _groups(groups)
        dev = self._group_tensors[0].device
        fixed = None
        if bk is not None:
            bk = _lib.to_device(np.asarray(bk, dtype=np.uint8) if not _lib.is_cuda_tensor(bk) else bk.to(torch.uint8),
                                np.uint8)
            if bk.numel() != self.N:
                raise ValueError('bk must have N entries')
            fixed = bk
        h = c_vp()
        err = _lib.err_word()
        rc = lib.fe3d_pattern_build_elements(arr, len(groups), self.N, _lib.ptr(fixed), ctypes.byref(h),
                                             _lib.ptr(err), _lib.stream_ptr())
        _lib.check(rc, 'fe3d_pattern_build_elements', err)
        self._h = h
        nr, nz, ni = c_i64(), c_i64(), c_i64()
        lib.fe3d_pattern_info(h, ctypes.byref(nr), ctypes.byref(nz), ctypes.byref(ni))
        self.nrows, self.nnz, self.nnz_in = nr.value, nz.value, ni.value
        self.rowptr = torch.empty(self.nrows + 1, dtype=torch.int64, device=dev)
        self.colind = torch.empty(max(self.nnz, 1), dtype=torch.int32, device=dev)[:self.nnz]
        self.dof_of_row = torch.empty(max(self.nrows, 1), dtype=torch.int64, device=dev)[:self.nrows]
        rc = lib.fe3d_pattern_copy(h, _lib.ptr(self.rowptr), _lib.ptr(self.colind) if self.nnz else None,
                                   _lib.ptr(self.dof_of_row) if self.nrows else None, _lib.stream_ptr())
        _lib.check(rc, 'fe3d_pattern_copy')

    def assemble(self, Kv, out=None):
        raise TypeError('an element pattern has no COO slots: assemble its values with FusedMap')


class FusedMap:
    """Element -> CSR scatter map of the groups of an :class:`ElementPattern`
    (same groups, same order).  Elements are coloured so that no two
    elements of a colour share a node; each colour is one launch, so the
    values are summed without atomics in a fixed order.

    ``mode='assign'`` (default): the first contributor of each node-pair
    block stores, the others add; after every group has run in order the
    values are K whatever the array held.  ``mode='add'`` adds every block.
    ``mode='atomic'`` (fused Quad4 KC0 only) adds every block in one launch
    with atomic additions: no colour passes, but the summation order of
    entries with three or more contributions varies between runs.
    """

    MODES = {'add': 0, 'assign': 1, 'atomic': 2}

    def __init__(self, pattern, groups):
        lib = _lib.load()
        if not isinstance(pattern, ElementPattern):
            raise TypeError('a FusedMap needs an ElementPattern')
        self.pattern = pattern
        arr, devs = _groups(groups)
        self.nn = [int(t.shape[1]) for t in devs]
        self.E = [int(t.shape[0]) for t in devs]
        h = c_vp()
        err = _lib.err_word()
        rc = lib.fe3d_fmap_build(pattern.handle, arr, len(groups), ctypes.byref(h), _lib.ptr(err),
                                 _lib.stream_ptr())
        _lib.check(rc, 'fe3d_fmap_build', err)
        self._h = h

    @property
    def handle(self):
        return self._h

    def colors(self, g=0):
        """Element count of every colour of group g."""
        n = c_int()
        counts = np.zeros(64, dtype=np.int64)
        _lib.check(_lib.load().fe3d_fmap_info(self._h, int(g), ctypes.byref(n), counts.ctypes.data),
                   'fe3d_fmap_info')
        return counts[:n.value].copy()

    def __del__(self):
        h = getattr(self, '_h', None)
        if h is not None and _lib._lib is not None:
            try:
                _lib._lib.fe3d_fmap_free(h)
            except Exception:
                pass
            self._h = None

    def new_values(self, device=None):
        torch = _lib.torch_mod()
        return torch.zeros(max(self.pattern.nnz, 1), dtype=torch.float64,
                           device=device or self.pattern.rowptr.device)[:self.pattern.nnz]

    def scatter(self, vals, g, init_k, Kv, mode='assign'):
        """vals (+)= group g's element matrices held values-only in Kv at
        init_k (e.g. a values-only update_KC0 into a zeroed array)."""
        lib = _lib.load()
        ik = _lib.to_device(init_k, np.int64).reshape(-1).contiguous()
        kv = _lib.to_device(Kv, np.float64)
        if ik.numel() != self.E[g]:
            raise ValueError('init_k must have one offset per element of group %d' % g)
        err = _lib.err_word()
        rc = lib.fe3d_csr_scatter(self._h, int(g), _lib.ptr(ik), _lib.ptr(kv), kv.numel(), _lib.ptr(vals),
                                  self.MODES[mode], _lib.ptr(err), _lib.stream_ptr())
        _lib.check(rc, 'fe3d_csr_scatter', err)
        return vals


class Solver:
    """Block-Jacobi PCG bound to a pattern (6 DOFs per node by default)."""

    def __init__(self, pattern, block_size=6):
        lib = _lib.load()
        self.pattern = pattern
        h = c_vp()
        rc = lib.fe3d_solver_create(pattern.handle, int(block_size), ctypes.byref(h))
        _lib.check(rc, 'fe3d_solver_create')
        self._h = h
        self.vals = None
        self.nonpos_blocks = 0

    def __del__(self):
        h = getattr(self, '_h', None)
        if h is not None and _lib._lib is not None:
            try:
                _lib._lib.fe3d_solver_free(h)
            except Exception:
                pass
            self._h = None

    def setup(self, vals, mixed=False, split=False):
        """Factor the nodal blocks of the reduced matrix values (kept alive
        here); ``mixed`` prepares precision 1, ``split`` precision 2."""
        lib = _lib.load()
        self.vals = vals
        nonpos = c_int()
        rc = lib.fe3d_solver_setup(self._h, _lib.ptr(vals), int(bool(mixed)) | (2 if split else 0),
                                   ctypes.byref(nonpos), _lib.stream_ptr())
        _lib.check(rc, 'fe3d_solver_setup')
        self.nonpos_blocks = nonpos.value
        self.mixed_ready = bool(mixed)
        self.split_ready = bool(split)
        return self

    def solve(self, f, u0=None, tol=1e-8, maxiter=None, precision=0, check_every=50, replace_every=None,
              flexible=False, fallback=True, inner_tol=1e-2):
        """Solve K u = f on the reduced system; returns (u, stats dict).

        precision 0: FP64 block-Jacobi PCG; 1: FP32 SpMV and preconditioner
        with FP64 reliable updates every ``replace_every`` (100) iterations;
        2: split-FP32 SpMV; 3: nested iterative refinement, inner FP32 PCG
        to ``inner_tol`` (``replace_every`` caps one inner solve, default
        none) inside the FP64 residual loop.  Precision 1 or 3 that stagnates
        (FP32 directions can no longer reduce the FP64 residual) continues in
        FP64 from its iterate when ``fallback``; the stats then sum both
        phases and carry ``fp64_iterations``."""
        lib = _lib.load()
        torch = _lib.torch_mod()
        f = _lib.to_device(f, np.float64)
        n = self.pattern.nrows
        if f.numel() != n:
            raise ValueError('right-hand side has %d entries, the reduced system %d' % (f.numel(), n))
        u = torch.zeros(n, dtype=torch.float64, device=f.device) if u0 is None else \
            _lib.to_device(u0, np.float64).clone()
        if (precision in (1, 3) and not getattr(self, 'mixed_ready', False)) or \
                (precision == 2 and not getattr(self, 'split_ready', False)):
            self.setup(self.vals, mixed=precision in (1, 3) or getattr(self, 'mixed_ready', False),
                       split=precision == 2 or getattr(self, 'split_ready', False))
        if replace_every is None:
            replace_every = 0 if precision == 3 else 100
        o = SolveOpts(tol=float(tol), maxiter=int(maxiter if maxiter is not None else 20 * n + 1000),
                      precision=int(precision), check_every=int(check_every),
                      replace_every=int(replace_every), flexible=int(bool(flexible)), inner_tol=float(inner_tol))
        st = SolveStats()
        rc = lib.fe3d_solver_solve(self._h, _lib.ptr(f), _lib.ptr(u), ctypes.byref(o), ctypes.byref(st),
                                   _lib.stream_ptr())
        _lib.check(rc, 'fe3d_solver_solve')
        d = st.as_dict()
        if precision in (1, 3) and fallback and d['status'] == 'stagnated':
            left = max(o.maxiter - d['iterations'], 0)
            u, d2 = self.solve(f, u0=u, tol=tol, maxiter=left, precision=0, check_every=check_every,
                               flexible=flexible)
            d2['fp64_iterations'] = d2['iterations']
            d2['iterations'] += d['iterations']
            d2['replacements'] += d['replacements']
            d = d2
        return u, d


class BatchSolver:
    """Block-Jacobi PCG over many independent instances at once.

    ``pattern`` holds the block-diagonal matrix of all instances;
    ``inst_of_dof`` (length N, full DOF numbering) gives each DOF's instance
    in ``[0, ninst)``.  Each instance converges on its own test
    ``||f_i - K_i u_i|| <= tol ||f_i||``.
    """

    def __init__(self, pattern, inst_of_dof, ninst, block_size=6):
        lib = _lib.load()
        torch = _lib.torch_mod()
        self.pattern = pattern
        self.ninst = int(ninst)
        inst = _lib.to_device(inst_of_dof, np.int32)
        if inst.numel() != pattern.N:
            raise ValueError('inst_of_dof must have N entries')
        self.inst_of_row = inst[pattern.dof_of_row].to(torch.int32).contiguous()
        h = c_vp()
        rc = lib.fe3d_bsolver_create(pattern.handle, int(block_size), self.ninst, _lib.ptr(self.inst_of_row),
                                     ctypes.byref(h))
        _lib.check(rc, 'fe3d_bsolver_create')
        self._h = h
        self.vals = None
        self.mixed_ready = False

    def __del__(self):
        h = getattr(self, '_h', None)
        if h is not None and _lib._lib is not None:
            try:
                _lib._lib.fe3d_bsolver_free(h)
            except Exception:
                pass
            self._h = None

    def setup(self, vals, mixed=False):
        lib = _lib.load()
        self.vals = vals
        nonpos = c_int()
        rc = lib.fe3d_bsolver_setup(self._h, _lib.ptr(vals), int(bool(mixed)), ctypes.byref(nonpos),
                                    _lib.stream_ptr())
        _lib.check(rc, 'fe3d_bsolver_setup')
        self.nonpos_blocks = nonpos.value
        self.mixed_ready = bool(mixed)
        return self

    def lanes(self):
        """SpMV lanes per row chosen at setup: (FP64, FP32)."""
        a, b = c_int(), c_int()
        _lib.check(_lib.load().fe3d_bsolver_info(self._h, ctypes.byref(a), ctypes.byref(b)), 'fe3d_bsolver_info')
        return a.value, b.value

    def set_split(self, max_rows):
        """Work split of FP64 solves: instances of at most ``max_rows``
        contiguous reduced rows are solved each by one thread block of a
        block-resident PCG kernel, concurrently with the lockstep recurrence of
        the others (0: all lockstep).  Returns how many instances qualify."""
        e = ctypes.c_int64()
        _lib.check(_lib.load().fe3d_bsolver_set_split(self._h, int(max_rows), ctypes.byref(e)),
                   'fe3d_bsolver_set_split')
        self.split_rows = int(max_rows)
        return int(e.value)

    def solve(self, f, u0=None, tol=1e-8, maxiter=None, precision=0, check_every=50, replace_every=None,
              fallback=True, inner_tol=1e-2):
        """Solve every instance; returns (u, stats) with per-instance arrays
        ``inst_status``, ``inst_iters`` and ``inst_relres`` in stats.

        precision 0: FP64; 1: FP32 SpMV/preconditioner with FP64 reliable
        updates; 3: nested iterative refinement (inner FP32 PCG per instance
        to ``inner_tol``, outer FP64 residual and restart).
        Instances that stagnate in precision 1 or 3 continue in FP64 from their
        iterates when ``fallback`` (the others stop at once: their FP64
        residual already meets the tolerance); ``fp64_instances`` counts
        them and their iterations add up."""
        lib = _lib.load()
        torch = _lib.torch_mod()
        f = _lib.to_device(f, np.float64)
        n = self.pattern.nrows
        if f.numel() != n:
            raise ValueError('right-hand side has %d entries, the reduced system %d' % (f.numel(), n))
        u = torch.zeros(n, dtype=torch.float64, device=f.device) if u0 is None else \
            _lib.to_device(u0, np.float64).clone()
        if precision in (1, 3) and not self.mixed_ready:
            self.setup(self.vals, mixed=True)
        if replace_every is None:
            replace_every = 0 if precision == 3 else 100
        o = SolveOpts(tol=float(tol), maxiter=int(maxiter if maxiter is not None else 20 * n + 1000),
                      precision=int(precision), check_every=int(check_every),
                      replace_every=int(replace_every), flexible=0, inner_tol=float(inner_tol))
        st = SolveStats()
        K = self.ninst
        status = np.zeros(K, dtype=np.int32)
        iters = np.zeros(K, dtype=np.int64)
        relres = np.zeros(K, dtype=np.float64)
        rc = lib.fe3d_bsolver_solve(self._h, _lib.ptr(f), _lib.ptr(u), ctypes.byref(o),
                                    status.ctypes.data, iters.ctypes.data, relres.ctypes.data,
                                    ctypes.byref(st), _lib.stream_ptr())
        _lib.check(rc, 'fe3d_bsolver_solve')
        d = st.as_dict()
        d.update(inst_status=status, inst_iters=iters, inst_relres=relres)
        if precision in (1, 3) and fallback and (status == 4).any():
            u, d2 = self.solve(f, u0=u, tol=tol, maxiter=maxiter, precision=0, check_every=check_every)
            d2['inst_iters'] = d2['inst_iters'] + iters
            d2['iterations'] += d['iterations']
            d2['fp64_instances'] = int((status == 4).sum())
            d = d2
        return u, d


def static_solve_coo(Kr, Kc, Kv, N, bk, f, tol=1e-8, precision=0, maxiter=None, return_stats=False):
    """One-call equivalent of coo -> csc -> K[bu][:, bu] -> spsolve -> u[bu].

    Returns the full displacement vector as a numpy array (zeros at bk).
    """
    pat = CSRPattern(Kr, Kc, N, bk)
    vals = pat.assemble(Kv)
    s = Solver(pat).setup(vals, mixed=(precision == 1), split=(precision == 2))
    fr = pat.reduce(f)
    ur, stats = s.solve(fr, tol=tol, precision=precision, maxiter=maxiter)
    u = pat.expand(ur).cpu().numpy()
    return (u, stats) if return_stats else u
