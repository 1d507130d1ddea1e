"""Allocation-free solve entry point (collected last on purpose).

Some callers cannot allocate device memory themselves: a host application
whose GPU memory belongs to another runtime's pool, or a code path where a
cudaMalloc would synchronise the device or is forbidden.  For them the
library exports ``fe3d_jacobi_pcg_noalloc``, which solves K u = f with only
the caller's CSR arrays and vectors plus a fixed-size array that the library
holds in device memory.  These tests call it through the C ABI and compare
its displacements with those of the regular solver entry point
(``fe3d_solver_solve``), within the displacement tolerance used by the other
solver tests (1e-7 relative), on two calls in a row: the shared array keeps
the previous call's contents, so the second call checks that nothing stale
leaks into a new solve.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

DISP_TOL = 1e-7


def _plate_system():
    import torch
    from pyfe3d_gb300 import batch
    from pyfe3d_gb300.meshes import config2
    from pyfe3d_gb300.solver import CSRPattern
    m, props, pid, bk, f = config2(25)
    nk = 576 * m.E
    dev = torch.device('cuda')
    Kr = torch.zeros(nk, dtype=torch.int64, device=dev)
    Kc = torch.zeros(nk, dtype=torch.int64, device=dev)
    Kv = torch.zeros(nk, dtype=torch.float64, device=dev)
    batch.quad4_update_KC0(Kr, Kc, Kv, m.x, m.cdof, m.init_k(576), props, pid=pid)
    pat = CSRPattern(Kr, Kc, m.N, bk)
    vals = pat.assemble(Kv)
    return pat, vals, pat.reduce(f)


def _noalloc_solve(lib, pat, vals, fr, tol):
    import torch
    from pyfe3d_gb300 import _lib
    from pyfe3d_gb300.solver import SolveOpts, SolveStats
    u = torch.zeros_like(fr)
    o = SolveOpts(tol=tol, maxiter=200000, precision=0, check_every=50, replace_every=0, flexible=0)
    st = SolveStats()
    rc = lib.fe3d_jacobi_pcg_noalloc(pat.nrows, _lib.ptr(pat.rowptr), _lib.ptr(pat.colind),
                                     _lib.ptr(vals), _lib.ptr(fr), _lib.ptr(u), ctypes.byref(o),
                                     ctypes.byref(st), _lib.stream_ptr())
    assert rc == 0, _lib.FE3D_ERRORS.get(rc, rc)
    return u, st.as_dict()


def test_noalloc_matches_regular_solver_twice(gpulib):
    from pyfe3d_gb300 import _lib
    from pyfe3d_gb300.solver import Solver
    lib = _lib.load()
    pat, vals, fr = _plate_system()
    assert pat.nrows <= lib.fe3d_noalloc_max_rows()
    ref, st_ref = Solver(pat).setup(vals).solve(fr, tol=1e-10)
    assert st_ref['status'] == 'converged'
    ref = ref.cpu().numpy()
    for call in range(2):
        u, st = _noalloc_solve(lib, pat, vals, fr, 1e-10)
        assert st['status'] == 'converged' and st['relres'] <= 1e-10, (call, st)
        err = np.linalg.norm(u.cpu().numpy() - ref) / np.linalg.norm(ref)
        assert err <= DISP_TOL, (call, err)


def test_noalloc_rejects_sizes_above_its_maximum(gpulib):
    from pyfe3d_gb300 import _lib
    from pyfe3d_gb300.solver import SolveOpts, SolveStats
    lib = _lib.load()
    n = lib.fe3d_noalloc_max_rows() + 1
    o = SolveOpts(tol=1e-8, maxiter=10, precision=0, check_every=10, replace_every=0, flexible=0)
    st = SolveStats()
    # rejected on the host before any pointer is touched
    rc = lib.fe3d_jacobi_pcg_noalloc(n, None, None, None, None, None, ctypes.byref(o),
                                     ctypes.byref(st), None)
    assert rc == -7
    assert 'allocation-free maximum' in _lib.FE3D_ERRORS[rc]


@pytest.mark.parametrize('kind', ['diagonal', 'spd6'])
def test_noalloc_exact_solve_before_first_check(gpulib, kind):
    """Systems CG solves exactly within the first check period: the residual
    reaches zero, later iterations see p = 0 and must take no step (no 0/0)."""
    import torch
    from pyfe3d_gb300 import _lib
    from pyfe3d_gb300.solver import SolveOpts, SolveStats
    lib = _lib.load()
    rng = np.random.default_rng(11)
    if kind == 'diagonal':
        n = 40
        K = np.diag(rng.uniform(1., 10., n))
    else:
        n = 6
        a = rng.standard_normal((n, n))
        K = a @ a.T + n * np.eye(n)
    rows, cols = np.nonzero(K)
    rowptr = np.zeros(n + 1, np.int64)
    np.add.at(rowptr, rows + 1, 1)
    rowptr = np.cumsum(rowptr)
    dev = torch.device('cuda')
    t_rowptr = torch.as_tensor(rowptr, device=dev)
    t_col = torch.as_tensor(cols.astype(np.int32), device=dev)
    t_val = torch.as_tensor(K[rows, cols], device=dev)
    f = rng.standard_normal(n)
    t_f = torch.as_tensor(f, device=dev)
    o = SolveOpts(tol=1e-12, maxiter=1000, precision=0, check_every=50, replace_every=0, flexible=0)
    for call in range(2):
        u = torch.zeros(n, dtype=torch.float64, device=dev)
        st = SolveStats()
        rc = lib.fe3d_jacobi_pcg_noalloc(n, _lib.ptr(t_rowptr), _lib.ptr(t_col), _lib.ptr(t_val),
                                         _lib.ptr(t_f), _lib.ptr(u), ctypes.byref(o), ctypes.byref(st),
                                         _lib.stream_ptr())
        assert rc == 0, _lib.FE3D_ERRORS.get(rc, rc)
        d = st.as_dict()
        un = u.cpu().numpy()
        assert np.isfinite(un).all(), (call, kind)
        assert d['status'] == 'converged', (call, kind, d)
        ref = np.linalg.solve(K, f)
        assert np.linalg.norm(un - ref) / np.linalg.norm(ref) <= DISP_TOL, (call, kind)
