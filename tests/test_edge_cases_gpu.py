"""Edge cases of the C ABI on the GPU: empty inputs, all-constrained
systems, argument checks and single-instance batches."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_empty_element_sets_are_no_ops(gpulib):
    from pyfe3d_gb300 import _lib
    lib = _lib.load()
    sp = _lib.stream_ptr()
    assert lib.fe3d_quad4_kc0(0, None, None, None, 0, None, 0, None, None, None, None, None, 0, None, None, None,
                              None, 0, 0, None, sp) == 0
    assert lib.fe3d_quad4_kg(0, None, None, None, 0, None, 0, None, 0, None, None, None, None, None, 0, None, None,
                             None, None, 0, None, sp) == 0
    assert lib.fe3d_quad4_m(0, None, None, None, 0, None, None, None, None, 0, None, None, None, None, 0, 0, None,
                            sp) == 0
    assert lib.fe3d_quad4_kg_given_stress(0, None, None, None, 0, None, 0, None, None, None, 0, None, None, None, 0,
                                          None, sp) == 0
    assert lib.fe3d_beamc_kc0(0, None, None, None, None, None, 0, None, None, None, None, 0, 0, None, sp) == 0
    assert lib.fe3d_beamc_fint(0, None, None, None, None, None, 0, None, None, 0, None, None, sp) == 0
    assert lib.fe3d_quad4_kc0_host(0, None, None, None, 0, None, 1, None, None, None, None, 0, 0, 0, None, sp) == 0
    assert lib.fe3d_isotropic_plate_records(0, None, 0, None, 0, None, 0, None, 0, None, 0, 1, None, sp) == 0


def test_argument_errors_are_reported_before_launch(gpulib):
    from pyfe3d_gb300 import _lib
    lib = _lib.load()
    sp = _lib.stream_ptr()
    # negative sizes, missing arrays, bad modes
    assert lib.fe3d_quad4_kc0(-1, None, None, None, 0, None, 0, None, None, None, None, None, 0, None, None, None,
                              None, 0, 0, None, sp) == -1
    assert lib.fe3d_quad4_kc0(5, None, None, None, 0, None, 0, None, None, None, None, None, 0, None, None, None,
                              None, 0, 0, None, sp) == -1
    assert lib.fe3d_quad4_m(1, None, None, None, 0, None, None, None, None, 0, None, None, None, None, 0, 7, None,
                            sp) == -1
    assert lib.fe3d_spmm(None, None, None, None, 4, sp) == -1
    assert lib.fe3d_isotropic_plate_records(4, None, 1, None, 1, None, 1, None, 0, None, 0, 1, None, sp) == -1


def test_all_constrained_system_and_trivial_solve(gpulib):
    from pyfe3d_gb300 import batch
    from pyfe3d_gb300.meshes import config1
    from pyfe3d_gb300.solver import CSRPattern, Solver
    m, props, pid, bk, f = config1()
    n = 576 * m.E
    r = np.zeros(n, np.int64); c = np.zeros(n, np.int64); v = np.zeros(n)
    batch.quad4_update_KC0(r, c, v, m.x, m.cdof, m.init_k(576), props)
    pat = CSRPattern(r, c, m.N, np.ones(m.N, bool))
    assert pat.nrows == 0 and pat.nnz == 0
    s = Solver(pat).setup(pat.assemble(v))
    u, st = s.solve(np.zeros(0), tol=1e-8)
    assert st['status'] == 'converged' and u.numel() == 0


def test_single_instance_batch_equals_solver(gpulib):
    from pyfe3d_gb300 import batch
    from pyfe3d_gb300.meshes import config2
    from pyfe3d_gb300.solver import BatchSolver, CSRPattern, Solver
    m, props, pid, bk, f = config2(15)
    n = 576 * m.E
    r = np.zeros(n, np.int64); c = np.zeros(n, np.int64); v = np.zeros(n)
    batch.quad4_update_KC0(r, c, v, m.x, m.cdof, m.init_k(576), props, pid=pid)
    pat = CSRPattern(r, c, m.N, bk)
    vals = pat.assemble(v)
    fr = pat.reduce(f)
    u1, st1 = Solver(pat).setup(vals).solve(fr, tol=1e-9)
    u2, st2 = BatchSolver(pat, np.zeros(m.N, np.int32), 1).setup(vals).solve(fr, tol=1e-9)
    assert st1['status'] == st2['status'] == 'converged'
    a, b = u1.cpu().numpy(), u2.cpu().numpy()
    assert np.linalg.norm(a - b) <= 1e-7 * np.linalg.norm(a)


def test_spmm_matches_spmv_columns(gpulib):
    import torch
    from pyfe3d_gb300 import batch, eigen
    from pyfe3d_gb300.meshes import config2
    from pyfe3d_gb300.solver import CSRPattern
    m, props, pid, bk, f = config2(11)
    n = 576 * m.E
    r = np.zeros(n, np.int64); c = np.zeros(n, np.int64); v = np.zeros(n)
    batch.quad4_update_KC0(r, c, v, m.x, m.cdof, m.init_k(576), props, pid=pid)
    pat = CSRPattern(r, c, m.N, bk)
    vals = pat.assemble(v)
    A = pat.to_scipy(vals)
    rng = np.random.default_rng(2)
    for k in (1, 3, 8, 13, 16, 20):
        X = rng.standard_normal((pat.nrows, k))
        Y = eigen.CSROperator(pat, vals).matmul(torch.from_numpy(X).cuda()).cpu().numpy()
        ref = A @ X
        assert np.abs(Y - ref).max() <= 1e-13 * np.abs(ref).max(), k


def test_wide_rows_fall_back_to_32_bit_columns(gpulib):
    """A row whose columns span more than 65,535 (a beam tying the first node
    of a long chain to the last) cannot use the 16-bit column offsets; the
    SpMV and the solve take the 32-bit columns and still match scipy."""
    import torch
    from pyfe3d_gb300 import batch
    from pyfe3d_gb300.meshes import stringer_records
    from pyfe3d_gb300.solver import CSRPattern, Solver
    nn = 12000
    x = np.zeros((nn, 3))
    x[:, 0] = np.linspace(0., 10., nn)
    x[:, 1] = 0.02 * np.sin(np.arange(nn))
    conn = np.stack([np.arange(nn - 1), np.arange(1, nn)], 1)
    conn = np.vstack([conn, [[0, nn - 1]]])
    cdof = (6 * conn).astype(np.int64)
    E = len(conn)
    N = 6 * nn
    r = np.zeros(144 * E, np.int64); c = np.zeros(144 * E, np.int64); v = np.zeros(144 * E)
    batch.beamc_update_KC0(r, c, v, x.ravel(), cdof, 144 * np.arange(E), np.array([0., 0., 1.]),
                           stringer_records()[None, :])
    bk = np.zeros(N, bool)
    bk[:6] = True  # clamp node 0
    pat = CSRPattern(r, c, N, bk)
    vals = pat.assemble(v)
    A = pat.to_scipy(vals)
    xs = np.random.default_rng(3).standard_normal(pat.nrows)
    y = pat.spmv(vals, torch.from_numpy(xs).cuda()).cpu().numpy()
    assert np.abs(y - A @ xs).max() <= 1e-12 * np.abs(A @ xs).max()
    # the solver's SpMV launches through the same dispatch: iterations on
    # this (very ill-conditioned) chain run and report finite residuals
    f = np.zeros(N)
    f[6 * (nn // 2) + 2] = 1.
    _, st = Solver(pat).setup(vals).solve(pat.reduce(f), tol=1e-300, maxiter=40, check_every=10)
    assert np.isfinite(st['relres']) and st['iterations'] == 40
