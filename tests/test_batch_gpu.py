"""Batched solve of many independent uneven plates (one block-diagonal system).

Each plate's displacements are checked against scipy's direct solve of that
plate alone, built from oracle triplets (the loop of
tests/test_quad4_static_point_load.py:80-102 run once per plate), within the
solver tolerances: FP64 relative residual 1e-8 and relative displacement
error 1e-7.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RESID_TOL = 1e-8
DISP_TOL = 1e-7


def _batch_system(bp):
    import torch
    from pyfe3d_gb300 import batch
    from pyfe3d_gb300.solver import CSRPattern
    nk = 576 * bp.E
    dev = torch.device('cuda')
    Kr = torch.zeros(nk, dtype=torch.int64, device=dev)
    Kc = torch.zeros(nk, dtype=torch.int64, device=dev)
    Kv = torch.zeros(nk, dtype=torch.float64, device=dev)
    batch.quad4_update_KC0(Kr, Kc, Kv, bp.x, bp.cdof, bp.init_k(576), bp.props, pid=bp.pid)
    pat = CSRPattern(Kr, Kc, bp.N, bp.bk)
    return pat, pat.assemble(Kv)


def _plate_direct(oracle, bp, i):
    """scipy direct solve of plate i alone from oracle triplets."""
    from scipy.sparse import coo_matrix
    from scipy.sparse.linalg import spsolve
    e = slice(int(bp.elem0[i]), int(bp.elem0[i + 1]))
    d = bp.plate_dofs(i)
    cdof = bp.cdof[e] - bp.dof0[i]
    n0, n1 = int(bp.node0[i]), int(bp.node0[i + 1])
    x = bp.x[3 * n0:3 * n1]
    E = cdof.shape[0]
    r, c, v = oracle.q4_kc0_batch(cdof, 576 * np.arange(E, dtype=np.int64), x, bp.props[i:i + 1])
    N = d.stop - d.start
    K = coo_matrix((v, (r, c)), shape=(N, N)).tocsc()
    bu = ~bp.bk[d]
    u = np.zeros(N)
    u[bu] = spsolve(K[bu][:, bu], bp.f[d][bu])
    return u


@pytest.fixture(scope='module')
def small_batch():
    from pyfe3d_gb300.meshes import BatchedPlates
    return BatchedPlates(nplates=12, nmin=4, nmax=16, seed=11)


@pytest.mark.parametrize('precision', [0, 1])
def test_batched_plates_match_direct_solves(gpulib, oracle, small_batch, precision):
    from pyfe3d_gb300.solver import BatchSolver
    bp = small_batch
    pat, vals = _batch_system(bp)
    bs = BatchSolver(pat, bp.inst_of_dof, bp.P).setup(vals, mixed=(precision == 1))
    lanes = bs.lanes()
    assert lanes[0] in (4, 8, 16, 32)
    if precision == 1:
        assert lanes[1] in (4, 8, 16, 32)
    fr = pat.reduce(bp.f)
    tol = 1e-10 if precision == 0 else RESID_TOL
    ur, st = bs.solve(fr, tol=tol, precision=precision, check_every=20, replace_every=100)
    assert st['status'] == 'converged', st
    assert (st['inst_status'] == 0).all()
    assert (st['inst_relres'] <= tol).all()
    u = pat.expand(ur).cpu().numpy()
    for i in range(bp.P):
        ref = _plate_direct(oracle, bp, i)
        got = u[bp.plate_dofs(i)]
        err = np.linalg.norm(got - ref) / np.linalg.norm(ref)
        assert err <= DISP_TOL, (i, err)


def test_batched_matches_one_at_a_time_iterations(gpulib, small_batch):
    """Each instance follows its own recurrence: its iteration count matches
    the single-system solver on that plate up to the check granularity."""
    import torch
    from pyfe3d_gb300 import batch
    from pyfe3d_gb300.solver import BatchSolver, CSRPattern, Solver
    bp = small_batch
    pat, vals = _batch_system(bp)
    bs = BatchSolver(pat, bp.inst_of_dof, bp.P).setup(vals)
    ur, st = bs.solve(pat.reduce(bp.f), tol=1e-8, check_every=2)
    dev = torch.device('cuda')
    for i in (0, bp.P // 2, bp.P - 1):
        e = slice(int(bp.elem0[i]), int(bp.elem0[i + 1]))
        cdof = bp.cdof[e] - bp.dof0[i]
        n0, n1 = int(bp.node0[i]), int(bp.node0[i + 1])
        E = cdof.shape[0]
        d = bp.plate_dofs(i)
        N = d.stop - d.start
        Kr = torch.zeros(576 * E, dtype=torch.int64, device=dev)
        Kc = torch.zeros_like(Kr)
        Kv = torch.zeros(576 * E, dtype=torch.float64, device=dev)
        batch.quad4_update_KC0(Kr, Kc, Kv, bp.x[3 * n0:3 * n1], cdof, 576 * np.arange(E, dtype=np.int64),
                               bp.props[i:i + 1])
        p1 = CSRPattern(Kr, Kc, N, bp.bk[d])
        u1, st1 = Solver(p1).setup(p1.assemble(Kv)).solve(p1.reduce(bp.f[d]), tol=1e-8, check_every=2)
        assert st1['status'] == 'converged'
        # same recurrence up to rounding (atomic summation order) and the
        # single-system solver's residual replacements (reliable updates),
        # which shift the stopping point by a few percent
        slack = max(8, st1['iterations'] // 20)
        assert abs(int(st['inst_iters'][i]) - st1['iterations']) <= slack, (i, st['inst_iters'][i], st1)
        ub = pat.expand(ur).cpu().numpy()[d]
        us = p1.expand(u1).cpu().numpy()
        assert np.linalg.norm(ub - us) <= 1e-6 * np.linalg.norm(us)


def test_zero_load_instance_and_initial_guess(gpulib, small_batch):
    from pyfe3d_gb300.solver import BatchSolver
    bp = small_batch
    pat, vals = _batch_system(bp)
    f = bp.f.copy()
    f[bp.plate_dofs(3)] = 0.
    bs = BatchSolver(pat, bp.inst_of_dof, bp.P).setup(vals)
    fr = pat.reduce(f)
    u0 = pat.reduce(np.ones(bp.N))
    ur, st = bs.solve(fr, u0=u0, tol=1e-9)
    assert st['status'] == 'converged', st
    u = pat.expand(ur).cpu().numpy()
    assert np.all(u[bp.plate_dofs(3)] == 0.)
    assert st['inst_iters'][3] == 0 and st['inst_relres'][3] == 0.
    # a second solve from the converged answer stops at once
    ur2, st2 = bs.solve(fr, u0=ur, tol=1e-9)
    assert st2['iterations'] == 0 and (st2['inst_iters'] == 0).all()


def test_bad_instance_maps_raise(gpulib, small_batch):
    from pyfe3d_gb300 import _lib
    from pyfe3d_gb300.solver import BatchSolver
    bp = small_batch
    pat, vals = _batch_system(bp)
    inst = bp.inst_of_dof.copy()
    inst[bp.plate_dofs(0)] = bp.P  # out of range
    with pytest.raises(_lib.Fe3dError, match='out of range|outside'):
        BatchSolver(pat, inst, bp.P)
    # the first plate's centre node moved to another instance: the matrix
    # then couples two instances
    inst = bp.inst_of_dof.copy()
    d = bp.plate_dofs(0)
    nxn, nyn = int(bp.nx[0]) + 1, int(bp.ny[0]) + 1  # nodes
    c = (nxn // 2) * nyn + nyn // 2
    inst[d.start + 6 * c:d.start + 6 * c + 6] = 1
    with pytest.raises(_lib.Fe3dError, match='argument'):
        BatchSolver(pat, inst, bp.P)
    # one node's DOFs split between two instances
    inst = bp.inst_of_dof.copy()
    free = np.where(~bp.bk[d])[0]
    inst[d.start + free[0]] = 1
    with pytest.raises(_lib.Fe3dError):
        BatchSolver(pat, inst, bp.P)


@pytest.mark.parametrize('split', ['all', 'mixed'])
def test_work_split_block_resident_solver(gpulib, oracle, small_batch, split):
    """Work split: instances up to a row limit are solved each by one thread
    block of the block-resident kernel, the others by the lockstep recurrence
    on the other stream ('mixed': the limit is the median plate size, so both
    paths run in the same solve).  Every plate still matches its direct solve,
    and repeating the solve gives bit-identical plates on the block-resident
    path (fixed-order block reductions)."""
    from pyfe3d_gb300.solver import BatchSolver
    bp = small_batch
    pat, vals = _batch_system(bp)
    bs = BatchSolver(pat, bp.inst_of_dof, bp.P).setup(vals)
    rows = np.bincount(bs.inst_of_row.cpu().numpy(), minlength=bp.P)
    limit = int(rows.max()) if split == 'all' else int(np.median(rows))
    n_split = bs.set_split(limit)
    assert n_split == int((rows <= limit).sum())
    assert (split == 'all') == (n_split == bp.P)
    fr = pat.reduce(bp.f)
    ur, st = bs.solve(fr, tol=1e-10, check_every=20)
    assert st['status'] == 'converged', st
    assert (st['inst_status'] == 0).all()
    assert (st['inst_relres'] <= 1e-10).all()
    assert (st['inst_iters'] > 0).all()
    u = pat.expand(ur).cpu().numpy()
    for i in range(bp.P):
        ref = _plate_direct(oracle, bp, i)
        got = u[bp.plate_dofs(i)]
        err = np.linalg.norm(got - ref) / np.linalg.norm(ref)
        assert err <= DISP_TOL, (i, err)
    ur2, st2 = bs.solve(fr, tol=1e-10, check_every=20)
    u2 = pat.expand(ur2).cpu().numpy()
    for i in np.nonzero(rows <= limit)[0]:
        assert np.array_equal(u2[bp.plate_dofs(i)], u[bp.plate_dofs(i)]), i
        assert st2['inst_iters'][i] == st['inst_iters'][i]
    # the lockstep-only solve of the same system agrees within the tolerance
    bs.set_split(0)
    ur3, st3 = bs.solve(fr, tol=1e-10, check_every=20)
    assert (st3['inst_status'] == 0).all()
    u3 = pat.expand(ur3).cpu().numpy()
    assert np.linalg.norm(u3 - u) <= 1e-8 * np.linalg.norm(u3)
