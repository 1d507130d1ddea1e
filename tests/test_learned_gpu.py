"""Learned block preconditioner: CUDA features, MLP forward/backward, blocks,
loss and weight gradients against the CPU oracle (oracle/lpc_oracle.py,
itself pinned by finite differences), then training on FP64-solver pairs and
the flexible PCG with the trained blocks against plain block Jacobi."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _system(p):
    import torch
    from pyfe3d_gb300 import batch
    from pyfe3d_gb300.solver import CSRPattern
    dev = torch.device('cuda')
    nk = 576 * p.E
    Kr = torch.zeros(nk, dtype=torch.int64, device=dev)
    Kc = torch.zeros(nk, dtype=torch.int64, device=dev)
    Kv = torch.zeros(nk, dtype=torch.float64, device=dev)
    batch.quad4_update_KC0(Kr, Kc, Kv, p.x, p.cdof, p.init_k(576), p.props, pid=p.pid)
    pat = CSRPattern(Kr, Kc, p.N, p.bk)
    return pat, pat.assemble(Kv)


@pytest.mark.parametrize('mode', [0, 1])
def test_kernels_match_cpu_oracle(gpulib, mode):
    import torch
    from scipy.sparse.linalg import spsolve
    from oracle import lpc_oracle as lo
    from pyfe3d_gb300 import learned
    from pyfe3d_gb300.meshes import RandomFieldPlate
    from pyfe3d_gb300.solver import Solver
    p = RandomFieldPlate(6, seed=7)
    pat, vals = _system(p)
    K = pat.to_scipy(vals)
    dof = pat.dof_of_row.cpu().numpy()
    nn = p.nnodes
    W = lo.init_weights(seed=2, out_std=0.5).astype(np.float32)
    # the kernels take the output scale as an FP32 argument
    scale = float(np.float32(0.1))
    pc = learned.LearnedPC(weights=W, out_scale=scale, mode=mode)
    s = Solver(pat).setup(vals)
    ctx = learned._Ctx(s)
    # features
    feat_ref, sdiag_ref = lo.features(K, dof, nn)
    feat = ctx.feat.cpu().numpy().reshape(nn, -1)
    assert np.allclose(ctx.sdiag.cpu().numpy()[:pat.nrows], sdiag_ref, rtol=1e-14)
    assert np.abs(feat - feat_ref).max() <= 1e-5 * max(1., np.abs(feat_ref).max())
    # forward pass, blocks, fallback
    W64 = W.astype(np.float64)
    out_ref, h1, h2 = lo.forward(feat_ref, W64)
    pc._forward_blocks(ctx, train=True)
    out = ctx.out.cpu().numpy().reshape(nn, -1)
    assert np.abs(out - out_ref).max() <= 1e-4 * np.abs(out_ref).max()
    act = ctx.act.cpu().numpy().reshape(nn, -1)
    assert np.abs(act[:, :64] - h1).max() <= 1e-4 and np.abs(act[:, 64:] - h2).max() <= 1e-4
    Bs, lis, rows = lo.blocks(K, dof, nn, sdiag_ref, out.astype(np.float64), scale)
    blocks = ctx.blocks.cpu().numpy().reshape(nn, 6, 6)
    for j, rs in enumerate(rows):
        b = len(rs)
        if b:
            assert np.abs(blocks[j, :b, :b] - Bs[j]).max() <= 1e-12 * np.abs(Bs[j]).max()
    inv, fb = lo.block_inverses(K, dof, nn, Bs, rows)
    assert not fb.any() and not ctx.fallback.cpu().numpy().any()
    # loss and weight gradients for two residual samples
    rng = np.random.default_rng(0)
    samples, weights = [], []
    for _ in range(2):
        r = rng.standard_normal(pat.nrows)
        e = spsolve(K.tocsc(), r)
        samples.append(r)
        weights.append(1. / (e @ r))

    class _Sys:
        def context(self, feature_set=0):
            return self.ctx
    sysm = _Sys()
    sysm.pattern, sysm.vals, sysm.ctx = pat, vals, ctx
    sysm.samples = torch.tensor(np.stack(samples), device='cuda')
    sysm.weights = np.array(weights)
    loss = float(pc.loss_grad(sysm, [0, 1]).item())
    L_ref, grad_ref, gout_ref = lo.loss_and_grad(K, dof, nn, W64, samples, np.array(weights), scale, mode,
                                                 factor=0.5)
    assert abs(loss - L_ref) <= 1e-6 * abs(L_ref)
    gout = ctx.gout.cpu().numpy().reshape(nn, -1)
    assert np.abs(gout - gout_ref).max() <= 1e-4 * np.abs(gout_ref).max()
    grad = pc.grad.cpu().numpy()
    for a, b in ((0, lo.OB1), (lo.OB1, lo.OW2), (lo.OW2, lo.OB2), (lo.OB2, lo.OW3), (lo.OW3, lo.OB3),
                 (lo.OB3, lo.NW)):
        ref = grad_ref[a:b]
        assert np.abs(grad[a:b] - ref).max() <= 2e-3 * np.abs(ref).max() + 1e-12, (a, b)


def test_feature_set_29_matches_cpu_oracle(gpulib):
    """The 29-input feature set (normalised diagonal block and neighbour-block
    norms) against its CPU restatement."""
    from oracle import lpc_oracle as lo
    from pyfe3d_gb300 import learned
    from pyfe3d_gb300.meshes import RandomFieldPlate
    from pyfe3d_gb300.solver import Solver
    p = RandomFieldPlate(6, seed=8)
    pat, vals = _system(p)
    K = pat.to_scipy(vals)
    dof = pat.dof_of_row.cpu().numpy()
    s = Solver(pat).setup(vals)
    ctx = learned._Ctx(s, feature_set=1)
    ref, _ = lo.features29(K, dof, p.nnodes)
    feat = ctx.feat.cpu().numpy().reshape(p.nnodes, -1)
    assert np.abs(feat - ref).max() <= 1e-6 * max(1., np.abs(ref).max())
    assert (feat[:, 29:] == 0).all()
    # a free DOF has 1 on the normalised diagonal
    free = ref[:, [lo.ut_index(i, i) for i in range(6)]]
    assert np.allclose(free[free != 0], 1.)


@pytest.mark.parametrize('feature_set', [0, 1])
def test_training_gain_and_flexible_pcg(gpulib, feature_set):
    """Train on FP64-solver pairs of a few plates; on a held-out plate the
    learned blocks inside flexible CG reach the FP64 tolerance, the solution
    matches the direct solve, and the learned blocks take no more iterations
    than block Jacobi (flexible and plain PCG)."""
    from scipy.sparse.linalg import spsolve
    from pyfe3d_gb300 import learned
    from pyfe3d_gb300.meshes import RandomFieldPlate
    from pyfe3d_gb300.solver import Solver
    systems = []
    for k, nel in enumerate((12, 14, 16)):
        p = RandomFieldPlate(nel, seed=100 + k)
        pat, vals = _system(p)
        systems.append(learned.make_training_system(pat, vals, pat.reduce(p.f), npairs=16))
    pc = learned.LearnedPC(seed=0, out_scale=0.1, feature_set=feature_set)
    before = pc.evaluate(systems)
    pc.train(systems, steps=600, batch=8, lr=2e-3)
    after = pc.evaluate(systems)
    assert after < before, (before, after)
    # held-out plate
    p = RandomFieldPlate(16, seed=999)
    pat, vals = _system(p)
    fr = pat.reduce(p.f)
    s0 = Solver(pat).setup(vals)
    u0, st0 = s0.solve(fr, tol=1e-8, check_every=2)
    s1 = Solver(pat).setup(vals)
    pc.install(s1)
    u1, st1 = s1.solve(fr, tol=1e-8, check_every=2, flexible=True)
    assert st0['status'] == 'converged' and st1['status'] == 'converged', (st0, st1)
    assert st1['relres'] <= 1e-8
    ref = spsolve(pat.to_scipy(vals).tocsc(), fr.cpu().numpy())
    err = np.linalg.norm(u1.cpu().numpy() - ref) / np.linalg.norm(ref)
    assert err <= 1e-7, err
    # the installed blocks are symmetric positive definite (Cholesky per
    # node, else block Jacobi), so plain PCG with them converges as well
    s2 = Solver(pat).setup(vals)
    pc.install(s2)
    u2, st2 = s2.solve(fr, tol=1e-8, check_every=2)
    assert st2['status'] == 'converged' and st2['relres'] <= 1e-8, st2
    err2 = np.linalg.norm(u2.cpu().numpy() - ref) / np.linalg.norm(ref)
    assert err2 <= 1e-7, err2
    # the gain: no more iterations than block Jacobi on the held-out plate
    assert st1['iterations'] <= st0['iterations'], (st0['iterations'], st1['iterations'])
    assert st2['iterations'] <= st0['iterations'], (st0['iterations'], st2['iterations'])
    print('\nlearned PC (features %d): objective %.4f -> %.4f; held-out iterations block Jacobi %d, learned %d '
          '(flexible), %d (plain)' % (feature_set, before, after, st0['iterations'], st1['iterations'],
                                      st2['iterations']))
