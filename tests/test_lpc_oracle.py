"""Pins the CPU oracle of the learned preconditioner: its weight gradient
against central finite differences of its own loss (float64, CPU)."""
import numpy as np
import pytest


def small_system(oracle, nel=4, seed=3):
    from scipy.sparse import coo_matrix
    from pyfe3d_gb300.meshes import RandomFieldPlate
    p = RandomFieldPlate(nel, seed=seed)
    r, c, v = oracle.q4_kc0_batch(p.cdof, p.init_k(576), p.x, p.props, pid=p.pid)
    K = coo_matrix((v, (r, c)), shape=(p.N, p.N)).tocsr()
    bu = ~p.bk
    Kuu = K[bu][:, bu].tocsr()
    Kuu.sort_indices()
    dof_of_row = np.nonzero(bu)[0]
    return p, Kuu, dof_of_row


@pytest.mark.parametrize('mode', [0, 1])
def test_oracle_gradient_matches_finite_differences(oracle, mode):
    from oracle import lpc_oracle as lo
    from scipy.sparse.linalg import spsolve
    p, K, dof = small_system(oracle)
    nnodes = p.nnodes
    rng = np.random.default_rng(0)
    samples, weights = [], []
    for _ in range(3):
        r = rng.standard_normal(K.shape[0])
        e = spsolve(K.tocsc(), r)
        samples.append(r)
        weights.append(1. / (e @ r))
    W = lo.init_weights(seed=1, out_std=0.5)
    scale = 0.1
    L, grad, _ = lo.loss_and_grad(K, dof, nnodes, W, samples, weights, scale, mode)
    # the relative squared energy error lies in (0, 1): mode 0 reports it minus one
    if mode == 0:
        assert -len(samples) < L < 0
    else:
        assert 0 < L < len(samples)
    idx = np.concatenate([rng.choice(np.arange(lo.OW1, lo.OB1), 4), rng.choice(np.arange(lo.OW2, lo.OB2), 4),
                          rng.choice(np.arange(lo.OW3, lo.NW), 6), [lo.OB1 + 3, lo.OB2 + 5, lo.OB3 + 7]])
    h = 1e-5
    for i in idx:
        Wp, Wm = W.copy(), W.copy()
        Wp[i] += h
        Wm[i] -= h
        Lp = lo.loss_and_grad(K, dof, nnodes, Wp, samples, weights, scale, mode)[0]
        Lm = lo.loss_and_grad(K, dof, nnodes, Wm, samples, weights, scale, mode)[0]
        fd = (Lp - Lm) / (2 * h)
        assert abs(fd - grad[i]) <= 1e-6 + 1e-4 * abs(fd), (i, fd, grad[i])
