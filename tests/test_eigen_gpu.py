"""Device LOBPCG against scipy (eigsh, the reference tests' solver,
tests/test_quad4_natural_freq.py:117-120, and a dense generalised eigh for the
buckling pencil of tests/test_quad4_linear_buckling_plate_rotated.py:129-131)
on the same reduced matrices assembled on the GPU."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _plate(nx=15, ny=11, a=1.0, b=0.7):
    from pyfe3d_gb300.meshes import PlateMesh
    from pyfe3d_gb300.shellprop import isotropic_plate_records
    m = PlateMesh(nx, ny, a, b)
    props = isotropic_plate_records(0.004, 70e9, 0.33, rho=2700.)
    bk = m.bc_mask((0, 1, 2))
    return m, props, bk


def _reduced(m, bk, size, fill):
    import torch
    from pyfe3d_gb300.solver import CSRPattern
    dev = torch.device('cuda')
    nk = size * m.E
    Kr = torch.zeros(nk, dtype=torch.int64, device=dev)
    Kc = torch.zeros_like(Kr)
    Kv = torch.zeros(nk, dtype=torch.float64, device=dev)
    fill(Kr, Kc, Kv)
    pat = CSRPattern(Kr, Kc, m.N, bk)
    return pat, pat.assemble(Kv)


def test_natural_frequencies_match_eigsh(gpulib):
    from scipy.sparse.linalg import eigsh
    from pyfe3d_gb300 import batch, eigen
    m, props, bk = _plate()
    pk, vk = _reduced(m, bk, 576, lambda r, c, v: batch.quad4_update_KC0(r, c, v, m.x, m.cdof, m.init_k(576), props))
    pm, vm = _reduced(m, bk, 480, lambda r, c, v: batch.quad4_update_M(r, c, v, m.x, m.cdof, m.init_k(480), props))
    assert pk.nrows == pm.nrows
    K, M = eigen.CSROperator(pk, vk), eigen.CSROperator(pm, vm)
    omega, X, info = eigen.natural_frequencies(K, M, 4, tol=1e-8)
    assert info['converged'], info
    ev = np.sort(eigsh(pk.to_scipy(vk).tocsc(), k=4, M=pm.to_scipy(vm).tocsc(), sigma=-1., which='LM')[0])
    assert np.allclose(omega ** 2, ev, rtol=1e-7), (omega ** 2, ev)
    # the modes are M-orthonormal
    G = (X.T @ M.matmul(X.contiguous())).cpu().numpy()
    assert np.abs(G - np.eye(4)).max() < 1e-8


def test_buckling_load_matches_dense_eigh(gpulib):
    from pyfe3d_gb300 import batch, eigen
    m, props, bk = _plate()
    Nxx = -1.
    pk, vk = _reduced(m, bk, 576, lambda r, c, v: batch.quad4_update_KC0(r, c, v, m.x, m.cdof, m.init_k(576), props))
    pg, vg = _reduced(m, bk, 144, lambda r, c, v: batch.quad4_update_KG_given_stress(r, c, v, m.x, m.cdof,
                                                                                      m.init_k(144), [Nxx, 0., 0.]))
    assert pk.nrows == pg.nrows
    lam, X, info = eigen.buckling(eigen.CSROperator(pk, vk), eigen.CSROperator(pg, vg), 3, tol=1e-6)
    assert info['converged'], info
    # dense generalised eigenproblem of the same matrices: the most negative mu
    import scipy.linalg
    mu = scipy.linalg.eigh(pg.to_scipy(vg).toarray(), pk.to_scipy(vk).toarray(), eigvals_only=True)
    ref = np.sort(-1. / mu[:3])
    assert np.allclose(np.sort(lam), ref, rtol=1e-6), (lam, ref)
    assert lam.min() > 0


def test_dense_projection_kernels_match_numpy(gpulib):
    """The LOBPCG's projection kernels: X^T Y (fixed-order sum of per-block
    partials; identical bits on a second call) and Y = beta Y + alpha X T."""
    import torch
    from pyfe3d_gb300 import eigen
    rng = np.random.default_rng(4)
    for n, k1, k2 in ((1, 1, 1), (1000, 7, 5), (123457, 64, 42)):
        X = rng.standard_normal((n, k1))
        Y = rng.standard_normal((n, k2))
        Xd, Yd = torch.from_numpy(X).cuda(), torch.from_numpy(Y).cuda()
        G = eigen.gram(Xd, Yd)
        ref = X.T @ Y
        assert np.abs(G - ref).max() <= 1e-12 * max(np.abs(ref).max(), 1.) * np.sqrt(n)
        assert np.array_equal(G, eigen.gram(Xd, Yd))
        T = rng.standard_normal((k1, k2))
        Z0 = rng.standard_normal((n, k2))
        Z = eigen.gemm(Xd, T, alpha=-0.5, beta=2., Y=torch.from_numpy(Z0).cuda()).cpu().numpy()
        refz = 2. * Z0 - 0.5 * X @ T
        assert np.abs(Z - refz).max() <= 1e-12 * np.abs(refz).max()
