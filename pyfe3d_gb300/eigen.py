"""Generalised symmetric eigenproblems on the device: LOBPCG.

Stands in for the reference tests' shift-invert ``eigsh`` calls on the
reduced matrices:

* natural frequencies, ``K x = lam M x``, smallest lam
  (tests/test_quad4_natural_freq.py:117-120): ``lobpcg(K, M, k)``;
* linear buckling, ``KC0 x = -lam KG x``, smallest load multiplier
  (tests/test_quad4_linear_buckling_plate_rotated.py:129-131): solved as
  ``KG x = mu KC0 x`` for the most negative mu, lam = -1/mu:
  ``buckling(KC0, KG, k)``.

The block products A X, B X run in the library's CSR SpMM kernel
(``fe3d_spmm``), the preconditioner is the 6x6 nodal block-Jacobi of the
SPD matrix (``fe3d_solver_precond_multi``) or a few PCG iterations per
column; the Rayleigh-Ritz projections (X^T Y and X T of tall-skinny blocks)
run in the library's dense kernels (``fe3d_dense_gram``, a fixed-order sum of
per-block partials, and ``fe3d_dense_gemm_tall``) and the small projected
eigenproblems (3m x 3m) are solved on the host.
"""
import numpy as np
import scipy.linalg

from . import _lib
from .solver import Solver


class CSROperator:
    """A reduced CSR matrix (pattern + values) applied to row-major blocks."""

    def __init__(self, pattern, vals):
        self.pattern = pattern
        self.vals = vals
        self.n = pattern.nrows
        self.device = vals.device

    def matmul(self, X, Y=None):
        lib = _lib.load()
        torch = _lib.torch_mod()
        X = X.contiguous()
        k = X.shape[1]
        if Y is None:
            Y = torch.empty_like(X)
        for j0 in range(0, k, 16):
            j1 = min(k, j0 + 16)
            xs = X[:, j0:j1].contiguous() if (j0 or j1 < k) else X
            ys = torch.empty_like(xs) if (j0 or j1 < k) else Y
            rc = lib.fe3d_spmm(self.pattern.handle, _lib.ptr(self.vals), _lib.ptr(xs), _lib.ptr(ys), j1 - j0,
                               _lib.stream_ptr())
            _lib.check(rc, 'fe3d_spmm')
            if ys is not Y:
                Y[:, j0:j1] = ys
        return Y


class BlockJacobi:
    """Z = Dinv R with the nodal block inverses of an SPD matrix."""

    def __init__(self, op):
        self.solver = Solver(op.pattern).setup(op.vals)

    def __call__(self, R):
        lib = _lib.load()
        torch = _lib.torch_mod()
        R = R.contiguous()
        Z = torch.empty_like(R)
        rc = lib.fe3d_solver_precond_multi(self.solver._h, _lib.ptr(R), _lib.ptr(Z), R.shape[1], _lib.stream_ptr())
        _lib.check(rc, 'fe3d_solver_precond_multi')
        return Z


class InnerPCG:
    """Z ~ A^-1 R column by column: a fixed number of block-Jacobi PCG
    iterations of the library's solver (a variable preconditioner, which
    LOBPCG tolerates)."""

    def __init__(self, op, iters=20):
        self.solver = Solver(op.pattern).setup(op.vals)
        self.iters = int(iters)

    def __call__(self, R):
        torch = _lib.torch_mod()
        Z = torch.empty_like(R)
        for j in range(R.shape[1]):
            z, _ = self.solver.solve(R[:, j].contiguous(), tol=1e-300, maxiter=self.iters,
                                     check_every=self.iters + (self.iters & 1))
            Z[:, j] = z
        return Z


MAX_BLOCK = 64  # columns of the blocks the dense kernels take
_scratch = {}


def gram(X, Y):
    """X^T Y (host numpy, k1 x k2) of row-major n x k1 and n x k2 device
    blocks by the library's Gram kernel (deterministic)."""
    lib = _lib.load()
    torch = _lib.torch_mod()
    X = X.contiguous()
    Y = Y.contiguous()
    n, k1 = X.shape
    k2 = Y.shape[1]
    G = torch.empty((k1, k2), dtype=torch.float64, device=X.device)
    need = int(lib.fe3d_dense_gram_scratch(k1, k2))
    buf = _scratch.get(X.device)
    if buf is None or buf.numel() < need:
        buf = torch.empty(need, dtype=torch.float64, device=X.device)
        _scratch[X.device] = buf
    rc = lib.fe3d_dense_gram(n, k1, k2, _lib.ptr(X), _lib.ptr(Y), _lib.ptr(G), _lib.ptr(buf), _lib.stream_ptr())
    _lib.check(rc, 'fe3d_dense_gram')
    return G.cpu().numpy()


def gemm(X, T, alpha=1., beta=0., Y=None):
    """Y = beta Y + alpha X T for a row-major n x k device block X and a small
    k x m matrix T (numpy); a new Y when Y is None (beta ignored)."""
    lib = _lib.load()
    torch = _lib.torch_mod()
    X = X.contiguous()
    T = torch.from_numpy(np.ascontiguousarray(T, dtype=np.float64)).to(X.device)
    n, k = X.shape
    m = T.shape[1]
    if Y is None:
        Y = torch.empty((n, m), dtype=torch.float64, device=X.device)
        beta = 0.
    rc = lib.fe3d_dense_gemm_tall(n, k, m, _lib.ptr(X), _lib.ptr(T), float(alpha), float(beta), _lib.ptr(Y),
                                  _lib.stream_ptr())
    _lib.check(rc, 'fe3d_dense_gemm_tall')
    return Y


def _col_norms(V):
    return np.sqrt(np.maximum(np.diag(gram(V, V)), 0.))


def _b_orthonormalize(V, BV, AV=None):
    """V, BV (and AV) -> times L^-T with V^T B V = L L^T; None if singular."""
    G = gram(V, BV)
    G = 0.5 * (G + G.T)
    try:
        L = np.linalg.cholesky(G)
    except np.linalg.LinAlgError:
        return None
    Linv = np.linalg.inv(L).T
    return (gemm(V, Linv), gemm(BV, Linv)) if AV is None else (gemm(V, Linv), gemm(BV, Linv), gemm(AV, Linv))


def lobpcg(A, B, k, precond=None, m=None, X0=None, tol=1e-8, maxiter=2000, seed=0, verbose=False):
    """The k smallest eigenpairs of A x = lam B x (A symmetric, B SPD; B None
    for the identity) by block LOBPCG (Knyazev 2001) with block size m >= k.

    Returns (lam (k,), X (n, k) CUDA tensor B-orthonormal, info dict with the
    iteration count and the relative residuals
    ||A x - lam B x|| / (||A x|| + |lam| ||B x||))."""
    torch = _lib.torch_mod()
    dev = getattr(A, 'device', None) or _lib.device()
    n = A.n
    m = max(k, m if m is not None else min(k + 4, 2 * k))
    if 3 * m > n:
        raise ValueError('the block (%d) is too large for n = %d' % (m, n))
    if 3 * m > MAX_BLOCK:
        raise ValueError('block size %d: the projections take at most %d columns (3 m)' % (m, MAX_BLOCK))
    Bmul = (lambda V: B.matmul(V)) if B is not None else (lambda V: V.clone())
    T = precond if precond is not None else (lambda R: R)
    if X0 is None:
        rng = np.random.default_rng(seed)
        X = torch.from_numpy(rng.standard_normal((n, m))).to(dev)
    else:
        X = _lib.to_device(X0, np.float64).reshape(n, -1)
        if X.shape[1] < m:
            rng = np.random.default_rng(seed)
            X = torch.cat([X, torch.from_numpy(rng.standard_normal((n, m - X.shape[1]))).to(dev)], 1)
    X = X.contiguous()
    r = _b_orthonormalize(X, Bmul(X))
    if r is None:
        raise RuntimeError('initial block is B-singular')
    X, BX = r
    AX = A.matmul(X)
    H = gram(X, AX)
    theta, C = scipy.linalg.eigh(0.5 * (H + H.T))
    X, AX, BX = gemm(X, C), gemm(AX, C), gemm(BX, C)
    P = AP = BP = None
    res = np.full(m, np.inf)
    it = 0
    for it in range(1, maxiter + 1):
        R = gemm(BX, -np.diag(theta[:m]), beta=1., Y=AX.clone())  # A X - B X diag(theta)
        rn = _col_norms(R)
        den = _col_norms(AX) + np.abs(theta[:m]) * _col_norms(BX)
        res = rn / np.maximum(den, 1e-300)
        if verbose and it % 50 == 0:
            print(it, theta[:k], res[:k].max())
        if (res[:k] <= tol).all():
            break
        W = T(R)
        # B-orthogonalise the residual directions against X, then among themselves
        BW = Bmul(W)
        W = gemm(X, gram(X, BW), alpha=-1., beta=1., Y=W.clone())  # W - X (X^T B W)
        BW = Bmul(W)
        r = _b_orthonormalize(W, BW)
        if r is None:
            P = None
            continue
        W, BW = r
        AW = A.matmul(W)
        blocks = [(X, AX, BX), (W, AW, BW)]
        if P is not None:
            r = _b_orthonormalize(P, BP, AP)
            if r is not None:
                P, BP, AP = r
                blocks.append((P, AP, BP))
        S = torch.cat([b[0] for b in blocks], 1)
        AS = torch.cat([b[1] for b in blocks], 1)
        BS = torch.cat([b[2] for b in blocks], 1)
        GA = gram(S, AS)
        GB = gram(S, BS)
        GA = 0.5 * (GA + GA.T)
        GB = 0.5 * (GB + GB.T)
        try:
            theta_all, Call = scipy.linalg.eigh(GA, GB)
        except (np.linalg.LinAlgError, ValueError):
            # drop the P block and retry with [X, W]
            P = None
            S, AS, BS = S[:, :2 * m], AS[:, :2 * m], BS[:, :2 * m]
            GA = gram(S, AS)
            GB = gram(S, BS)
            theta_all, Call = scipy.linalg.eigh(0.5 * (GA + GA.T), 0.5 * (GB + GB.T))
        theta = theta_all[:m]
        Cm = np.ascontiguousarray(Call[:, :m])
        Cp = Cm.copy()
        Cp[:m] = 0.  # the non-X part of the update is the next search direction
        X, AX, BX = gemm(S, Cm), gemm(AS, Cm), gemm(BS, Cm)
        P, AP, BP = gemm(S, Cp), gemm(AS, Cp), gemm(BS, Cp)
    info = {'iterations': it, 'residuals': res[:k].copy(), 'converged': bool((res[:k] <= tol).all())}
    return theta[:k].copy(), X[:, :k], info


def natural_frequencies(K, M, k, tol=1e-8, precond='pcg', **kw):
    """Smallest k eigenvalues lam = omega^2 of K x = lam M x (reduced CSR
    operators); returns (omega, modes, info)."""
    T = InnerPCG(K) if precond == 'pcg' else BlockJacobi(K)
    lam, X, info = lobpcg(K, M, k, precond=T, tol=tol, **kw)
    return np.sqrt(np.maximum(lam, 0.)), X, info


def buckling(KC0, KG, k, tol=1e-6, precond='pcg', inner=50, **kw):
    """Smallest k load multipliers lam of KC0 x = -lam KG x: the most
    negative mu of KG x = mu KC0 x, lam = -1 / mu; returns (lam, modes, info).
    The residual tolerance applies to the (KG, KC0) pencil, whose buckling
    eigenvalues sit next to the large null space of KG; the load multipliers
    are accurate to about the square of it."""
    T = InnerPCG(KC0, iters=inner) if precond == 'pcg' else BlockJacobi(KC0)
    mu, X, info = lobpcg(KG, KC0, k, precond=T, tol=tol, **kw)
    return -1. / mu, X, info
