"""CPU oracle of the learned block preconditioner (test infrastructure only).

The learned preconditioner has no counterpart in the reference (whose tests
solve with spsolve/cg: tests/test_quad4_static_point_load.py:102); this
module restates, in float64 numpy, the computation the CUDA kernels perform
so the tests can check the features, the MLP forward pass, the
preconditioner blocks, the loss and every weight gradient against it.  Its
own gradient is pinned by central finite differences in the tests.

Layout (shared with the kernels): weights W1[64][35] b1[64] W2[64][64]
b2[64] W3[21][64] b3[21]; outputs are the upper triangle (row-major) of the
symmetric 6x6 correction C of each node in the coordinates S^-1 D S^-1,
S = sqrt(diag K); the block is B = D + scale S C S over the free DOFs.
"""
import numpy as np

NF, NH, NO = 35, 64, 21
OW1 = 0
OB1 = OW1 + NH * NF
OW2 = OB1 + NH
OB2 = OW2 + NH * NH
OW3 = OB2 + NH
OB3 = OW3 + NO * NH
NW = OB3 + NO


def ut_index(i, k):
    return i * 6 - i * (i - 1) // 2 + (k - i)


def off_index(i, k):
    return i * 5 - i * (i - 1) // 2 + (k - i - 1)


def unpack(W):
    W = np.asarray(W, dtype=np.float64)
    return (W[OW1:OB1].reshape(NH, NF), W[OB1:OW2], W[OW2:OB2].reshape(NH, NH), W[OB2:OW3],
            W[OW3:OB3].reshape(NO, NH), W[OB3:NW])


def node_rows(dof_of_row, nnodes):
    """Rows of each node (free DOFs in increasing DOF order)."""
    rows = [[] for _ in range(nnodes)]
    for r, d in enumerate(np.asarray(dof_of_row)):
        rows[int(d) // 6].append(r)
    return rows


def features(K, dof_of_row, nnodes):
    K = K.tocsr()
    dof_of_row = np.asarray(dof_of_row)
    d = K.diagonal()
    sdiag = np.where(d > 0, np.sqrt(np.where(d > 0, d, 1.)), 1.)
    rows = node_rows(dof_of_row, nnodes)
    feat = np.zeros((nnodes, NF))
    for j, rs in enumerate(rows):
        if not rs:
            continue
        li = [int(dof_of_row[r]) - 6 * j for r in rs]
        ld = [2 * np.log(sdiag[r]) for r in rs]
        mean = np.mean(ld)
        nsum = {}
        for a, r in enumerate(rs):
            feat[j, 15 + li[a]] = (ld[a] - mean) / 10.
            feat[j, 21 + li[a]] = 1.
            for b in range(a + 1, len(rs)):
                feat[j, off_index(li[a], li[b])] = K[r, rs[b]] / (sdiag[r] * sdiag[rs[b]])
            for k in range(K.indptr[r], K.indptr[r + 1]):
                c = K.indices[k]
                nd = int(dof_of_row[c]) // 6
                if nd == j:
                    continue
                nsum[nd] = nsum.get(nd, 0.) + (K.data[k] / (sdiag[r] * sdiag[c])) ** 2
        norms = sorted((np.sqrt(v) for v in nsum.values()), reverse=True)[:8]
        feat[j, 27:27 + len(norms)] = norms
    return feat, sdiag


def features29(K, dof_of_row, nnodes):
    """Feature set 1: the 21 unique entries of S^-1 D S^-1 (upper triangle)
    and the 8 largest Frobenius norms of S_j^-1 K_jk S_k^-1 (slots 29-34 zero)."""
    K = K.tocsr()
    dof_of_row = np.asarray(dof_of_row)
    d = K.diagonal()
    sdiag = np.where(d > 0, np.sqrt(np.where(d > 0, d, 1.)), 1.)
    rows = node_rows(dof_of_row, nnodes)
    feat = np.zeros((nnodes, NF))
    for j, rs in enumerate(rows):
        if not rs:
            continue
        li = [int(dof_of_row[r]) - 6 * j for r in rs]
        nsum = {}
        for a, r in enumerate(rs):
            for b in range(a, len(rs)):
                feat[j, ut_index(li[a], li[b])] = K[r, rs[b]] / (sdiag[r] * sdiag[rs[b]])
            for k in range(K.indptr[r], K.indptr[r + 1]):
                c = K.indices[k]
                nd = int(dof_of_row[c]) // 6
                if nd == j:
                    continue
                nsum[nd] = nsum.get(nd, 0.) + (K.data[k] / (sdiag[r] * sdiag[c])) ** 2
        norms = sorted((np.sqrt(v) for v in nsum.values()), reverse=True)[:8]
        feat[j, 21:21 + len(norms)] = norms
    return feat, sdiag


def forward(feat, W):
    W1, b1, W2, b2, W3, b3 = unpack(W)
    h1 = np.tanh(feat @ W1.T + b1)
    h2 = np.tanh(h1 @ W2.T + b2)
    out = h2 @ W3.T + b3
    return out, h1, h2


def correction(o):
    C = np.zeros((6, 6))
    for i in range(6):
        for k in range(i, 6):
            C[i, k] = C[k, i] = o[ut_index(i, k)]
    return C


def blocks(K, dof_of_row, nnodes, sdiag, out, scale):
    """B_j over the node's free DOFs (list of arrays) and the local DOFs."""
    K = K.tocsr()
    rows = node_rows(dof_of_row, nnodes)
    Bs, lis = [], []
    for j, rs in enumerate(rows):
        li = [int(dof_of_row[r]) - 6 * j for r in rs]
        D = K[rs][:, rs].toarray() if rs else np.zeros((0, 0))
        C = correction(out[j])[np.ix_(li, li)]
        s = sdiag[rs]
        Bs.append(D + scale * s[:, None] * s[None, :] * C)
        lis.append(li)
    return Bs, lis, rows


def block_inverses(K, dof_of_row, nnodes, Bs, rows):
    """Inverse of each B_j (Cholesky succeeds) or of the diagonal block."""
    K = K.tocsr()
    inv, fallback = [], []
    for j, rs in enumerate(rows):
        B = Bs[j]
        try:
            np.linalg.cholesky(B) if len(rs) else None
            inv.append(np.linalg.inv(B) if len(rs) else B)
            fallback.append(False)
        except np.linalg.LinAlgError:
            inv.append(np.linalg.inv(K[rs][:, rs].toarray()))
            fallback.append(True)
    return inv, np.array(fallback)


def apply(inv, rows, r):
    z = np.zeros_like(r)
    for j, rs in enumerate(rows):
        if rs:
            z[rs] = inv[j] @ r[rs]
    return z


def loss_grad_out(K, dof_of_row, nnodes, sdiag, inv, fallback, rows, r, w, scale, mode=0, factor=1.):
    """Loss and dL/d(outputs) for one residual sample (w = 1 / (e.r)):
    mode 0: L = factor w (z.Kz - 2 z.r); mode 1: L = factor (1 - w (z.r)^2 / z.Kz)."""
    z = apply(inv, rows, r)
    Kz = K @ z
    if mode == 0:
        L = factor * w * (z @ Kz - 2 * z @ r)
        g = 2 * factor * w * (Kz - r)
    else:
        a, b = z @ r, z @ Kz
        L = factor * (1 - w * a * a / b)
        g = factor * (2 * w * a / b) * ((a / b) * Kz - r)
    gout = np.zeros((nnodes, NO))
    for j, rs in enumerate(rows):
        if not rs or fallback[j]:
            continue
        li = [int(dof_of_row[q]) - 6 * j for q in rs]
        wv = inv[j] @ g[rs]
        s = sdiag[rs]
        G = -scale * (s * wv)[:, None] * (s * z[rs])[None, :]
        for a in range(len(rs)):
            for b in range(a, len(rs)):
                p, q = min(li[a], li[b]), max(li[a], li[b])
                gout[j, ut_index(p, q)] += G[a, b] + (G[b, a] if a != b else 0.)
    return L, gout


def backward(feat, W, h1, h2, gout):
    W1, b1, W2, b2, W3, b3 = unpack(W)
    d3 = gout
    d2 = (d3 @ W3) * (1 - h2 ** 2)
    d1 = (d2 @ W2) * (1 - h1 ** 2)
    grad = np.zeros(NW)
    grad[OW3:OB3] = (d3.T @ h2).ravel()
    grad[OB3:NW] = d3.sum(0)
    grad[OW2:OB2] = (d2.T @ h1).ravel()
    grad[OB2:OW3] = d2.sum(0)
    grad[OW1:OB1] = (d1.T @ feat).ravel()
    grad[OB1:OW2] = d1.sum(0)
    return grad


def loss_and_grad(K, dof_of_row, nnodes, W, samples, weights, scale, mode=0, factor=1.):
    """Total loss over residual samples and its gradient in the weights."""
    feat, sdiag = features(K, dof_of_row, nnodes)
    out, h1, h2 = forward(feat, W)
    Bs, lis, rows = blocks(K, dof_of_row, nnodes, sdiag, out, scale)
    inv, fallback = block_inverses(K, dof_of_row, nnodes, Bs, rows)
    L = 0.
    gout = np.zeros((nnodes, NO))
    for r, w in zip(samples, weights):
        l, g = loss_grad_out(K, dof_of_row, nnodes, sdiag, inv, fallback, rows, r, w, scale, mode, factor)
        L += l
        gout += g
    return L, backward(feat, W, h1, h2, gout), gout


def init_weights(seed=0, out_std=0.05):
    rng = np.random.default_rng(seed)
    W = np.zeros(NW)
    W[OW1:OB1] = rng.normal(0, 1 / np.sqrt(NF), NH * NF)
    W[OW2:OB2] = rng.normal(0, 1 / np.sqrt(NH), NH * NH)
    W[OW3:OB3] = rng.normal(0, out_std / np.sqrt(NH), NO * NH)
    return W
