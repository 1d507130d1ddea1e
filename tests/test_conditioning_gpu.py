"""Quad4 KC0 and KG on ill-conditioned flat elements against the oracle.

The KC0 kernel evaluates the Jacobian, its inverse and the shape-function
derivative products of elements flat in the XY plane in float-float
arithmetic (about 48 significant bits on the FP32 pipe) and the blocks in
FP64.  Cancellation in det J multiplies the rounding error of both the
oracle (FP64, the reference's order of operations, quad4.pyx:755-1171) and
the kernel by the element's conditioning, so these cases check that the
float-float evaluation still meets the 1e-12 per-element contract where
the conditioning is poor: interior nodes moved by up to 0.45 of the element
size (beyond the reference's own distorted-mesh test, 0.4,
tests/test_quad4_natural_freq_distorted_mat_coord.py:48-54), elements of
aspect ratio 1:1000, and quadrilaterals with one angle below 5 degrees.
"""
import numpy as np
import pytest

from conftest import REL_TOL, blockwise_rel_err

pytestmark = pytest.mark.gpu

LAM = (142.5e9, 8.7e9, 0.28, 5.1e9, 5.1e9, 5.1e9)
KINDS = ['perturbed_045', 'aspect_1000', 'aspect_1000_perturbed', 'sliver_5deg']


def _props(E, rng, laminated):
    from pyfe3d_gb300.shellprop import isotropic_plate_records, shell_record
    from pyfe3d_gb300.shellprop_utils import laminated_plate
    if laminated:
        return shell_record(laminated_plate([0, 45, -45, 90, 30], plyt=0.0011, laminaprop=LAM,
                                            offset=0.001))[None, :], None
    h = rng.uniform(0.0005, 0.3, E)  # thin and thick elements
    return isotropic_plate_records(h, 70e9, 0.3), np.arange(E, dtype=np.int32)


def sliver_quads(E, rng, max_angle_deg=5.):
    """E convex quadrilaterals in the XY plane, each with one interior angle
    below max_angle_deg, random size, position and orientation (4 nodes
    each, no sharing)."""
    quads = []
    while len(quads) < E:
        th = np.deg2rad(rng.uniform(0.5, max_angle_deg))
        L1, L2 = rng.uniform(0.5, 2.0, 2)
        p1 = np.zeros(2)
        p2 = np.array([L1, 0.])
        p4 = L2 * np.array([np.cos(th), np.sin(th)])
        # the third node just beyond the p2-p4 diagonal keeps the quad convex
        t = rng.uniform(0.2, 0.8)
        p3 = p2 + t * (p4 - p2) + rng.uniform(0.05, 0.5) * L1 * np.sin(th) * np.array([np.sin(th), np.cos(th)])
        q = np.array([p1, p2, p3, p4])
        ok = True
        for k in range(4):
            a, b, c = q[k - 1], q[k], q[(k + 1) % 4]
            d1, d2 = b - a, c - b
            if d1[0] * d2[1] - d1[1] * d2[0] <= 0:
                ok = False
        if not ok:
            continue
        ang = []
        for k in range(4):
            u, v = q[k - 1] - q[k], q[(k + 1) % 4] - q[k]
            ang.append(np.degrees(np.arccos(np.dot(u, v) / np.linalg.norm(u) / np.linalg.norm(v))))
        if min(ang) >= max_angle_deg:
            continue
        phi = rng.uniform(0, 2 * np.pi)
        R = np.array([[np.cos(phi), -np.sin(phi)], [np.sin(phi), np.cos(phi)]])
        q = q @ R.T + rng.uniform(-5, 5, 2)
        quads.append(q)
    q = np.array(quads)
    x = np.zeros((4 * E, 3))
    x[:, :2] = q.reshape(-1, 2)
    cdof = (6 * np.arange(4 * E)).reshape(E, 4).astype(np.int64)
    return x.ravel(), cdof


def _mesh(kind, rng):
    from pyfe3d_gb300.meshes import PlateMesh
    if kind == 'perturbed_045':
        m = PlateMesh(21, 17, 1.2, 0.9, perturb=0.45, seed=int(rng.integers(1 << 20)))
        return m.x, m.cdof
    if kind == 'aspect_1000':
        m = PlateMesh(9, 9, 1.0, 1e-3)
        return m.x, m.cdof
    if kind == 'aspect_1000_perturbed':
        m = PlateMesh(9, 9, 1.0, 1e-3, perturb=0.3, seed=5)
        return m.x, m.cdof
    return sliver_quads(160, rng)


@pytest.mark.parametrize('laminated', [False, True])
@pytest.mark.parametrize('kind', KINDS)
def test_ill_conditioned_flat_elements_match_oracle(gpulib, oracle, kind, laminated):
    from pyfe3d_gb300 import batch
    rng = np.random.default_rng(2 * KINDS.index(kind) + int(laminated))
    x, cdof = _mesh(kind, rng)
    E = cdof.shape[0]
    props, pid = _props(E, rng, laminated)
    init_k = 576 * np.arange(E, dtype=np.int64)
    r0, c0, v0 = oracle.q4_kc0_batch(cdof, init_k, x, props, pid=pid)
    n = 576 * E
    r = np.zeros(n, np.int64); c = np.zeros(n, np.int64); v = np.zeros(n)
    batch.quad4_update_KC0(r, c, v, x, cdof, init_k, props, pid=pid)
    assert (r == r0).all() and (c == c0).all()
    err = blockwise_rel_err(v, v0, 576)
    assert err < REL_TOL, (kind, laminated, err)


@pytest.mark.parametrize('kind', KINDS)
def test_ill_conditioned_flat_elements_kg_match_oracle(gpulib, oracle, kind):
    """Quad4 KG (float-float Jacobian and derivatives on flat elements, FP64
    strains, stress resultants and blocks) on the same meshes, from a random
    displacement field, against the oracle (quad4.pyx:1365-2257)."""
    from pyfe3d_gb300 import batch
    rng = np.random.default_rng(100 + KINDS.index(kind))
    x, cdof = _mesh(kind, rng)
    E = cdof.shape[0]
    props, pid = _props(E, rng, False)
    props[:, 6:12] = rng.normal(size=(len(props), 6)) * 1e3  # B coupling in the resultants
    N = int(cdof.max()) + 6
    u = rng.normal(size=N) * 1e-3
    init_k = 144 * np.arange(E, dtype=np.int64)
    r0, c0, v0 = oracle.q4_kg_batch(cdof, init_k, x, u, props, pid=pid)
    n = 144 * E
    r = np.zeros(n, np.int64); c = np.zeros(n, np.int64); v = np.zeros(n)
    batch.quad4_update_KG(r, c, v, x, u, cdof, init_k, props, pid=pid)
    assert (r == r0).all() and (c == c0).all()
    err = blockwise_rel_err(v, v0, 144)
    assert err < REL_TOL, (kind, err)
