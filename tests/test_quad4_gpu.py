"""Quad4 CUDA kernels against the reference's frozen outputs and the oracle."""
import numpy as np
import pytest

from conftest import REL_TOL, blockwise_rel_err

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(b).max(), 1e-300)


def _elements(golden):
    from pyfe3d_gb300 import Quad4, Quad4Probe
    from pyfe3d_gb300.shellprop import ShellProp, SHELL_FIELDS
    g = golden('quad4_elements')
    props = []
    for rec in g['props']:
        p = ShellProp()
        for i, f in enumerate(SHELL_FIELDS):
            setattr(p, f, float(rec[i]))
        props.append(p)
    return g, props, Quad4, Quad4Probe


def test_per_element_api_matches_reference(gpulib, golden):
    from pyfe3d_gb300 import INT
    g, props, Quad4, Quad4Probe = _elements(golden)
    probe = Quad4Probe()
    for t in range(len(g['x'])):
        q = Quad4(probe)
        q.c1, q.c2, q.c3, q.c4 = (int(v) for v in g['c'][t])
        xmat = g['xmat'][t]
        if np.isnan(xmat).any():
            q.update_rotation_matrix(g['x'][t])
        else:
            q.update_rotation_matrix(g['x'][t], *xmat)
        R = [q.r11, q.r12, q.r13, q.r21, q.r22, q.r23, q.r31, q.r32, q.r33]
        assert rel(R, g['R'][t]) < 1e-14
        assert rel([q.m11, q.m12, q.m21, q.m22], g['m'][t]) < 1e-14
        q.update_probe_xe(g['x'][t])
        assert rel(probe.xe, g['xe'][t]) < 1e-14
        # FP64 shoelace with fused multiply-adds on coordinates that agree to
        # rounding: the cancellation in the shoelace sum leaves ~1e-13
        assert abs(q.area - g['area'][t]) <= 1e-12 * g['area'][t]
        q.update_probe_ue(g['u'][t])
        assert rel(probe.ue, g['ue'][t]) < 1e-14
        prop = props[g['pid'][t]]
        # KC0 at a non-zero offset of a larger array, += onto existing values
        q.init_k_KC0 = 576
        r = np.zeros(3 * 576, INT); c = np.zeros(3 * 576, INT); v = np.zeros(3 * 576)
        v[576:1152] = 1.0
        q.update_KC0(r, c, v, prop)
        assert (r[576:1152] == g['KC0r'][t]).all() and (c[576:1152] == g['KC0c'][t]).all()
        assert blockwise_rel_err(v[576:1152] - 1.0, g['KC0v'][t], 576) < REL_TOL
        assert (v[:576] == 0).all() and (v[1152:] == 0).all() and (r[1152:] == 0).all()
        # values only: indices untouched
        r2 = np.full(576, -7, INT); c2 = np.full(576, -7, INT); v2 = np.zeros(576)
        q.init_k_KC0 = 0
        q.update_KC0(r2, c2, v2, prop, update_KC0v_only=1)
        assert (r2 == -7).all() and (c2 == -7).all()
        assert blockwise_rel_err(v2, g['KC0v'][t], 576) < REL_TOL
        if t < 4:
            # values only into a CUDA value array next to numpy index arrays:
            # the index arrays are neither checked as tensors nor written
            import torch
            v3 = torch.zeros(576, dtype=torch.float64, device='cuda')
            q.update_KC0(r2, c2, v3, prop, update_KC0v_only=1)
            assert (r2 == -7).all() and (c2 == -7).all()
            assert blockwise_rel_err(v3.cpu().numpy(), g['KC0v'][t], 576) < REL_TOL
        r = np.zeros(144, INT); c = np.zeros(144, INT); v = np.zeros(144)
        q.update_KG(r, c, v, prop)
        assert (r == g['KGr'][t]).all() and (c == g['KGc'][t]).all()
        assert blockwise_rel_err(v, g['KGv'][t], 144) < REL_TOL
        for mt, rk, ck, vk in ((0, 'M0r', 'M0c', 'M0v'), (1, 'M0r', 'M0c', 'M1v'),
                               (2, 'M2r', 'M2c', 'M2v')):
            r = np.zeros(480, INT); c = np.zeros(480, INT); v = np.zeros(480)
            q.update_M(r, c, v, prop, mtype=mt)
            assert (r == g[rk][t]).all() and (c == g[ck][t]).all(), mt
            assert blockwise_rel_err(v, g[vk][t], 480) < REL_TOL, mt
        f = np.zeros(24)
        q.update_fint(f, prop)
        assert rel(f, g['fint'][t]) < 1e-12


def _mesh(kind, seed=0):
    from pyfe3d_gb300.meshes import PlateMesh
    m = PlateMesh(13, 9, 1.3, 0.7, perturb=0.2, seed=seed)
    x = m.ncoords.copy()
    if kind == 'rotated':
        rng = np.random.default_rng(seed)
        q, _ = np.linalg.qr(rng.normal(size=(3, 3)))
        x = x @ q.T
    elif kind == 'curved':
        x[:, 2] = 0.2 * np.sin(2 * x[:, 0]) * np.cos(3 * x[:, 1])
    elif kind == 'offset':
        x[:, :2] += 1000.
    return m, x.ravel()


@pytest.mark.parametrize('kind', ['flat', 'rotated', 'curved', 'offset'])
@pytest.mark.parametrize('xmat', [False, True])
def test_batched_kc0_matches_oracle(gpulib, oracle, kind, xmat):
    from pyfe3d_gb300 import batch
    from pyfe3d_gb300.shellprop import isotropic_plate_records, shell_record
    from pyfe3d_gb300.shellprop_utils import laminated_plate
    m, x = _mesh(kind, seed=3)
    rng = np.random.default_rng(5)
    h = rng.uniform(0.002, 0.2, m.E)  # mixes thin and thick elements
    props = isotropic_plate_records(h, 70e9, 0.3, rho=2700.)
    lam = shell_record(laminated_plate([0, 45, -45, 90, 30], plyt=0.0011,
                                       laminaprop=(142.5e9, 8.7e9, 0.28, 5.1e9, 5.1e9, 5.1e9),
                                       offset=0.001))
    props[::3] = lam
    pid = rng.permutation(m.E).astype(np.int32)
    xm = rng.normal(size=(m.E, 3)) if xmat else None
    init_k = 576 * rng.permutation(m.E).astype(np.int64) + 576
    n = 576 * (m.E + 2)
    r0, c0, v0 = oracle.q4_kc0_batch(m.cdof, init_k, x, props, pid=pid, xmat=xm,
                                     Kr=np.zeros(n, np.int64), Kc=np.zeros(n, np.int64),
                                     Kv=np.full(n, 0.5))
    r = np.zeros(n, np.int64); c = np.zeros(n, np.int64); v = np.full(n, 0.5)
    batch.quad4_update_KC0(r, c, v, x, m.cdof, init_k, props, pid=pid, xmat=xm)
    assert (r == r0).all() and (c == c0).all()
    # Far from the origin (offset 1000 m for 0.1 m elements) the reference
    # loses log10(1000 / 0.1) = 4 digits to cancellation in the Jacobian
    # (coordinate differences of absolute local coordinates); the kernel
    # subtracts node 1 first, so agreement is bounded by the reference's own
    # rounding: 1e-12 scaled by the offset / element-size ratio.
    tol = REL_TOL * (1e4 if kind == 'offset' else 1.)
    assert blockwise_rel_err(v[576:-576] - 0.5, v0[576:-576] - 0.5, 576) < tol
    assert (v[:576] == 0.5).all() and (v[-576:] == 0.5).all()


def test_batched_kc0_cuda_tensors_in_place(gpulib, oracle):
    import torch
    from pyfe3d_gb300 import batch
    from pyfe3d_gb300.meshes import config1
    m, props, _, _, _ = config1()
    init_k = m.init_k(576)
    n = 576 * m.E
    r = torch.zeros(n, dtype=torch.int64, device='cuda')
    c = torch.zeros(n, dtype=torch.int64, device='cuda')
    v = torch.zeros(n, dtype=torch.float64, device='cuda')
    batch.quad4_update_KC0(r, c, v, m.x, m.cdof, init_k, props)
    r0, c0, v0 = oracle.q4_kc0_batch(m.cdof, init_k, m.x, props)
    assert (r.cpu().numpy() == r0).all() and (c.cpu().numpy() == c0).all()
    assert blockwise_rel_err(v.cpu().numpy(), v0, 576) < REL_TOL
    # a second update accumulates
    batch.quad4_update_KC0(r, c, v, m.x, m.cdof, init_k, props, update_KC0v_only=1)
    assert blockwise_rel_err(v.cpu().numpy(), 2 * v0, 576) < REL_TOL


@pytest.mark.parametrize('kind', ['flat', 'rotated'])
def test_batched_kg_and_m_match_oracle(gpulib, oracle, kind):
    from pyfe3d_gb300 import batch
    from pyfe3d_gb300.shellprop import isotropic_plate_records
    m, x = _mesh(kind, seed=7)
    rng = np.random.default_rng(1)
    props = isotropic_plate_records(rng.uniform(0.002, 0.02, m.E), 70e9, 0.3, rho=2700.)
    props[:, 6:12] = rng.normal(size=(m.E, 6)) * 1e3  # exercise B coupling in KG
    u = rng.normal(size=m.N) * 1e-3
    init_k = m.init_k(144)
    r0, c0, v0 = oracle.q4_kg_batch(m.cdof, init_k, x, u, props)
    n = 144 * m.E
    r = np.zeros(n, np.int64); c = np.zeros(n, np.int64); v = np.zeros(n)
    batch.quad4_update_KG(r, c, v, x, u, m.cdof, init_k, props)
    assert (r == r0).all() and (c == c0).all()
    assert blockwise_rel_err(v, v0, 144) < REL_TOL
    # += onto existing values: entries whose KG term is zero (on the flat
    # mesh all but the (w, w) couplings) keep the caller's value exactly
    v1 = rng.normal(size=n)
    v = v1.copy()
    batch.quad4_update_KG(r, c, v, x, u, m.cdof, init_k, props)
    assert blockwise_rel_err(v, v1 + v0, 144) < REL_TOL
    zero = v0 == 0.
    assert np.array_equal(v[zero], v1[zero])
    if kind == 'flat':
        assert zero.sum() >= 128 * m.E
    for mt in (0, 1, 2):
        init_k = m.init_k(480)
        r0, c0, v0 = oracle.q4_m_batch(m.cdof, init_k, x, props, mtype=mt)
        n = 480 * m.E
        r = np.zeros(n, np.int64); c = np.zeros(n, np.int64); v = np.zeros(n)
        batch.quad4_update_M(r, c, v, x, m.cdof, init_k, props, mtype=mt)
        assert (r == r0).all() and (c == c0).all()
        assert blockwise_rel_err(v, v0, 480) < REL_TOL


def test_out_of_range_offsets_raise(gpulib):
    from pyfe3d_gb300 import batch, _lib
    from pyfe3d_gb300.meshes import config1
    m, props, _, _, _ = config1()
    init_k = m.init_k(576)
    n = 576 * m.E - 10  # last element does not fit
    r = np.zeros(n, np.int64); c = np.zeros(n, np.int64); v = np.zeros(n)
    with pytest.raises(_lib.Fe3dError):
        batch.quad4_update_KC0(r, c, v, m.x, m.cdof, init_k, props)
    # the library is still usable afterwards
    n = 576 * m.E
    r = np.zeros(n, np.int64); c = np.zeros(n, np.int64); v = np.zeros(n)
    batch.quad4_update_KC0(r, c, v, m.x, m.cdof, init_k, props)
    assert np.isfinite(v).all()


def test_reference_point_load_plate(gpulib, golden):
    """tests/test_quad4_static_point_load.py of the reference through the
    per-element GPU API, solved with scipy's cg as in the reference test."""
    from scipy.sparse import coo_matrix
    from scipy.sparse.linalg import cg
    from pyfe3d_gb300 import Quad4, Quad4Data, Quad4Probe, INT, DOUBLE, DOF
    from pyfe3d_gb300.shellprop_utils import isotropic_plate
    data = Quad4Data()
    probe = Quad4Probe()
    nx, ny, a, b = 7, 11, 3, 7
    xtmp = np.linspace(0, a, nx)
    ytmp = np.linspace(0, b, ny)
    xmesh, ymesh = np.meshgrid(xtmp, ytmp)
    ncoords = np.vstack((xmesh.T.flatten(), ymesh.T.flatten(), np.zeros_like(ymesh.T.flatten()))).T
    x, y = ncoords[:, 0], ncoords[:, 1]
    ncf = ncoords.flatten()
    nids = 1 + np.arange(ncoords.shape[0])
    nid_pos = dict(zip(nids, np.arange(len(nids))))
    nm = nids.reshape(nx, ny)
    quads = []
    E = (nx - 1) * (ny - 1)
    KC0r = np.zeros(data.KC0_SPARSE_SIZE * E, dtype=INT)
    KC0c = np.zeros(data.KC0_SPARSE_SIZE * E, dtype=INT)
    KC0v = np.zeros(data.KC0_SPARSE_SIZE * E, dtype=DOUBLE)
    N = DOF * nx * ny
    prop = isotropic_plate(thickness=0.005, E=200e9, nu=0.3, calc_scf=True)
    init_k = 0
    for n1, n2, n3, n4 in zip(nm[:-1, :-1].flat, nm[1:, :-1].flat, nm[1:, 1:].flat,
                              nm[:-1, 1:].flat):
        q = Quad4(probe)
        q.c1, q.c2, q.c3, q.c4 = (DOF * nid_pos[n] for n in (n1, n2, n3, n4))
        q.init_k_KC0 = init_k
        q.K6ROT = 100.
        q.update_rotation_matrix(ncf)
        q.update_probe_xe(ncf)
        q.update_KC0(KC0r, KC0c, KC0v, prop)
        quads.append(q)
        init_k += data.KC0_SPARSE_SIZE
    KC0 = coo_matrix((KC0v, (KC0r, KC0c)), shape=(N, N)).tocsc()
    bk = np.zeros(N, dtype=bool)
    check = np.isclose(x, 0.) | np.isclose(x, a) | np.isclose(y, 0) | np.isclose(y, b)
    bk[2::DOF] = check
    bk[0::DOF] = True
    bk[1::DOF] = True
    bu = ~bk
    fext = np.zeros(N)
    fext[2::DOF][np.isclose(x, a / 2) & np.isclose(y, b / 2)] = 1.
    uu, info = cg(KC0[bu, :][:, bu], fext[bu], atol=1e-9)
    assert info == 0
    u = np.zeros(N)
    u[bu] = uu
    assert np.isclose(6.496928101916171e-05, u[2::DOF].max(), rtol=0.02)
    # equilibrium through update_fint (reference :117-132)
    fint = np.zeros(N)
    for q in quads:
        q.update_probe_xe(ncf)
        q.update_probe_ue(u)
        q.update_fint(fint, prop)
    fext[bk] = KC0[bk, :][:, bu] @ u[bu]
    assert np.allclose(fint, fext, atol=1e-5)


def test_config2_plate_kc0_matches_oracle(gpulib, oracle):
    """The measured workload's generator (perturbed clamped plate, one
    property record per element) at 41x41 nodes, every element compared."""
    from pyfe3d_gb300 import batch
    from pyfe3d_gb300.meshes import config2
    m, props, pid, bk, f = config2(41)
    init_k = m.init_k(576)
    r0, c0, v0 = oracle.q4_kc0_batch(m.cdof, init_k, m.x, props, pid=pid)
    n = 576 * m.E
    r = np.zeros(n, np.int64); c = np.zeros(n, np.int64); v = np.zeros(n)
    batch.quad4_update_KC0(r, c, v, m.x, m.cdof, init_k, props, pid=pid)
    assert (r == r0).all() and (c == c0).all()
    assert blockwise_rel_err(v, v0, 576) < REL_TOL


def test_config2_full_size_sampled(gpulib, oracle):
    """Full 1001x1001-node plate (1,000,000 elements, 576M triplets) on the
    device; 3000 random elements are checked against the oracle and every
    element block is checked for symmetry (a size-independent property)."""
    import torch
    from pyfe3d_gb300 import batch
    from pyfe3d_gb300.meshes import config2
    m, props, pid, bk, f = config2(1001)
    n = 576 * m.E
    dev = torch.device('cuda')
    r = torch.zeros(n, dtype=torch.int64, device=dev)
    c = torch.zeros(n, dtype=torch.int64, device=dev)
    v = torch.zeros(n, dtype=torch.float64, device=dev)
    batch.quad4_update_KC0(r, c, v, m.x, m.cdof, m.init_k(576), props, pid=pid)
    V = v.view(m.E, 24, 24)
    asym = (V - V.transpose(1, 2)).abs().amax(dim=(1, 2)) / V.abs().amax(dim=(1, 2))
    assert float(asym.max()) < 1e-13
    rng = np.random.default_rng(11)
    sample = np.sort(rng.choice(m.E, 3000, replace=False))
    idx = torch.as_tensor(sample, device=dev)
    vs = v.view(m.E, 576)[idx].cpu().numpy().ravel()
    rs = r.view(m.E, 576)[idx].cpu().numpy().ravel()
    r0, c0, v0 = oracle.q4_kc0_batch(m.cdof[sample], 576 * np.arange(len(sample)), m.x, props,
                                     pid=pid[sample])
    assert (rs == r0).all()
    assert blockwise_rel_err(vs, v0, 576) < REL_TOL
    del r, c, v, V
    torch.cuda.empty_cache()
