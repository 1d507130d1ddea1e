"""Tria3R and Quad4R CUDA kernels against the reference's frozen outputs and
the oracle (pyfe3d/tria3r.pyx, pyfe3d/quad4r.pyx)."""
import numpy as np
import pytest

from conftest import REL_TOL, blockwise_rel_err

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(b).max(), 1e-300)


def _props(g):
    from pyfe3d_gb300.shellprop import ShellProp, SHELL_FIELDS
    props = []
    for rec in g['props']:
        p = ShellProp()
        for i, f in enumerate(SHELL_FIELDS):
            setattr(p, f, float(rec[i]))
        props.append(p)
    return props


def test_tria3r_per_element_api_matches_reference(gpulib, golden):
    from pyfe3d_gb300 import INT, Tria3R, Tria3RProbe
    g = golden('tria3r_elements')
    props = _props(g)
    probe = Tria3RProbe()
    for t in range(len(g['x'])):
        el = Tria3R(probe)
        el.c1, el.c2, el.c3 = (int(v) for v in g['c'][t])
        el.K6ROT = float(g['k6rot'][t])
        el.alpha_shear_locking = float(g['alpha'][t])
        xmat = g['xmat'][t]
        if np.isnan(xmat).any():
            el.update_rotation_matrix(g['x'][t])
        else:
            el.update_rotation_matrix(g['x'][t], *xmat)
        R = [el.r11, el.r12, el.r13, el.r21, el.r22, el.r23, el.r31, el.r32, el.r33]
        assert rel(R, g['R'][t]) < 1e-14
        # m11 = m22 = cos(theta) to 1e-14; m12 = -m21 = +-sqrt(1 - cos^2) amplifies
        # a one-ulp difference of cos(theta) by cos/sin, so its bound scales so
        mr = np.asarray(g['m'][t])
        assert rel([el.m11, el.m22], mr[[0, 3]]) < 1e-14
        sin_bound = 1e-15 / max(abs(mr[1]), 1e-3)
        assert abs(el.m12 - mr[1]) <= sin_bound and abs(el.m21 - mr[2]) <= sin_bound
        el.update_probe_xe(g['x'][t])
        assert rel(probe.xe, g['xe'][t]) < 1e-14
        assert abs(el.area - g['area'][t]) <= 1e-13 * g['area'][t]
        el.update_probe_ue(g['u'][t])
        assert rel(probe.ue, g['ue'][t]) < 1e-14
        prop = props[g['pid'][t]]
        # KC0 at a non-zero offset of a larger array, += onto existing values
        el.init_k_KC0 = 324
        r = np.zeros(3 * 324, INT); c = np.zeros(3 * 324, INT); v = np.zeros(3 * 324)
        v[324:648] = 1.0
        el.update_KC0(r, c, v, prop)
        assert (r[324:648] == g['KC0r'][t]).all() and (c[324:648] == g['KC0c'][t]).all()
        assert blockwise_rel_err(v[324:648] - 1.0, g['KC0v'][t], 324) < REL_TOL
        assert (v[:324] == 0).all() and (v[648:] == 0).all() and (r[648:] == 0).all()
        r2 = np.full(324, -7, INT); c2 = np.full(324, -7, INT); v2 = np.zeros(324)
        el.init_k_KC0 = 0
        el.update_KC0(r2, c2, v2, prop, update_KC0v_only=1)
        assert (r2 == -7).all() and (c2 == -7).all()
        assert blockwise_rel_err(v2, g['KC0v'][t], 324) < REL_TOL
        r = np.zeros(81, INT); c = np.zeros(81, INT); v = np.zeros(81)
        el.update_KG(r, c, v, prop)
        assert (r == g['KGr'][t]).all() and (c == g['KGc'][t]).all()
        assert blockwise_rel_err(v, g['KGv'][t], 81) < REL_TOL
        r = np.full(81, -3, INT); c = np.full(81, -3, INT); v = np.zeros(81)
        el.update_KG_given_stress(*g['Nstress'][t], r, c, v, update_KGv_only=1)
        assert (r == -3).all() and (c == -3).all()
        assert blockwise_rel_err(v, g['KGsv'][t], 81) < REL_TOL
        for mt, rk, ck, vk, n in ((0, 'M0r', 'M0c', 'M0v', 270), (1, 'M0r', 'M0c', 'M1v', 270),
                                  (2, 'M2r', 'M2c', 'M2v', 162)):
            r = np.zeros(270, INT); c = np.zeros(270, INT); v = np.zeros(270)
            el.update_M(r, c, v, prop, mtype=mt)
            assert (r[:n] == g[rk][t][:n]).all() and (c[:n] == g[ck][t][:n]).all(), mt
            if np.abs(g[vk][t]).max() > 0:
                assert blockwise_rel_err(v, g[vk][t], 270) < REL_TOL, mt
        f = np.zeros(18)
        el.update_fint(f, prop)
        assert rel(f, g['fint'][t]) < 1e-12
        assert rel(probe.finte, g['finte'][t]) < 1e-12


def test_quad4r_per_element_api_matches_reference(gpulib, golden):
    from pyfe3d_gb300 import INT, Quad4R, Quad4RProbe
    g = golden('quad4r_elements')
    props = _props(g)
    probe = Quad4RProbe()
    for t in range(len(g['x'])):
        el = Quad4R(probe)
        el.c1, el.c2, el.c3, el.c4 = (int(v) for v in g['c'][t])
        el.K6ROT = float(g['k6rot'][t])
        hg = [float(h) for h in g['hg'][t]]
        xmat = g['xmat'][t]
        if np.isnan(xmat).any():
            el.update_rotation_matrix(g['x'][t])
        else:
            el.update_rotation_matrix(g['x'][t], *xmat)
        R = [el.r11, el.r12, el.r13, el.r21, el.r22, el.r23, el.r31, el.r32, el.r33]
        assert rel(R, g['R'][t]) < 1e-14
        el.update_probe_xe(g['x'][t])
        el.update_probe_ue(g['u'][t])
        assert rel(probe.ue, g['ue'][t]) < 1e-14
        prop = props[g['pid'][t]]
        r = np.zeros(576, INT); c = np.zeros(576, INT); v = np.zeros(576)
        el.update_KC0(r, c, v, prop, 0, *hg)
        assert (r == g['KC0r'][t]).all() and (c == g['KC0c'][t]).all()
        assert blockwise_rel_err(v, g['KC0v'][t], 576) < REL_TOL
        r = np.zeros(144, INT); c = np.zeros(144, INT); v = np.zeros(144)
        el.update_KG(r, c, v, prop)
        assert (r == g['KGr'][t]).all() and (c == g['KGc'][t]).all()
        assert blockwise_rel_err(v, g['KGv'][t], 144) < REL_TOL
        r = np.full(144, -5, INT); c = np.full(144, -5, INT); v = np.zeros(144)
        el.update_KG(r, c, v, prop, update_KGv_only=1)
        assert (r == -5).all() and (c == -5).all()
        assert blockwise_rel_err(v, g['KGv'][t], 144) < REL_TOL
        r = np.zeros(144, INT); c = np.zeros(144, INT); v = np.zeros(144)
        el.update_KG_given_stress(*g['Nstress'][t], r, c, v)
        assert blockwise_rel_err(v, g['KGsv'][t], 144) < REL_TOL
        for mt in range(3):
            r = np.zeros(480, INT); c = np.zeros(480, INT); v = np.zeros(480)
            el.update_M(r, c, v, prop, mtype=mt)
            ref = g['M%dv' % mt][t]
            if np.abs(ref).max() > 0:
                assert blockwise_rel_err(v, ref, 480) < REL_TOL, mt
        f = np.zeros(24)
        el.update_fint(f, prop, *hg)
        assert rel(f, g['fint'][t]) < 1e-12
        assert rel(probe.finte, g['finte'][t]) < 1e-12


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
    return m, x.ravel()


def _tri_cdof(m):
    """Each quadrilateral (n1, n2, n3, n4) split into (n1, n2, n3), (n1, n3, n4)."""
    t = np.empty((2 * m.E, 3), np.int64)
    t[0::2] = m.cdof[:, [0, 1, 2]]
    t[1::2] = m.cdof[:, [0, 2, 3]]
    return t


def _mixed_props(E, rng):
    from pyfe3d_gb300.shellprop import isotropic_plate_records, shell_record
    from pyfe3d_gb300.shellprop_utils import laminated_plate
    h = rng.uniform(0.002, 0.2, E)
    props = isotropic_plate_records(h, 70e9, 0.3, rho=2700.)
    lam = shell_record(laminated_plate([0, 45, -45, 90, 30], plyt=0.0011,
                                       laminaprop=(142.5e9, 8.7e9, 0.28, 5.1e9, 5.1e9, 5.1e9),
                                       offset=0.001, rho=1600.))
    props[::3] = lam
    return props


@pytest.mark.parametrize('elem', ['tria3r', 'quad4r'])
@pytest.mark.parametrize('kind', ['flat', 'rotated', 'curved'])
@pytest.mark.parametrize('xmat', [False, True])
def test_batched_kc0_matches_oracle(gpulib, oracle, elem, kind, xmat):
    from pyfe3d_gb300 import batch
    m, x = _mesh(kind, seed=3)
    rng = np.random.default_rng(5)
    cdof = _tri_cdof(m) if elem == 'tria3r' else m.cdof
    E = len(cdof)
    size = 324 if elem == 'tria3r' else 576
    props = _mixed_props(E, rng)
    pid = rng.permutation(E).astype(np.int32)
    xm = rng.normal(size=(E, 3)) if xmat else None
    k6 = rng.choice([100., 1e4, 3.7], E)
    init_k = size * rng.permutation(E).astype(np.int64) + size
    n = size * (E + 2)
    if elem == 'tria3r':
        alpha = rng.uniform(0.1, 1.5, E)
        r0, c0, v0 = oracle.t3_kc0_batch(cdof, init_k, x, props, pid=pid, xmat=xm, k6rot=k6, alpha=alpha)
        r = np.zeros(n, np.int64); c = np.zeros(n, np.int64); v = np.full(n, 0.5)
        batch.tria3r_update_KC0(r, c, v, x, cdof, init_k, props, pid=pid, xmat=xm, k6rot=k6, alpha=alpha)
    else:
        hg = rng.uniform(0.2, 3.0, (E, 5))
        r0, c0, v0 = oracle.q4r_kc0_batch(cdof, init_k, x, props, pid=pid, xmat=xm, k6rot=k6, hg=hg)
        r = np.zeros(n, np.int64); c = np.zeros(n, np.int64); v = np.full(n, 0.5)
        batch.quad4r_update_KC0(r, c, v, x, cdof, init_k, props, pid=pid, xmat=xm, k6rot=k6, hg=hg)
    sl = slice(size, size * (E + 1))
    assert (r[sl] == r0[sl]).all() and (c[sl] == c0[sl]).all()
    assert blockwise_rel_err(v[sl] - 0.5, v0[sl], size) < REL_TOL
    assert (v[:size] == 0.5).all() and (v[-size:] == 0.5).all()


@pytest.mark.parametrize('elem', ['tria3r', 'quad4r'])
def test_batched_kc0_values_only_and_cuda_tensors(gpulib, oracle, elem):
    import torch
    from pyfe3d_gb300 import batch
    m, x = _mesh('curved', seed=1)
    cdof = _tri_cdof(m) if elem == 'tria3r' else m.cdof
    E = len(cdof)
    size = 324 if elem == 'tria3r' else 576
    props = _mixed_props(E, np.random.default_rng(2))
    init_k = size * np.arange(E, dtype=np.int64)
    fn = batch.tria3r_update_KC0 if elem == 'tria3r' else batch.quad4r_update_KC0
    ref = oracle.t3_kc0_batch if elem == 'tria3r' else oracle.q4r_kc0_batch
    r0, c0, v0 = ref(cdof, init_k, x, props)
    r = torch.full((size * E,), -1, dtype=torch.int64, device='cuda')
    c = torch.full_like(r, -1)
    v = torch.zeros(size * E, dtype=torch.float64, device='cuda')
    fn(r, c, v, x, cdof, init_k, props, update_KC0v_only=1)
    assert (r == -1).all() and (c == -1).all()
    assert blockwise_rel_err(v.cpu().numpy(), v0, size) < REL_TOL
    fn(r, c, v, x, cdof, init_k, props)
    assert (r.cpu().numpy() == r0).all() and (c.cpu().numpy() == c0).all()
    assert blockwise_rel_err(v.cpu().numpy(), 2 * v0, size) < REL_TOL


@pytest.mark.parametrize('kind', ['flat', 'curved'])
def test_tria3r_batched_kg_m_fint_match_oracle(gpulib, oracle, kind):
    from pyfe3d_gb300 import batch
    m, x = _mesh(kind, seed=4)
    cdof = _tri_cdof(m)
    E = len(cdof)
    rng = np.random.default_rng(6)
    props = _mixed_props(E, rng)
    u = rng.normal(size=m.N) * 1e-3
    xm = rng.normal(size=(E, 3))
    # reference per element (oracle), then the batched device path
    Rs, ms, xes, areas, ues = [], [], [], [], []
    for e in range(E):
        R, mm = oracle.t3_rotation(x, cdof[e], xm[e])
        xe, ar = oracle.t3_probe_xe(x, cdof[e], R)
        Rs.append(R); ms.append(mm); xes.append(xe); areas.append(ar)
        ues.append(oracle.t3_probe_ue(u, cdof[e], R))
    init_k = 81 * np.arange(E, dtype=np.int64)
    r0, c0, v0 = np.zeros(81 * E, np.int64), np.zeros(81 * E, np.int64), np.zeros(81 * E)
    for e in range(E):
        oracle.t3_kg(Rs[e], ms[e], xes[e], areas[e], ues[e], props[e], cdof[e], 81 * e, r0, c0, v0)
    r = np.zeros(81 * E, np.int64); c = np.zeros(81 * E, np.int64); v = np.zeros(81 * E)
    batch.tria3r_update_KG(r, c, v, x, u, cdof, init_k, props, xmat=xm)
    assert (r == r0).all() and (c == c0).all()
    assert blockwise_rel_err(v, v0, 81) < REL_TOL
    ns = rng.normal(size=(E, 3)) * 1e3
    r0, c0, v0 = np.zeros(81 * E, np.int64), np.zeros(81 * E, np.int64), np.zeros(81 * E)
    for e in range(E):
        oracle.t3_kg_given_stress(Rs[e], xes[e], areas[e], ns[e], cdof[e], 81 * e, r0, c0, v0)
    r = np.zeros(81 * E, np.int64); c = np.zeros(81 * E, np.int64); v = np.zeros(81 * E)
    batch.tria3r_update_KG_given_stress(r, c, v, x, cdof, init_k, ns)
    assert (r == r0).all() and (c == c0).all()
    assert blockwise_rel_err(v, v0, 81) < REL_TOL
    for mt, size in ((0, 270), (1, 270), (2, 162)):
        ik = size * np.arange(E, dtype=np.int64)
        r0, c0, v0 = np.zeros(size * E, np.int64), np.zeros(size * E, np.int64), np.zeros(size * E)
        for e in range(E):
            oracle.t3_m(Rs[e], areas[e], props[e], cdof[e], size * e, r0, c0, v0, mt)
        r = np.zeros(size * E, np.int64); c = np.zeros(size * E, np.int64); v = np.zeros(size * E)
        batch.tria3r_update_M(r, c, v, x, cdof, ik, props, mtype=mt)
        assert (r == r0).all() and (c == c0).all()
        assert blockwise_rel_err(v, v0, size) < REL_TOL
    f0 = np.zeros(m.N)
    for e in range(E):
        oracle.t3_fint(Rs[e], ms[e], xes[e], areas[e], props[e], cdof[e], ues[e], f0)
    f = np.zeros(m.N)
    finte = batch.tria3r_update_fint(f, x, u, cdof, props, xmat=xm).cpu().numpy()
    assert rel(f, f0) < 1e-12
    fe0 = oracle.t3_finte(ms[7], xes[7], areas[7], props[7], ues[7])
    assert rel(finte[7], fe0) < 1e-12


def test_quad4r_batched_fint_matches_oracle(gpulib, oracle):
    from pyfe3d_gb300 import batch
    m, x = _mesh('curved', seed=8)
    E = m.E
    rng = np.random.default_rng(9)
    props = _mixed_props(E, rng)
    u = rng.normal(size=m.N) * 1e-3
    hg = rng.uniform(0.2, 3.0, 5)
    f0 = np.zeros(m.N)
    for e in range(E):
        R, mm = oracle.q4_rotation(x, m.cdof[e])
        xe, ar = oracle.q4_probe_xe(x, m.cdof[e], R)
        ue = oracle.q4_probe_ue(u, m.cdof[e], R)
        oracle.q4r_fint(R, mm, xe, ar, props[e], m.cdof[e], ue, f0, 100., hg)
    f = np.zeros(m.N)
    batch.quad4r_update_fint(f, x, u, m.cdof, props, hg=hg)
    assert rel(f, f0) < 1e-12


def test_tria3r_reference_plate(gpulib, golden):
    """The reference's Tria3R point-load plate (tests/test_tria3r_static_point_load.py):
    GPU KC0, GPU assembly and the GPU solver reproduce the reference's
    spsolve solution; the internal forces balance the external ones."""
    import torch
    from pyfe3d_gb300 import batch
    from pyfe3d_gb300.solver import CSRPattern, Solver
    g = golden('tria3r_static')
    cdof = 6 * g['conn']
    E = len(cdof)
    N = len(g['f'])
    Kr = torch.zeros(324 * E, dtype=torch.int64, device='cuda')
    Kc = torch.zeros_like(Kr)
    Kv = torch.zeros(324 * E, dtype=torch.float64, device='cuda')
    batch.tria3r_update_KC0(Kr, Kc, Kv, g['x'], cdof, 324 * np.arange(E), g['prop'])
    pat = CSRPattern(Kr, Kc, N, g['bk'])
    vals = pat.assemble(Kv)
    u_free, st = Solver(pat).setup(vals).solve(pat.reduce(g['f']), tol=1e-12)
    assert st['status'] == 'converged'
    u = pat.expand(u_free).cpu().numpy()
    assert np.abs(u - g['u']).max() <= 1e-7 * np.abs(g['u']).max()
    w = u[2::6]
    assert np.isclose(w.max(), 8.324614783831663e-05, rtol=0.02)


def test_reduced_shell_argument_errors(gpulib):
    from pyfe3d_gb300 import _lib
    lib = _lib.load()
    sp = _lib.stream_ptr()
    for fn in (lib.fe3d_tria3r_kc0, lib.fe3d_quad4r_kc0):
        assert fn(0, None, None, None, 0, None, 0, None, None, None, None, None, 0, None, None, 0, None, 0,
                  None, None, None, 0, 0, None, sp) == 0
        assert fn(-1, None, None, None, 0, None, 0, None, None, None, None, None, 0, None, None, 0, None, 0,
                  None, None, None, 0, 0, None, sp) == -1
        assert fn(4, None, None, None, 0, None, 0, None, None, None, None, None, 0, None, None, 0, None, 0,
                  None, None, None, 0, 0, None, sp) == -1
    assert lib.fe3d_tria3r_m(1, None, None, None, 0, None, None, None, 0, None, None, None, None, 0, 5, None,
                             sp) == -1


@pytest.mark.parametrize('mtype', [0, 1, 2])
def test_tria3r_natural_frequencies(gpulib, mtype):
    """The reference's Tria3R modal case (tests/test_tria3r_natural_freq.py: 9x11
    nodes, 0.3 x 0.5 m steel plate 10 mm thick, simply supported): GPU KC0 and M,
    device LOBPCG; against eigsh on the same matrices and the Kirchhoff plate's
    fundamental frequency pi^2 (1/a^2 + 1/b^2) sqrt(D / (rho h)) within 5 %."""
    import torch
    from scipy.sparse.linalg import eigsh
    from pyfe3d_gb300 import batch, eigen
    from pyfe3d_gb300.meshes import PlateMesh
    from pyfe3d_gb300.shellprop import isotropic_plate_records
    from pyfe3d_gb300.solver import CSRPattern
    a, b, h, E, nu, rho = 0.3, 0.5, 0.01, 203e9, 0.33, 7.83e3
    m = PlateMesh(9, 11, a, b)
    cdof = _tri_cdof(m)
    Et = len(cdof)
    props = isotropic_plate_records(h, E, nu, rho=rho)
    bk = m.bc_mask((0, 1, 2))
    dev = torch.device('cuda')

    def reduced(size, fill):
        Kr = torch.zeros(size * Et, dtype=torch.int64, device=dev)
        Kc = torch.zeros_like(Kr)
        Kv = torch.zeros(size * Et, dtype=torch.float64, device=dev)
        fill(Kr, Kc, Kv, size * np.arange(Et, dtype=np.int64))
        pat = CSRPattern(Kr, Kc, m.N, bk)
        return pat, pat.assemble(Kv)

    pk, vk = reduced(324, lambda r, c, v, ik: batch.tria3r_update_KC0(r, c, v, m.x, cdof, ik, props))
    pm, vm = reduced(270, lambda r, c, v, ik: batch.tria3r_update_M(r, c, v, m.x, cdof, ik, props, mtype=mtype))
    omega, X, info = eigen.natural_frequencies(eigen.CSROperator(pk, vk), eigen.CSROperator(pm, vm), 3, tol=1e-8)
    assert info['converged'], info
    ev = np.sort(eigsh(pk.to_scipy(vk).tocsc(), k=3, M=pm.to_scipy(vm).tocsc(), sigma=-1., which='LM')[0])
    assert np.allclose(omega ** 2, ev, rtol=1e-7), (omega ** 2, ev)
    D = E * h ** 3 / (12 * (1 - nu ** 2))
    w11 = np.pi ** 2 * (1 / a ** 2 + 1 / b ** 2) * np.sqrt(D / (rho * h))
    assert np.isclose(omega[0], w11, rtol=0.05), (omega[0], w11)


def test_quad4r_static_plate_matches_oracle(gpulib, oracle):
    """Quad4R point-loaded simply supported plate: GPU KC0 + assembly + PCG
    against the oracle's triplets assembled by scipy and solved with spsolve."""
    import scipy.sparse as sp
    from scipy.sparse.linalg import spsolve
    from pyfe3d_gb300 import batch
    from pyfe3d_gb300.meshes import PlateMesh
    from pyfe3d_gb300.shellprop import isotropic_plate_records
    from pyfe3d_gb300.solver import static_solve_coo
    m = PlateMesh(21, 17, 1.0, 0.8, perturb=0.15, seed=11)
    props = isotropic_plate_records(0.005, 70e9, 0.33)
    ik = 576 * np.arange(m.E, dtype=np.int64)
    r = np.zeros(576 * m.E, np.int64); c = np.zeros(576 * m.E, np.int64); v = np.zeros(576 * m.E)
    batch.quad4r_update_KC0(r, c, v, m.x, m.cdof, ik, props)
    bk = m.bc_mask((0, 1, 2))
    f = np.zeros(m.N)
    f[6 * m.nids[10, 8] + 2] = -1000.
    u = static_solve_coo(r, c, v, m.N, bk, f, tol=1e-11)
    r0, c0, v0 = oracle.q4r_kc0_batch(m.cdof, ik, m.x, props)
    K = sp.coo_matrix((v0, (r0, c0)), shape=(m.N, m.N)).tocsc()
    bu = ~bk
    u0 = np.zeros(m.N)
    u0[bu] = spsolve(K[bu, :][:, bu], f[bu])
    assert np.linalg.norm(u - u0) <= 1e-7 * np.linalg.norm(u0)


def test_tria3r_buckling_given_stress(gpulib):
    """The reference's Tria3R plate buckling under a given Nxx
    (tests/test_tria3r_linear_buckling_plate_given_stress.py: 31x15 nodes,
    2.0 x 0.5 m, h 2 mm, w simply supported, in-plane rigid-body modes and
    drilling removed): GPU KC0 and KG of given stress, device LOBPCG; the
    load multiplier against a dense generalised eigh of the same matrices and
    the critical load against the classical plate formula within 5 %."""
    import scipy.linalg
    import torch
    from pyfe3d_gb300 import batch, eigen
    from pyfe3d_gb300.meshes import PlateMesh
    from pyfe3d_gb300.shellprop import isotropic_plate_records
    from pyfe3d_gb300.solver import CSRPattern
    a, b, h, E, nu = 2.0, 0.5, 0.002, 203e9, 0.33
    m = PlateMesh(31, 15, a, b)
    cdof = _tri_cdof(m)
    Et = len(cdof)
    props = isotropic_plate_records(h, E, nu, rho=7.83e3)
    X, Y = m.ncoords[:, 0], m.ncoords[:, 1]
    bk = np.zeros(m.N, bool)
    bk[2::6] = m.edge
    bk[0::6] = np.isclose(X, a / 2) & (np.isclose(Y, 0.) | np.isclose(Y, b))
    bk[1::6] = np.isclose(Y, b / 2) & (np.isclose(X, 0.) | np.isclose(X, a))
    bk[5::6] = True
    dev = torch.device('cuda')

    def reduced(size, fill):
        Kr = torch.zeros(size * Et, dtype=torch.int64, device=dev)
        Kc = torch.zeros_like(Kr)
        Kv = torch.zeros(size * Et, dtype=torch.float64, device=dev)
        fill(Kr, Kc, Kv, size * np.arange(Et, dtype=np.int64))
        pat = CSRPattern(Kr, Kc, m.N, bk)
        return pat, pat.assemble(Kv)

    Nxx = -1.
    pk, vk = reduced(324, lambda r, c, v, ik: batch.tria3r_update_KC0(r, c, v, m.x, cdof, ik, props))
    pg, vg = reduced(81, lambda r, c, v, ik: batch.tria3r_update_KG_given_stress(r, c, v, m.x, cdof, ik,
                                                                                  [Nxx, 0., 0.]))
    lam, X_, info = eigen.buckling(eigen.CSROperator(pk, vk), eigen.CSROperator(pg, vg), 1, tol=1e-6)
    assert info['converged'], info
    mu = scipy.linalg.eigh(pg.to_scipy(vg).toarray(), pk.to_scipy(vk).toarray(), eigvals_only=True)
    ref = -1. / mu[0]
    assert np.isclose(lam[0], ref, rtol=1e-6), (lam, ref)
    kc = min((k * b / a + a / (k * b)) ** 2 for k in range(1, 21))
    P_theory = -kc * np.pi ** 2 * E / (12 * (1 - nu ** 2)) * h ** 2 / b ** 2 * h * b
    assert np.isclose(lam[0] * Nxx * b, P_theory, rtol=0.05), (lam[0] * Nxx * b, P_theory)
