"""The CPU oracle against the frozen outputs of the reference (no GPU)."""
import numpy as np

from conftest import REL_TOL, blockwise_rel_err


def rel(a, b):
    return np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(b).max(), 1e-300)


def test_quad4_frames_and_probes(oracle, golden):
    g = golden('quad4_elements')
    for t in range(len(g['x'])):
        xmat = g['xmat'][t]
        R, m = oracle.q4_rotation(g['x'][t], g['c'][t], None if np.isnan(xmat).any() else xmat)
        assert rel(R, g['R'][t]) < 1e-14
        assert rel(m, g['m'][t]) < 1e-14
        xe, area = oracle.q4_probe_xe(g['x'][t], g['c'][t], g['R'][t])
        assert rel(xe, g['xe'][t]) < 1e-14
        assert abs(area - g['area'][t]) <= 1e-14 * g['area'][t]
        ue = oracle.q4_probe_ue(g['u'][t], g['c'][t], g['R'][t])
        assert rel(ue, g['ue'][t]) < 1e-14


def test_quad4_matrices(oracle, golden):
    g = golden('quad4_elements')
    props = g['props']
    for t in range(len(g['x'])):
        P = props[g['pid'][t]]
        args = (g['R'][t], g['m'][t], g['xe'][t], float(g['area'][t]), P, g['c'][t], 0)
        r, c, v = np.zeros(576, np.int64), np.zeros(576, np.int64), np.zeros(576)
        oracle.q4_kc0(*args, r, c, v)
        assert (r == g['KC0r'][t]).all() and (c == g['KC0c'][t]).all()
        assert blockwise_rel_err(v, g['KC0v'][t], 576) < REL_TOL
        r, c, v = np.zeros(144, np.int64), np.zeros(144, np.int64), np.zeros(144)
        oracle.q4_kg(g['R'][t], g['m'][t], g['xe'][t], g['ue'][t], P, g['c'][t], 0, r, c, v)
        assert (r == g['KGr'][t]).all() and (c == g['KGc'][t]).all()
        assert blockwise_rel_err(v, g['KGv'][t], 144) < REL_TOL
        for mt, rk, ck, vk in ((0, 'M0r', 'M0c', 'M0v'), (1, 'M0r', 'M0c', 'M1v'),
                               (2, 'M2r', 'M2c', 'M2v')):
            r, c, v = np.zeros(480, np.int64), np.zeros(480, np.int64), np.zeros(480)
            oracle.q4_m(g['R'][t], g['xe'][t], float(g['area'][t]), P, g['c'][t], 0, r, c, v, mt)
            assert (r == g[rk][t]).all() and (c == g[ck][t]).all()
            assert blockwise_rel_err(v, g[vk][t], 480) < REL_TOL
        f = np.zeros(24)
        oracle.q4_fint(g['R'][t], g['m'][t], g['xe'][t], float(g['area'][t]), P, g['c'][t],
                       g['ue'][t], f)
        assert rel(f, g['fint'][t]) < 1e-12
        fe = oracle.q4_finte(g['m'][t], g['xe'][t], float(g['area'][t]), P, g['ue'][t])
        assert rel(fe, g['finte'][t]) < 1e-12
        r, c, v = np.zeros(144, np.int64), np.zeros(144, np.int64), np.zeros(144)
        oracle.q4_kg_given_stress(g['R'][t], g['xe'][t], g['Nstress'][t], g['c'][t], 0, r, c, v)
        assert (r == g['KGsr'][t]).all() and (c == g['KGsc'][t]).all()
        assert blockwise_rel_err(v, g['KGsv'][t], 144) < REL_TOL


def test_beamc(oracle, golden):
    g = golden('beamc_elements')
    for t in range(len(g['x'])):
        R = oracle.bc_rotation(g['x'][t], g['c'][t], g['vxy'][t])
        assert rel(R, g['R'][t]) < 1e-14
        xe, L = oracle.bc_probe_xe(g['x'][t], g['c'][t], g['R'][t])
        assert abs(L - g['length'][t]) <= 1e-14 * g['length'][t]
        ue = oracle.bc_probe_ue(g['u'][t], g['c'][t], g['R'][t])
        assert rel(ue, g['ue'][t]) < 1e-14
        P = g['prop'][t]
        L = float(g['length'][t])
        r, c, v = np.zeros(144, np.int64), np.zeros(144, np.int64), np.zeros(144)
        oracle.bc_kc0(g['R'][t], L, P, g['c'][t], 0, r, c, v)
        assert (r == g['KC0r'][t]).all() and (c == g['KC0c'][t]).all()
        assert blockwise_rel_err(v, g['KC0v'][t], 144) < REL_TOL
        r, c, v = np.zeros(144, np.int64), np.zeros(144, np.int64), np.zeros(144)
        oracle.bc_kg(g['R'][t], L, P, g['ue'][t], g['c'][t], 0, r, c, v)
        assert (r == g['KGr'][t]).all() and (c == g['KGc'][t]).all()
        assert blockwise_rel_err(v, g['KGv'][t], 144) < REL_TOL
        for mt, n in ((0, 144), (1, 36)):
            r, c, v = np.zeros(144, np.int64), np.zeros(144, np.int64), np.zeros(144)
            oracle.bc_m(g['R'][t], L, P, g['c'][t], 0, r, c, v, mt)
            assert (r == g['M%dr' % mt][t]).all() and (c == g['M%dc' % mt][t]).all()
            assert blockwise_rel_err(v[:n], g['M%dv' % mt][t][:n], n) < REL_TOL
        fint = np.zeros(12)
        fe = oracle.bc_fint(g['R'][t], L, P, g['c'][t], g['ue'][t], fint)
        assert rel(fe, g['finte'][t]) < 1e-12
        assert rel(fint, g['fint'][t]) < 1e-12


def test_beamc_batch_wrappers_reproduce_reference(oracle, golden):
    """The oracle's BeamC KG and M batch loops (frame, length and ue gathered
    per element from global arrays) give the reference's per-element outputs
    when the 32 frozen elements are laid out as one mesh of 64 nodes, and the
    per-element loop equals the C batch routine for KC0."""
    g = golden('beamc_elements')
    E = len(g['x'])
    # element t keeps its frozen node pair as nodes 2t, 2t+1 (DOF offsets + 12t)
    x = np.concatenate(list(g['x']))
    u = np.concatenate(list(g['u']))
    cdof = g['c'] + 12 * np.arange(E)[:, None]
    init_k = 144 * np.arange(E)
    r, c, v = oracle.bc_kg_batch(cdof, init_k, x, u, g['vxy'], g['prop'], pid=np.arange(E))
    assert blockwise_rel_err(v, g['KGv'], 144) < REL_TOL
    assert (r.reshape(E, 144) == g['KGr'] + 12 * np.arange(E)[:, None]).all()
    assert (c.reshape(E, 144) == g['KGc'] + 12 * np.arange(E)[:, None]).all()
    for mt, n in ((0, 144), (1, 36)):
        _, _, v = oracle.bc_m_batch(cdof, init_k, x, g['vxy'], g['prop'], pid=np.arange(E), mtype=mt)
        assert blockwise_rel_err(v.reshape(E, 144)[:, :n], g['M%dv' % mt][:, :n], n) < REL_TOL
    r0, c0, v0 = oracle.bc_kc0_batch(cdof, init_k, x, g['vxy'], g['prop'], pid=np.arange(E))
    Kr, Kc, Kv = np.zeros_like(r0), np.zeros_like(c0), np.zeros_like(v0)
    for e, ce, R, L, P in oracle._bc_elements(cdof, x, g['vxy'], g['prop'], np.arange(E)):
        oracle.bc_kc0(R, L, P, ce, int(init_k[e]), Kr, Kc, Kv)
    assert (Kr == r0).all() and (Kc == c0).all() and (Kv == v0).all()


def test_beamc_block_structure_used_by_the_kernel(oracle, golden):
    """The BeamC matrix kernel turns six of the ten upper 3x3 blocks of KC0
    and KG and derives the other four (T1T2 = -T1T1, T2T2 = T1T1,
    R1T2 = -(T1R1)^T, T2R2 = -T1R2), and leaves the exact zeros of the axial
    row of T1T1 and the first entry of T1R1 / T1R2 out of its products.  Both
    hold exactly in the local matrices (identity frame) and to rounding in
    the reference's own global outputs."""
    g = golden('beamc_elements')
    eye = np.eye(3).ravel()

    def blk(K, i, j):
        return K[3 * i:3 * i + 3, 3 * j:3 * j + 3]

    for t in range(len(g['x'])):
        P = g['prop'][t]
        L = float(g['length'][t])
        for kind in ('kc0', 'kg'):
            r, c, v = np.zeros(144, np.int64), np.zeros(144, np.int64), np.zeros(144)
            if kind == 'kc0':
                oracle.bc_kc0(eye, L, P, g['c'][t], 0, r, c, v)
            else:
                oracle.bc_kg(eye, L, P, g['ue'][t], g['c'][t], 0, r, c, v)
            K = v.reshape(12, 12)
            assert np.array_equal(blk(K, 0, 2), -blk(K, 0, 0)) and np.array_equal(blk(K, 2, 2), blk(K, 0, 0))
            assert np.array_equal(blk(K, 1, 2), -blk(K, 0, 1).T)
            assert np.array_equal(blk(K, 2, 3), -blk(K, 0, 3))
            assert K[0, 1] == 0. and K[0, 2] == 0. and K[0, 3] == 0. and K[0, 9] == 0.
        for key in ('KC0v', 'KGv'):
            K = np.asarray(g[key][t]).reshape(12, 12)
            tol = 1e-14 * np.abs(K).max()
            assert np.abs(blk(K, 0, 2) + blk(K, 0, 0)).max() <= tol
            assert np.abs(blk(K, 2, 2) - blk(K, 0, 0)).max() <= tol
            assert np.abs(blk(K, 1, 2) + blk(K, 0, 1).T).max() <= tol
            assert np.abs(blk(K, 2, 3) + blk(K, 0, 3)).max() <= tol


def test_quad4_kg_of_flat_elements_is_w_w_only(oracle):
    """The Quad4 KG kernel forms, adds and writes only the 16 (w, w) values
    of an element flat in the global x-y plane: every other of its 144 KG
    entries is an exact zero (r13 = r23 = 0 in r_m3 r_n3)."""
    from pyfe3d_gb300.meshes import config2
    from pyfe3d_gb300.shellprop import isotropic_plate_records
    m, props, pid, bk, f = config2(9)
    rng = np.random.default_rng(4)
    props = isotropic_plate_records(rng.uniform(0.002, 0.02, m.E), 70e9, 0.3, rho=2700.)
    props[:, 6:12] = rng.normal(size=(m.E, 6)) * 1e3
    u = rng.normal(size=m.N) * 1e-3
    r, c, v = oracle.q4_kg_batch(m.cdof, m.init_k(144), m.x, u, props)
    K = v.reshape(m.E, 12, 12)
    ww = np.zeros((12, 12), bool)
    ww[2::3, 2::3] = True
    assert (K[:, ~ww] == 0.).all()
    assert (np.abs(K[:, ww]) > 0.).mean() > 0.9


def test_beamc_kg_flag_semantics(golden):
    # update_KGv_only=1 leaves the index arrays untouched (beamc.pyx:1451)
    g = golden('beamc_elements')
    assert (g['KGv_only_r'] == 0).all()


def test_plate_static_oracle(oracle, golden):
    """Full 21x21 plate: oracle triplets reproduce the reference's solution."""
    from scipy.sparse import coo_matrix
    from scipy.sparse.linalg import spsolve
    g = golden('plate_static')
    cdof = 6 * g['conn']
    E = cdof.shape[0]
    init_k = 576 * np.arange(E)
    r, c, v = oracle.q4_kc0_batch(cdof, init_k, g['x'], g['prop'][None, :])
    assert (r[:8 * 576] == g['KC0r_first']).all() and (c[:8 * 576] == g['KC0c_first']).all()
    assert blockwise_rel_err(v[:8 * 576], g['KC0v_first'], 576) < REL_TOL
    N = len(g['u'])
    K = coo_matrix((v, (r, c)), shape=(N, N)).tocsc()
    assert K.nnz == int(g['nnz'])
    bu = ~g['bk']
    u = np.zeros(N)
    u[bu] = spsolve(K[bu, :][:, bu], g['f'][bu])
    assert np.abs(u - g['u']).max() <= 1e-10 * np.abs(g['u']).max()


def test_tria3r_oracle(oracle, golden):
    """Tria3R restatement against the reference (tria3r.pyx): frames, probes,
    KC0 (with the reference's rz transformation), finte/fint, KG, KG of
    given stress and the three mass matrices."""
    g = golden('tria3r_elements')
    props = g['props']
    for t in range(len(g['x'])):
        xmat = g['xmat'][t]
        R, m = oracle.t3_rotation(g['x'][t], g['c'][t], None if np.isnan(xmat).any() else xmat)
        assert rel(R, g['R'][t]) < 1e-14 and rel(m, g['m'][t]) < 1e-14
        xe, area = oracle.t3_probe_xe(g['x'][t], g['c'][t], g['R'][t])
        assert rel(xe, g['xe'][t]) < 1e-14
        assert abs(area - g['area'][t]) <= 1e-14 * g['area'][t]
        assert rel(oracle.t3_probe_ue(g['u'][t], g['c'][t], g['R'][t]), g['ue'][t]) < 1e-14
        P = props[g['pid'][t]]
        k6, al = float(g['k6rot'][t]), float(g['alpha'][t])
        R, m, xe, area, c = g['R'][t], g['m'][t], g['xe'][t], float(g['area'][t]), g['c'][t]
        r, cc, v = np.zeros(324, np.int64), np.zeros(324, np.int64), np.zeros(324)
        oracle.t3_kc0(R, m, xe, area, P, c, 0, r, cc, v, k6, al)
        assert (r == g['KC0r'][t]).all() and (cc == g['KC0c'][t]).all()
        assert blockwise_rel_err(v, g['KC0v'][t], 324) < REL_TOL
        fe = oracle.t3_finte(m, xe, area, P, g['ue'][t], k6, al)
        assert rel(fe, g['finte'][t]) < 1e-12
        f = np.zeros(18)
        oracle.t3_fint(R, m, xe, area, P, c, g['ue'][t], f, k6, al)
        assert rel(f, g['fint'][t]) < 1e-12
        r, cc, v = np.zeros(81, np.int64), np.zeros(81, np.int64), np.zeros(81)
        oracle.t3_kg(R, m, xe, area, g['ue'][t], P, c, 0, r, cc, v)
        assert (r == g['KGr'][t]).all() and (cc == g['KGc'][t]).all()
        assert blockwise_rel_err(v, g['KGv'][t], 81) < REL_TOL
        r, cc, v = np.zeros(81, np.int64), np.zeros(81, np.int64), np.zeros(81)
        oracle.t3_kg_given_stress(R, xe, area, g['Nstress'][t], c, 0, r, cc, v)
        assert (r == g['KGsr'][t]).all() and (cc == g['KGsc'][t]).all()
        assert blockwise_rel_err(v, g['KGsv'][t], 81) < REL_TOL
        for mt, rk, ck, vk, n in ((0, 'M0r', 'M0c', 'M0v', 270), (1, 'M0r', 'M0c', 'M1v', 270),
                                  (2, 'M2r', 'M2c', 'M2v', 162)):
            r, cc, v = np.zeros(270, np.int64), np.zeros(270, np.int64), np.zeros(270)
            oracle.t3_m(R, area, P, c, 0, r, cc, v, mt)
            assert (r[:n] == g[rk][t][:n]).all() and (cc[:n] == g[ck][t][:n]).all()
            if np.abs(g[vk][t]).max() > 0:
                assert blockwise_rel_err(v, g[vk][t], 270) < REL_TOL


def test_tria3r_kc0_drops_rz_couplings(oracle, golden):
    """The reference's global KC0 keeps only the rz_a - rz_a drilling terms
    while finte uses the whole local matrix: the restatement reproduces
    both, so KC0 u != R finte for a drilling-only displacement."""
    g = golden('tria3r_elements')
    t = 2
    P = g['props'][g['pid'][t]]
    Ke = oracle.t3_kc0_local(g['m'][t], g['xe'][t], float(g['area'][t]), P, float(g['k6rot'][t]),
                             float(g['alpha'][t]))
    assert np.abs(Ke[0, 5]) > 0  # the local matrix couples u and rz
    rz = np.zeros(18)
    rz[5] = 1.
    r, c, v = np.zeros(324, np.int64), np.zeros(324, np.int64), np.zeros(324)
    oracle.t3_kc0(np.eye(3).ravel(), g['m'][t], g['xe'][t], float(g['area'][t]), P, np.array([0, 6, 12]), 0,
                  r, c, v, float(g['k6rot'][t]), float(g['alpha'][t]))
    K = v.reshape(18, 18)
    assert K[0, 5] == 0. and K[5, 11] == 0. and K[5, 5] == Ke[5, 5]


def test_quad4r_oracle(oracle, golden):
    """Quad4R restatement against the reference (quad4r.pyx): KC0 with
    hourglass factors and K6ROT, finte/fint; KG, KG of given stress and mass
    are the Quad4 ones."""
    g = golden('quad4r_elements')
    props = g['props']
    for t in range(len(g['x'])):
        xmat = g['xmat'][t]
        R, m = oracle.q4_rotation(g['x'][t], g['c'][t], None if np.isnan(xmat).any() else xmat)
        assert rel(R, g['R'][t]) < 1e-14 and rel(m, g['m'][t]) < 1e-14
        P = props[g['pid'][t]]
        k6, hg = float(g['k6rot'][t]), g['hg'][t]
        R, m, xe, area, c = g['R'][t], g['m'][t], g['xe'][t], float(g['area'][t]), g['c'][t]
        r, cc, v = np.zeros(576, np.int64), np.zeros(576, np.int64), np.zeros(576)
        oracle.q4r_kc0(R, m, xe, area, P, c, 0, r, cc, v, k6, hg)
        assert (r == g['KC0r'][t]).all() and (cc == g['KC0c'][t]).all()
        assert blockwise_rel_err(v, g['KC0v'][t], 576) < REL_TOL
        fe = oracle.q4r_finte(m, xe, area, P, g['ue'][t], k6, hg)
        assert rel(fe, g['finte'][t]) < 1e-12
        f = np.zeros(24)
        oracle.q4r_fint(R, m, xe, area, P, c, g['ue'][t], f, k6, hg)
        assert rel(f, g['fint'][t]) < 1e-12
        r, cc, v = np.zeros(144, np.int64), np.zeros(144, np.int64), np.zeros(144)
        oracle.q4_kg(R, m, xe, g['ue'][t], P, c, 0, r, cc, v)
        assert (r == g['KGr'][t]).all() and (cc == g['KGc'][t]).all()
        assert blockwise_rel_err(v, g['KGv'][t], 144) < REL_TOL
        r, cc, v = np.zeros(144, np.int64), np.zeros(144, np.int64), np.zeros(144)
        oracle.q4_kg_given_stress(R, xe, g['Nstress'][t], c, 0, r, cc, v)
        assert blockwise_rel_err(v, g['KGsv'][t], 144) < REL_TOL
        for mt in range(3):
            r, cc, v = np.zeros(480, np.int64), np.zeros(480, np.int64), np.zeros(480)
            oracle.q4_m(R, xe, area, P, c, 0, r, cc, v, mt)
            ref = g['M%dv' % mt][t]
            if np.abs(ref).max() > 0:
                assert blockwise_rel_err(v, ref, 480) < REL_TOL


def test_tria3r_static_oracle(oracle, golden):
    """The reference's 7x11-node Tria3R plate: the oracle's KC0 assembled
    with scipy reproduces the reference solution."""
    import scipy.sparse as sp
    from scipy.sparse.linalg import spsolve
    g = golden('tria3r_static')
    conn = g['conn']
    cdof = 6 * conn
    E = len(conn)
    N = len(g['f'])
    r, c, v = oracle.t3_kc0_batch(cdof, 324 * np.arange(E), g['x'], g['prop'])
    K = sp.coo_matrix((v, (r, c)), shape=(N, N)).tocsc()
    assert np.allclose(K.diagonal(), g['Kdiag'], rtol=1e-12, atol=0)
    bu = ~g['bk']
    u = np.zeros(N)
    u[bu] = spsolve(K[bu, :][:, bu], g['f'][bu])
    assert np.abs(u - g['u']).max() <= 1e-10 * np.abs(g['u']).max()
