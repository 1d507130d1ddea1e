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
