"""BeamC CUDA kernels against the reference's frozen outputs and the oracle."""
import numpy as np
import pytest

from conftest import REL_TOL, blockwise_rel_err

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(b).max(), 1e-300)


def _prop(rec):
    from pyfe3d_gb300.shellprop import BeamProp, BEAM_FIELDS
    p = BeamProp()
    for i, f in enumerate(BEAM_FIELDS):
        setattr(p, f, float(rec[i]))
    return p


def test_per_element_api_matches_reference(gpulib, golden):
    from pyfe3d_gb300 import BeamC, BeamCProbe, INT
    g = golden('beamc_elements')
    probe = BeamCProbe()
    for t in range(len(g['x'])):
        b = BeamC(probe)
        b.c1, b.c2 = (int(v) for v in g['c'][t])
        b.update_rotation_matrix(*g['vxy'][t], g['x'][t])
        R = [b.r11, b.r12, b.r13, b.r21, b.r22, b.r23, b.r31, b.r32, b.r33]
        assert rel(R, g['R'][t]) < 1e-14
        b.update_probe_xe(g['x'][t])
        assert rel(probe.xe, g['xe'][t]) < 1e-14
        assert abs(b.length - g['length'][t]) <= 1e-14 * g['length'][t]
        b.update_probe_ue(g['u'][t])
        assert rel(probe.ue, g['ue'][t]) < 1e-14
        prop = _prop(g['prop'][t])
        r = np.zeros(144, INT); c = np.zeros(144, INT); v = np.zeros(144)
        b.update_KC0(r, c, v, prop)
        assert (r == g['KC0r'][t]).all() and (c == g['KC0c'][t]).all()
        assert blockwise_rel_err(v, g['KC0v'][t], 144) < REL_TOL
        r = np.zeros(144, INT); c = np.zeros(144, INT); v = np.zeros(144)
        b.update_KG(r, c, v, prop)
        assert (r == g['KGr'][t]).all() and (c == g['KGc'][t]).all()
        assert blockwise_rel_err(v, g['KGv'][t], 144) < REL_TOL
        r = np.zeros(144, INT); c = np.zeros(144, INT); v = np.zeros(144)
        b.update_KG(r, c, v, prop, update_KGv_only=1)
        assert (r == 0).all() and (c == 0).all()
        for mt, n in ((0, 144), (1, 36)):
            r = np.zeros(144, INT); c = np.zeros(144, INT); v = np.zeros(144)
            b.update_M(r, c, v, prop, mtype=mt)
            assert (r == g['M%dr' % mt][t]).all() and (c == g['M%dc' % mt][t]).all()
            assert blockwise_rel_err(v[:n], g['M%dv' % mt][t][:n], n) < REL_TOL


def test_batched_beams_match_oracle(gpulib, oracle, golden):
    from pyfe3d_gb300 import batch
    g = golden('beamc_elements')
    rng = np.random.default_rng(2)
    nn = 40
    x = rng.normal(size=3 * nn)
    E = 60
    conn = np.stack([rng.integers(0, nn, E), rng.integers(0, nn, E)], 1)
    conn[conn[:, 0] == conn[:, 1], 1] = (conn[conn[:, 0] == conn[:, 1], 0] + 1) % nn
    cdof = 6 * conn
    vxy = rng.normal(size=(E, 3))
    props = g['prop']
    pid = rng.integers(0, len(props), E).astype(np.int32)
    init_k = 144 * np.arange(E)
    r0, c0, v0 = oracle.bc_kc0_batch(cdof, init_k, x, vxy, props, pid=pid)
    r = np.zeros(144 * E, np.int64); c = np.zeros(144 * E, np.int64); v = np.zeros(144 * E)
    batch.beamc_update_KC0(r, c, v, x, cdof, init_k, vxy, props, pid=pid)
    assert (r == r0).all() and (c == c0).all()
    assert blockwise_rel_err(v, v0, 144) < REL_TOL


def _random_beams(golden, E=173, seed=7):
    """E random 3D beams (E not a multiple of the 32-beam tile: the last tile is
    partial), varied vxy, every golden property record, shuffled non-contiguous
    offsets with untouched slots at both ends, and a global displacement field."""
    g = golden('beamc_elements')
    rng = np.random.default_rng(seed)
    nn = 90
    x = rng.normal(size=3 * nn)
    conn = np.stack([rng.integers(0, nn, E), rng.integers(0, nn, E)], 1)
    same = conn[:, 0] == conn[:, 1]
    conn[same, 1] = (conn[same, 0] + 1) % nn
    vxy = rng.normal(size=(E, 3))
    props = g['prop']
    pid = (np.arange(E) % len(props))[rng.permutation(E)].astype(np.int32)
    init_k = 144 * rng.permutation(E).astype(np.int64) + 144
    u = rng.normal(scale=1e-3, size=6 * nn)
    return 6 * conn, x, vxy, props, pid, init_k, u, 144 * (E + 2)


@pytest.mark.parametrize('values_only', [0, 1])
def test_batched_beam_kg_matches_oracle(gpulib, oracle, golden, values_only):
    """BeamC KG of many beams (several 32-beam tiles, warp-uniform block turns,
    u gathered from the global field) against the oracle (beamc.pyx:1392-2179);
    += onto existing values; with update_KGv_only=1 the indices stay untouched."""
    from pyfe3d_gb300 import batch
    cdof, x, vxy, props, pid, init_k, u, n = _random_beams(golden)
    rng = np.random.default_rng(3)
    v_init = rng.normal(size=n)
    r_init = np.full(n, -5, np.int64)
    r0, c0, v0 = oracle.bc_kg_batch(cdof, init_k, x, u, vxy, props, pid=pid, Kr=r_init.copy(),
                                    Kc=r_init.copy(), Kv=v_init.copy(), values_only=values_only)
    r, c, v = r_init.copy(), r_init.copy(), v_init.copy()
    batch.beamc_update_KG(r, c, v, x, u, cdof, init_k, vxy, props, pid=pid, update_KGv_only=values_only)
    assert (r == r0).all() and (c == c0).all()
    if values_only:
        assert (r == -5).all() and (c == -5).all()
    else:
        assert (r[144:-144] >= 0).all()
    assert (v[:144] == v_init[:144]).all() and (v[-144:] == v_init[-144:]).all()
    assert blockwise_rel_err(v[144:-144] - v_init[144:-144], v0[144:-144] - v_init[144:-144], 144) < REL_TOL


@pytest.mark.parametrize('mtype', [0, 1])
def test_batched_beam_mass_matches_oracle(gpulib, oracle, golden, mtype):
    """BeamC M of many beams, consistent (mtype 0, 144 slots) and lumped (mtype 1,
    36 slots; the other 108 stay untouched) against the oracle (beamc.pyx:2181-3152)."""
    from pyfe3d_gb300 import batch
    cdof, x, vxy, props, pid, init_k, u, n = _random_beams(golden, seed=8)
    rng = np.random.default_rng(4)
    v_init = rng.normal(size=n)
    r_init = np.full(n, -5, np.int64)
    r0, c0, v0 = oracle.bc_m_batch(cdof, init_k, x, vxy, props, pid=pid, Kr=r_init.copy(),
                                   Kc=r_init.copy(), Kv=v_init.copy(), mtype=mtype)
    r, c, v = r_init.copy(), r_init.copy(), v_init.copy()
    batch.beamc_update_M(r, c, v, x, cdof, init_k, vxy, props, pid=pid, mtype=mtype)
    assert (r == r0).all() and (c == c0).all()
    assert (v[:144] == v_init[:144]).all() and (v[-144:] == v_init[-144:]).all()
    if mtype == 1:
        untouched = np.ones(n, bool)
        for k in init_k:
            untouched[k:k + 36] = False
        assert (v[untouched] == v_init[untouched]).all() and (r[untouched] == -5).all()
    d = (v - v_init)[144:-144]
    d0 = (v0 - v_init)[144:-144]
    assert np.abs(d0).max() > 0
    assert blockwise_rel_err(d, d0, 144) < REL_TOL


def test_reference_cantilever_tip(gpulib):
    """tests/test_beamc_static_point_load.py of the reference through the GPU
    per-element API: tip deflection 7.48768 within rtol 1e-3."""
    from scipy.sparse import coo_matrix
    from scipy.sparse.linalg import spsolve
    from pyfe3d_gb300 import BeamC, BeamCData, BeamCProbe, BeamProp, DOF, INT, DOUBLE
    n, L, a, P = 9, 8, 5, -10.e3
    E, nu = 203.e9, 0.3
    x = np.linspace(0, L, n)
    ncoords = np.vstack((x, np.ones_like(x), np.zeros_like(x))).T
    ncf = ncoords.flatten()
    hy = hz = 0.05
    prop = BeamProp()
    prop.A = hy * hz
    prop.E = E
    prop.G = 5 / 6. * E / 2 / (1 + nu)
    prop.Izz = hz * hy ** 3 / 12
    prop.Iyy = hz ** 3 * hy / 12
    prop.J = prop.Izz + prop.Iyy
    data = BeamCData()
    ne = n - 1
    KC0r = np.zeros(data.KC0_SPARSE_SIZE * ne, dtype=INT)
    KC0c = np.zeros(data.KC0_SPARSE_SIZE * ne, dtype=INT)
    KC0v = np.zeros(data.KC0_SPARSE_SIZE * ne, dtype=DOUBLE)
    N = DOF * n
    probe = BeamCProbe()
    for e in range(ne):
        beam = BeamC(probe)
        beam.init_k_KC0 = e * data.KC0_SPARSE_SIZE
        beam.c1 = DOF * e
        beam.c2 = DOF * (e + 1)
        beam.update_rotation_matrix(1., 1., 0, ncf)
        beam.update_probe_xe(ncf)
        beam.update_KC0(KC0r, KC0c, KC0v, prop)
    KC0 = coo_matrix((KC0v, (KC0r, KC0c)), shape=(N, N)).tocsc()
    bk = np.zeros(N, dtype=bool)
    bk[:DOF] = True
    bu = ~bk
    fext = np.zeros(N)
    load = np.isclose(x, a)
    fext[1::DOF][load] = P
    fext[2::DOF][load] = -P
    u = np.zeros(N)
    u[bu] = spsolve(KC0[bu, :][:, bu], fext[bu])
    assert np.isclose(u[1::DOF].min(), -7.48768, rtol=0.001)
    assert np.isclose(u[2::DOF].max(), +7.48768, rtol=0.001)
