"""Internal forces (update_probe_finte / update_fint) of Quad4 and BeamC and
Quad4.update_KG_given_stress: per-element API against the reference's frozen
outputs, batched kernels against the oracle."""
import numpy as np
import pytest

from conftest import REL_TOL, blockwise_rel_err

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(b).max(), 1e-300)


def test_quad4_per_element_finte_and_kg_given_stress(gpulib, golden):
    from pyfe3d_gb300 import INT, Quad4, Quad4Probe
    from pyfe3d_gb300.shellprop import SHELL_FIELDS, ShellProp
    g = golden('quad4_elements')
    props = []
    for rec in g['props']:
        p = ShellProp()
        for i, f in enumerate(SHELL_FIELDS):
            setattr(p, f, float(rec[i]))
        props.append(p)
    probe = Quad4Probe()
    for t in range(len(g['x'])):
        q = Quad4(probe)
        q.c1, q.c2, q.c3, q.c4 = (int(v) for v in g['c'][t])
        xmat = g['xmat'][t]
        if np.isnan(xmat).any():
            q.update_rotation_matrix(g['x'][t])
        else:
            q.update_rotation_matrix(g['x'][t], *xmat)
        q.update_probe_xe(g['x'][t])
        q.update_probe_ue(g['u'][t])
        prop = props[g['pid'][t]]
        q.update_probe_finte(prop)
        assert rel(probe.finte, g['finte'][t]) < 1e-12, t
        # given stress: += onto existing values at a non-zero offset
        q.init_k_KG = 144
        r = np.zeros(3 * 144, INT); c = np.zeros(3 * 144, INT); v = np.zeros(3 * 144)
        v[144:288] = 2.0
        N = g['Nstress'][t]
        q.update_KG_given_stress(float(N[0]), float(N[1]), float(N[2]), r, c, v)
        assert (r[144:288] == g['KGsr'][t]).all() and (c[144:288] == g['KGsc'][t]).all()
        assert blockwise_rel_err(v[144:288] - 2.0, g['KGsv'][t], 144) < REL_TOL
        assert (v[:144] == 0).all() and (v[288:] == 0).all()


def test_beamc_per_element_finte_and_fint(gpulib, golden):
    from pyfe3d_gb300 import BeamC, BeamCProbe
    from pyfe3d_gb300.shellprop import BEAM_FIELDS, BeamProp
    g = golden('beamc_elements')
    probe = BeamCProbe()
    for t in range(len(g['x'])):
        b = BeamC(probe)
        b.c1, b.c2 = (int(v) for v in g['c'][t])
        b.update_rotation_matrix(*g['vxy'][t], g['x'][t])
        b.update_probe_xe(g['x'][t])
        b.update_probe_ue(g['u'][t])
        bp = BeamProp()
        for i, f in enumerate(BEAM_FIELDS):
            setattr(bp, f, float(g['prop'][t][i]))
        b.update_probe_finte(bp)
        assert rel(probe.finte, g['finte'][t]) < 1e-12, t
        fint = np.ones(12)
        b.update_fint(fint, bp)
        assert rel(fint - 1., g['fint'][t]) < 1e-12, t


def test_batched_kg_given_stress_matches_oracle(gpulib, oracle):
    from pyfe3d_gb300 import batch
    from pyfe3d_gb300.meshes import config2
    m, props, pid, bk, f = config2(21)
    rng = np.random.default_rng(3)
    x = m.x.copy()
    x[2::3] = rng.uniform(-0.01, 0.01, m.nnodes)   # a slightly curved (non-flat) surface
    N = rng.normal(size=(m.E, 3)) * 1e3
    nk = 144 * m.E
    r = np.zeros(nk, np.int64); c = np.zeros(nk, np.int64); v = np.zeros(nk)
    batch.quad4_update_KG_given_stress(r, c, v, x, m.cdof, m.init_k(144), N)
    R, mm, xe, area = (t.cpu().numpy() for t in batch.quad4_frames(x, m.cdof))
    ro = np.zeros(nk, np.int64); co = np.zeros(nk, np.int64); vo = np.zeros(nk)
    for e in range(m.E):
        oracle.q4_kg_given_stress(R[e], xe[e], N[e], m.cdof[e], 144 * e, ro, co, vo)
    assert (r == ro).all() and (c == co).all()
    assert blockwise_rel_err(v, vo, 144) < REL_TOL
    # one stress state shared by all elements
    v1 = np.zeros(nk)
    batch.quad4_update_KG_given_stress(r, c, v1, x, m.cdof, m.init_k(144), N[0])
    vo1 = np.zeros(nk)
    for e in range(m.E):
        oracle.q4_kg_given_stress(R[e], xe[e], N[0], m.cdof[e], 144 * e, ro, co, vo1)
    assert blockwise_rel_err(v1, vo1, 144) < REL_TOL


def test_batched_fint_is_K_times_u(gpulib, oracle):
    """fint assembled over all elements equals K u (the reference's
    equilibrium check, tests/test_quad4_static_point_load.py:117-132)."""
    from scipy.sparse import coo_matrix
    from pyfe3d_gb300 import batch
    from pyfe3d_gb300.meshes import config2, stringer_records
    m, props, pid, bk, f = config2(21)
    rng = np.random.default_rng(4)
    u = rng.normal(size=m.N) * 1e-3
    r, c, v = oracle.q4_kc0_batch(m.cdof, m.init_k(576), m.x, props, pid=pid)
    Ku = coo_matrix((v, (r, c)), shape=(m.N, m.N)).tocsr() @ u
    fint = np.zeros(m.N)
    batch.quad4_update_fint(fint, m.x, u, m.cdof, props, pid=pid)
    assert np.abs(fint - Ku).max() <= 1e-11 * np.abs(Ku).max()
    # beams along the x = const grid lines
    nids = m.nids
    bcdof = (6 * np.stack([nids[:-1, 5].ravel(), nids[1:, 5].ravel()], 1)).astype(np.int64)
    Eb = bcdof.shape[0]
    brec = stringer_records()[None, :]
    vxy = np.array([0., 1., 0.])
    rb, cb, vb = oracle.bc_kc0_batch(bcdof, 144 * np.arange(Eb), m.x, np.tile(vxy, (Eb, 1)), brec)
    Kbu = coo_matrix((vb, (rb, cb)), shape=(m.N, m.N)).tocsr() @ u
    fb = np.zeros(m.N)
    finte = batch.beamc_update_fint(fb, m.x, u, bcdof, vxy, brec)
    assert np.abs(fb - Kbu).max() <= 1e-11 * np.abs(Kbu).max()
    assert tuple(finte.shape) == (Eb, 12)
