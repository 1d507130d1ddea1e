"""Fused element -> CSR assembly against the triplet path.

The reference's users assemble with `coo_matrix((v, (r, c))).tocsc()` and
slice out the free DOFs (tests/test_quad4_static_point_load.py:80-99).  The
triplet path here (update_KC0 -> CSRPattern -> assemble) is pinned to that
by test_solver_gpu.py; the fused path (ElementPattern + FusedMap, no
triplets) must give the same pattern bit for bit and the same values up to
the order in which the <= 4 element contributions of an entry are summed.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

# entries are sums of up to four element contributions added in another
# order: |v - v_ref| <= SUM_TOL * max |row of v_ref|
SUM_TOL = 1e-14


def _coo_csr(m, props, pid, bk, x=None, xmat=None):
    import torch
    from pyfe3d_gb300 import batch
    from pyfe3d_gb300.solver import CSRPattern
    dev = torch.device('cuda')
    n = 576 * m.E
    Kr = torch.zeros(n, dtype=torch.int64, device=dev)
    Kc = torch.zeros(n, dtype=torch.int64, device=dev)
    Kv = torch.zeros(n, dtype=torch.float64, device=dev)
    batch.quad4_update_KC0(Kr, Kc, Kv, m.x if x is None else x, m.cdof, m.init_k(576), props, pid=pid, xmat=xmat)
    pat = CSRPattern(Kr, Kc, m.N, bk)
    return pat, pat.assemble(Kv)


def _rowwise_err(pat, v, v0):
    rp = pat.rowptr.cpu().numpy()
    a = np.abs(v0)
    d = np.abs(v - v0)
    rmax = np.maximum.reduceat(a, rp[:-1]) if len(a) else a
    dmax = np.maximum.reduceat(d, rp[:-1]) if len(d) else d
    rmax[rmax == 0] = 1.
    return (dmax / rmax).max()


def _same_pattern(p1, p0):
    assert p1.nrows == p0.nrows and p1.nnz == p0.nnz
    assert (p1.rowptr.cpu().numpy() == p0.rowptr.cpu().numpy()).all()
    assert (p1.colind.cpu().numpy() == p0.colind.cpu().numpy()).all()
    assert (p1.dof_of_row.cpu().numpy() == p0.dof_of_row.cpu().numpy()).all()


def _plates():
    from pyfe3d_gb300.meshes import config1, config2
    yield 'config1', config1()
    yield 'config2_101', config2(101)


@pytest.mark.parametrize('case', ['config1', 'config2_101'])
def test_quad4_fused_matches_triplet_assembly(gpulib, case):
    from pyfe3d_gb300 import batch
    from pyfe3d_gb300.solver import ElementPattern, FusedMap
    m, props, pid, bk, f = dict(_plates())[case]
    pat0, v0 = _coo_csr(m, props, pid, bk)
    pat = ElementPattern([m.cdof], m.N, bk)
    _same_pattern(pat, pat0)
    fm = FusedMap(pat, [m.cdof])
    assert fm.colors().sum() == m.E and len(fm.colors()) == 4
    vals = fm.new_values()
    vals.fill_(123.)  # assign mode overwrites whatever the array held
    batch.quad4_update_KC0_csr(vals, fm, m.x, props, pid=pid)
    v = vals.cpu().numpy()
    assert _rowwise_err(pat, v, v0.cpu().numpy()) <= SUM_TOL
    # deterministic: a second update gives the same bits
    batch.quad4_update_KC0_csr(vals, fm, m.x, props, pid=pid)
    assert (vals.cpu().numpy() == v).all()
    # add mode accumulates onto the existing values
    vals.fill_(1.)
    batch.quad4_update_KC0_csr(vals, fm, m.x, props, pid=pid, mode='add')
    assert _rowwise_err(pat, vals.cpu().numpy() - 1., v0.cpu().numpy()) <= 1e-12


@pytest.mark.parametrize('kind', ['rotated', 'curved'])
def test_quad4_fused_non_flat_laminated(gpulib, kind):
    """Elements evaluated in their own frame (FP64, block rotation), laminated
    and isotropic records mixed, material directions, SS edges."""
    from pyfe3d_gb300 import batch
    from pyfe3d_gb300.meshes import PlateMesh
    from pyfe3d_gb300.shellprop import isotropic_plate_records, shell_record
    from pyfe3d_gb300.shellprop_utils import laminated_plate
    from pyfe3d_gb300.solver import ElementPattern, FusedMap
    m = PlateMesh(17, 13, 1.1, 0.9, perturb=0.2, seed=4)
    x = m.ncoords.copy()
    rng = np.random.default_rng(9)
    if kind == 'rotated':
        q, _ = np.linalg.qr(rng.normal(size=(3, 3)))
        x = x @ q.T
    else:
        x[:, 2] = 0.15 * np.sin(2 * x[:, 0]) * np.cos(3 * x[:, 1])
    x = x.ravel()
    props = isotropic_plate_records(rng.uniform(0.002, 0.05, m.E), 70e9, 0.3)
    props[::4] = shell_record(laminated_plate([0, 45, -45, 90, 30], plyt=0.0011,
                                              laminaprop=(142.5e9, 8.7e9, 0.28, 5.1e9, 5.1e9, 5.1e9),
                                              offset=0.001))
    pid = rng.permutation(m.E).astype(np.int32)
    xmat = rng.normal(size=(m.E, 3))
    bk = m.bc_mask((0, 1, 2))
    pat0, v0 = _coo_csr(m, props, pid, bk, x=x, xmat=xmat)
    pat = ElementPattern([m.cdof], m.N, bk)
    _same_pattern(pat, pat0)
    fm = FusedMap(pat, [m.cdof])
    vals = fm.new_values()
    batch.quad4_update_KC0_csr(vals, fm, x, props, pid=pid, xmat=xmat)
    assert _rowwise_err(pat, vals.cpu().numpy(), v0.cpu().numpy()) <= SUM_TOL


def test_panel_quads_and_beams_fused(gpulib):
    """Stiffened panel (laminated skin + BeamC stringers on shared nodes): the
    skin through the fused Quad4 kernel, the stringers through a values-only
    update_KC0 scattered by the map, against the triplet assembly of both."""
    import torch
    from pyfe3d_gb300 import batch
    from pyfe3d_gb300.meshes import config3
    from pyfe3d_gb300.solver import CSRPattern, ElementPattern, FusedMap
    p = config3(50)
    dev = torch.device('cuda')
    nq, nb = p.coo_sizes()
    Kr = torch.zeros(nq + nb, dtype=torch.int64, device=dev)
    Kc = torch.zeros_like(Kr)
    Kv = torch.zeros(nq + nb, dtype=torch.float64, device=dev)
    sk = p.skin
    batch.quad4_update_KC0(Kr, Kc, Kv, sk.x, sk.cdof, sk.init_k(576), p.shell_props)
    bik = nq + 144 * np.arange(p.Eb, dtype=np.int64)
    batch.beamc_update_KC0(Kr, Kc, Kv, sk.x, p.beam_cdof, bik, p.vxy, p.beam_props)
    pat0 = CSRPattern(Kr, Kc, p.N, p.bk)
    v0 = pat0.assemble(Kv).cpu().numpy()
    groups = [sk.cdof, p.beam_cdof]
    pat = ElementPattern(groups, p.N, p.bk)
    _same_pattern(pat, pat0)
    fm = FusedMap(pat, groups)
    assert len(fm.colors(1)) == 2  # a chain of beams takes two colours
    vals = fm.new_values()
    vals.fill_(-7.)
    batch.quad4_update_KC0_csr(vals, fm, sk.x, p.shell_props, group=0)
    kb = torch.zeros(144 * p.Eb, dtype=torch.float64, device=dev)
    batch.beamc_update_KC0(None, None, kb, sk.x, p.beam_cdof, 144 * np.arange(p.Eb), p.vxy, p.beam_props,
                           update_KC0v_only=1)
    fm.scatter(vals, 1, 144 * np.arange(p.Eb), kb)
    assert _rowwise_err(pat, vals.cpu().numpy(), v0) <= SUM_TOL


def test_fused_static_solve_matches_reference(gpulib, golden):
    """The 21x21-node plate solved from fused values against the reference's
    own spsolve displacements (frozen)."""
    from pyfe3d_gb300 import batch
    from pyfe3d_gb300.meshes import config1
    from pyfe3d_gb300.solver import ElementPattern, FusedMap, Solver
    g = golden('plate_static')
    m, props, pid, bk, f = config1()
    pat = ElementPattern([m.cdof], m.N, bk)
    fm = FusedMap(pat, [m.cdof])
    vals = batch.quad4_update_KC0_csr(fm.new_values(), fm, m.x, props)
    ur, st = Solver(pat).setup(vals).solve(pat.reduce(f), tol=1e-10)
    assert st['status'] == 'converged'
    u = pat.expand(ur).cpu().numpy()
    uref = g['u']
    assert np.linalg.norm(u - uref) / np.linalg.norm(uref) < 1e-7


def test_fused_rejects_triplet_assembly_and_bad_groups(gpulib):
    import torch
    from pyfe3d_gb300 import _lib
    from pyfe3d_gb300.meshes import config1
    from pyfe3d_gb300.solver import ElementPattern, FusedMap
    m, props, pid, bk, f = config1()
    pat = ElementPattern([m.cdof], m.N, bk)
    with pytest.raises(TypeError):
        pat.assemble(torch.zeros(10, dtype=torch.float64, device='cuda'))
    bad = m.cdof.copy()
    bad[3, 1] = bad[3, 0]  # repeated node
    with pytest.raises(_lib.Fe3dError):
        FusedMap(pat, [bad])


def test_mixed_quads_and_triangles_fused(gpulib):
    """A plate whose left half is Quad4 and right half Tria3R (each quad split
    in two), sharing the nodes of the seam: the Quad4 group through the fused
    kernel, the Tria3R group (3-node blocks) scattered by the map from its
    values-only update_KC0; simply supported edges plus a fully clamped corner
    node (no free DOF).  Assign mode against the triplet assembly of both
    groups, then add mode over both groups onto existing values."""
    import torch
    from pyfe3d_gb300 import batch
    from pyfe3d_gb300.meshes import PlateMesh
    from pyfe3d_gb300.shellprop import isotropic_plate_records
    from pyfe3d_gb300.solver import CSRPattern, ElementPattern, FusedMap
    m = PlateMesh(15, 11, 1.4, 1.0, perturb=0.2, seed=9)
    ex = m.ncoords[m.conn].mean(axis=1)[:, 0]
    quads = m.cdof[ex < 0.7]
    split = m.cdof[ex >= 0.7]
    trias = np.concatenate([split[:, [0, 1, 2]], split[:, [0, 2, 3]]])
    bk = m.bc_mask((0, 1, 2))
    bk[0:6] = True
    rng = np.random.default_rng(3)
    Eq, Et = len(quads), len(trias)
    pq = isotropic_plate_records(rng.uniform(0.002, 0.03, Eq), 70e9, 0.3)
    pt = isotropic_plate_records(rng.uniform(0.002, 0.03, Et), 70e9, 0.3)
    pidq, pidt = np.arange(Eq, dtype=np.int32), np.arange(Et, dtype=np.int32)
    dev = torch.device('cuda')
    nq, nt = 576 * Eq, 324 * Et
    Kr = torch.zeros(nq + nt, dtype=torch.int64, device=dev)
    Kc = torch.zeros_like(Kr)
    Kv = torch.zeros(nq + nt, dtype=torch.float64, device=dev)
    batch.quad4_update_KC0(Kr, Kc, Kv, m.x, quads, 576 * np.arange(Eq), pq, pid=pidq)
    batch.tria3r_update_KC0(Kr, Kc, Kv, m.x, trias, nq + 324 * np.arange(Et), pt, pid=pidt)
    pat0 = CSRPattern(Kr, Kc, m.N, bk)
    v0 = pat0.assemble(Kv).cpu().numpy()
    pat = ElementPattern([quads, trias], m.N, bk)
    _same_pattern(pat, pat0)
    fm = FusedMap(pat, [quads, trias])
    kt = torch.zeros(nt, dtype=torch.float64, device=dev)
    batch.tria3r_update_KC0(None, None, kt, m.x, trias, 324 * np.arange(Et), pt, pid=pidt, update_KC0v_only=1)
    vals = fm.new_values()
    vals.fill_(5.)
    batch.quad4_update_KC0_csr(vals, fm, m.x, pq, pid=pidq, group=0)
    fm.scatter(vals, 1, 324 * np.arange(Et), kt)
    assert _rowwise_err(pat, vals.cpu().numpy(), v0) <= SUM_TOL
    # add mode: both groups onto existing values
    vals.fill_(1.)
    batch.quad4_update_KC0_csr(vals, fm, m.x, pq, pid=pidq, group=0, mode='add')
    fm.scatter(vals, 1, 324 * np.arange(Et), kt, mode='add')
    assert _rowwise_err(pat, vals.cpu().numpy() - 1., v0) <= 1e-12
    # the map rejects a Quad4 kernel call on the triangle group
    with pytest.raises(ValueError):
        batch.quad4_update_KC0_csr(vals, fm, m.x, pt, group=1)


def test_fused_values_not_16_byte_aligned(gpulib):
    """A value array that starts 8 bytes past a 16-byte boundary takes the
    8-byte scatter; the result equals the aligned one bit for bit."""
    import torch
    from pyfe3d_gb300 import batch
    from pyfe3d_gb300.meshes import config2
    from pyfe3d_gb300.solver import ElementPattern, FusedMap
    m, props, pid, bk, f = config2(31)
    pat = ElementPattern([m.cdof], m.N, bk)
    fm = FusedMap(pat, [m.cdof])
    ref = batch.quad4_update_KC0_csr(fm.new_values(), fm, m.x, props, pid=pid)
    buf = torch.zeros(pat.nnz + 1, dtype=torch.float64, device='cuda')
    vals = buf[1:]
    assert vals.data_ptr() % 16 == 8
    for mode in ('assign', 'add'):
        vals.zero_()
        batch.quad4_update_KC0_csr(vals, fm, m.x, props, pid=pid, mode=mode)
        assert torch.equal(vals, ref), mode
