"""Seeded mesh generators: shapes, boundary conditions and loads (CPU)."""
import numpy as np

from pyfe3d_gb300.meshes import DOF, BatchedPlates, config2, config3


def test_batched_plates_layout():
    bp = BatchedPlates(nplates=20, nmin=8, nmax=40, seed=7)
    assert bp.E == int((bp.nx * bp.ny).sum()) and bp.nnodes == int(((bp.nx + 1) * (bp.ny + 1)).sum())
    assert bp.nx.min() >= 8 and bp.nx.max() <= 40 and bp.ny.min() >= 8 and bp.ny.max() <= 40
    assert (bp.a >= 0.5).all() and (bp.a <= 2.0).all() and (bp.b >= 0.5).all() and (bp.b <= 2.0).all()
    assert bp.inst_of_dof.shape == (bp.N,)
    assert np.all(np.diff(bp.inst_of_dof) >= 0)
    for i in range(bp.P):
        e = slice(int(bp.elem0[i]), int(bp.elem0[i + 1]))
        d = bp.plate_dofs(i)
        # every element of plate i references only plate i's DOFs
        assert bp.cdof[e].min() >= d.start and bp.cdof[e].max() < d.stop
        assert (bp.pid[e] == i).all()
        assert (bp.inst_of_dof[d] == i).all()
        # one -1000 N point load on w at the centre
        fi = bp.f[d]
        assert np.count_nonzero(fi) == 1 and fi.min() == -1000.
        k = int(np.nonzero(fi)[0][0])
        assert k % DOF == 2
        # edges: clamped -> 6 fixed DOFs per edge node, else u, v, w
        bki = bp.bk[d].reshape(-1, DOF)
        nedge = 2 * (int(bp.nx[i]) + 1 + int(bp.ny[i]) + 1) - 4
        assert bki.any(axis=1).sum() == nedge
        assert bki.sum() == nedge * (6 if bp.clamped[i] else 3)
    # property records: one per plate, isotropic (B = 0)
    assert bp.props.shape[0] == bp.P


def test_batched_plates_is_seeded():
    a = BatchedPlates(nplates=5, seed=3)
    b = BatchedPlates(nplates=5, seed=3)
    assert np.array_equal(a.x, b.x) and np.array_equal(a.props, b.props) and np.array_equal(a.bk, b.bk)


def test_config2_and_config3_shapes():
    m, props, pid, bk, f = config2(11)
    assert m.E == 100 and props.shape[0] == 100 and pid.shape == (100,)
    assert (f[bk] == 0).all() and (f[2::DOF][~bk[2::DOF]] == -1.).all()
    p = config3(20)
    assert p.Eq == 400 and p.Eb == 9 * 20
    assert p.beam_cdof.max() < p.N
