"""Stiffened panel: laminated Quad4 skin plus BeamC stringers sharing its
nodes, assembled into one COO system and solved on the GPU (the mixed-element
configuration, which no reference test covers; pinned here by the oracle's
element triplets and scipy's direct solve of the same matrix)."""
import numpy as np
import pytest

from conftest import REL_TOL, blockwise_rel_err

pytestmark = pytest.mark.gpu


def _assemble(p):
    import torch
    from pyfe3d_gb300 import batch
    nq, nb = p.coo_sizes()
    dev = torch.device('cuda')
    Kr = torch.zeros(nq + nb, dtype=torch.int64, device=dev)
    Kc = torch.zeros(nq + nb, dtype=torch.int64, device=dev)
    Kv = torch.zeros(nq + nb, dtype=torch.float64, device=dev)
    batch.quad4_update_KC0(Kr, Kc, Kv, p.skin.x, p.skin.cdof, p.skin.init_k(576), p.shell_props)
    batch.beamc_update_KC0(Kr, Kc, Kv, p.skin.x, p.beam_cdof, nq + 144 * np.arange(p.Eb), p.vxy,
                           p.beam_props)
    return Kr, Kc, Kv


def test_panel_triplets_match_oracle(gpulib, oracle):
    from pyfe3d_gb300.meshes import config3
    p = config3(50)
    nq, nb = p.coo_sizes()
    Kr, Kc, Kv = _assemble(p)
    r, c, v = Kr.cpu().numpy(), Kc.cpu().numpy(), Kv.cpu().numpy()
    r0, c0, v0 = oracle.q4_kc0_batch(p.skin.cdof, p.skin.init_k(576), p.skin.x, p.shell_props)
    assert (r[:nq] == r0).all() and (c[:nq] == c0).all()
    assert blockwise_rel_err(v[:nq], v0, 576) < REL_TOL
    vxy = np.tile(p.vxy, (p.Eb, 1))
    r1, c1, v1 = oracle.bc_kc0_batch(p.beam_cdof, 144 * np.arange(p.Eb), p.skin.x, vxy, p.beam_props)
    assert (r[nq:] == r1).all() and (c[nq:] == c1).all()
    assert blockwise_rel_err(v[nq:], v1, 144) < REL_TOL


@pytest.mark.parametrize('precision', [0, 1, 2])
def test_panel_static_solve(gpulib, precision):
    from scipy.sparse.linalg import spsolve
    from pyfe3d_gb300.meshes import config3
    from pyfe3d_gb300.solver import CSRPattern, Solver
    p = config3(50)
    Kr, Kc, Kv = _assemble(p)
    pat = CSRPattern(Kr, Kc, p.N, p.bk)
    vals = pat.assemble(Kv)
    s = Solver(pat).setup(vals, mixed=precision == 1, split=precision == 2)
    fr = pat.reduce(p.f)
    ur, st = s.solve(fr, tol=1e-8, precision=precision)
    assert st['status'] == 'converged' and st['relres'] <= 1e-8, st
    uref = spsolve(pat.to_scipy(vals).tocsc(), fr.cpu().numpy())
    err = np.linalg.norm(ur.cpu().numpy() - uref) / np.linalg.norm(uref)
    assert err <= 1e-7, err
