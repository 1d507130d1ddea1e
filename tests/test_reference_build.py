"""The reference's own element modules compiled by oracle/build_ref.py (the
CPU reference of the benchmark) reproduce the frozen reference outputs."""
import numpy as np
import pytest

from conftest import REL_TOL, blockwise_rel_err


@pytest.fixture(scope='module')
def ref():
    from oracle import build_ref
    build_ref.build()
    r = build_ref.load()
    if r is None:
        pytest.skip('the reference modules are not built here (no generated sources)')
    return r


def test_compiled_reference_matches_frozen_outputs(ref, golden):
    from pyfe3d_gb300.shellprop import SHELL_FIELDS
    g = golden('quad4_elements')
    probe = ref.Quad4Probe()
    for t in range(len(g['x'])):
        q = ref.Quad4(probe)
        q.c1, q.c2, q.c3, q.c4 = (int(v) for v in g['c'][t])
        xmat = g['xmat'][t]
        if np.isnan(xmat).any():
            q.update_rotation_matrix(g['x'][t])
        else:
            q.update_rotation_matrix(g['x'][t], *xmat)
        q.update_probe_xe(g['x'][t])
        p = ref.ShellProp()
        for i, f in enumerate(SHELL_FIELDS):
            setattr(p, f, float(g['props'][g['pid'][t]][i]))
        r = np.zeros(576, ref.INT)
        c = np.zeros(576, ref.INT)
        v = np.zeros(576)
        q.update_KC0(r, c, v, p)
        assert (r == g['KC0r'][t]).all() and (c == g['KC0c'][t]).all()
        assert blockwise_rel_err(v, g['KC0v'][t], 576) < REL_TOL


def test_bench_reference_loop_matches_oracle(ref):
    """The benchmark's reference loop (bench._refw_run) assembles the same
    triplet values as the oracle on the first elements of the plate."""
    import bench
    from oracle import oracle
    bench._refw_init(21)
    m, props, pid = bench._REFW['m'], bench._REFW['props'], bench._REFW['pid']
    n, dt, checksum = bench._refw_run(0, 50)
    _, _, v0 = oracle.q4_kc0_batch(m.cdof[:50], 576 * np.arange(50), m.x, props, pid=pid[:50])
    assert n == 50 and dt > 0
    assert abs(checksum - np.abs(v0).sum()) <= 1e-12 * np.abs(v0).sum()
