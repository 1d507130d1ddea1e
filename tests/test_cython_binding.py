"""The compiled Cython binding of the C ABI (``pyfe3d_gb300.fe3d_cy``, built
from pyfe3d_gb300/cy/) loads, and on the GPU gives the same triplets as the
ctypes layer: the route a Cython build of pyfe3d would take."""
import numpy as np
import pytest


def _mod():
    from pyfe3d_gb300 import build
    if build.build_cython() is None:
        pytest.skip('no Cython and no generated C++ for the binding here')
    from pyfe3d_gb300 import fe3d_cy
    return fe3d_cy


def test_binding_loads_without_gpu():
    cy = _mod()
    from pyfe3d_gb300 import _lib
    assert cy.version() == _lib.load().fe3d_version()
    assert cy.error_string(-1) == 'invalid argument'


@pytest.mark.gpu
def test_binding_kc0_matches_ctypes_path(gpulib):
    import torch
    from pyfe3d_gb300 import _lib, batch
    from pyfe3d_gb300.meshes import config2
    cy = _mod()
    m, props, pid, bk, f = config2(31)
    dev = torch.device('cuda')
    n = 576 * m.E
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    x, cdof, ik, P, pd = t(m.x), t(m.cdof), t(m.init_k(576)), t(props), t(pid)
    out = [torch.zeros(n, dtype=dt, device=dev) for dt in (torch.int64, torch.int64, torch.float64)]
    err = _lib.err_word()
    rc = cy.quad4_kc0(m.E, cdof.data_ptr(), ik.data_ptr(), x.data_ptr(), x.numel(), P.data_ptr(), P.shape[0],
                      pd.data_ptr(), out[0].data_ptr(), out[1].data_ptr(), out[2].data_ptr(), n, 0,
                      err.data_ptr(), torch.cuda.current_stream().cuda_stream)
    assert rc == 0
    _lib.check(rc, 'fe3d_cy.quad4_kc0', err)
    ref = [torch.zeros(n, dtype=dt, device=dev) for dt in (torch.int64, torch.int64, torch.float64)]
    batch.quad4_update_KC0(ref[0], ref[1], ref[2], x, cdof, ik, P, pid=pd)
    for a, b in zip(out, ref):
        assert torch.equal(a, b)
