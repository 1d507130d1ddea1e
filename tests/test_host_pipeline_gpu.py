"""update_KC0 on host buffers (numpy / pinned CPU tensors): the pipelined
chunked path (fe3d_quad4_kc0_host) gives bit-identical triplets to the
device path, keeps the += semantics and leaves untouched slots alone."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _plate(n=41):
    from pyfe3d_gb300.meshes import config2
    return config2(n)


def _device_ref(m, props, pid, k0, nk, Kv0):
    import torch
    from pyfe3d_gb300 import batch
    dev = torch.device('cuda')
    Kr = torch.full((nk,), -7, dtype=torch.int64, device=dev)
    Kc = torch.full((nk,), -7, dtype=torch.int64, device=dev)
    Kv = torch.tensor(Kv0, device=dev)
    batch.quad4_update_KC0(Kr, Kc, Kv, m.x, m.cdof, m.init_k(576, start=k0), props, pid=pid)
    return Kr.cpu().numpy(), Kc.cpu().numpy(), Kv.cpu().numpy()


@pytest.mark.parametrize('pinned', [False, True])
def test_host_path_matches_device_path(gpulib, pinned):
    import torch
    from pyfe3d_gb300 import _lib, batch
    m, props, pid, bk, f = _plate()
    k0 = 100                         # slots before and after the elements stay untouched
    nk = k0 + 576 * m.E + 50
    rng = np.random.default_rng(0)
    Kv0 = rng.normal(size=nk)        # += onto existing values
    rr, cr, vr = _device_ref(m, props, pid, k0, nk, Kv0)
    Kr = np.full(nk, -7, dtype=np.int64)
    Kc = np.full(nk, -7, dtype=np.int64)
    Kv = Kv0.copy()
    args = (m.x, m.cdof, m.init_k(576, start=k0), props)
    if pinned:
        Kr, Kc, Kv = (torch.from_numpy(a).pin_memory() for a in (Kr, Kc, Kv))
        args = tuple(torch.from_numpy(np.ascontiguousarray(a)).pin_memory() for a in args)
    batch.quad4_update_KC0(Kr, Kc, Kv, *args, pid=pid)
    Kr, Kc, Kv = (np.asarray(a) for a in (Kr, Kc, Kv))
    assert np.array_equal(Kr, rr) and np.array_equal(Kc, cr)
    assert np.array_equal(Kv, vr)
    assert (Kr[:k0] == -7).all() and (Kr[-50:] == -7).all() and np.array_equal(Kv[:k0], Kv0[:k0])
    # values only, small chunks (several rounds of the three staging sets)
    Kv2 = Kv0.copy()
    err = ctypes.c_int(0)
    lib = _lib.load()
    ik = m.init_k(576, start=k0)
    P = np.ascontiguousarray(props)
    rc = lib.fe3d_quad4_kc0_host(m.E, m.cdof.ctypes.data, ik.ctypes.data, m.x.ctypes.data, m.x.size,
                                 P.ctypes.data, P.shape[0], pid.ctypes.data, None, None, Kv2.ctypes.data, nk,
                                 1, 97, ctypes.byref(err), _lib.stream_ptr())
    assert rc == 0 and err.value == 0
    assert np.array_equal(Kv2, vr)


def test_non_contiguous_offsets_take_the_staged_device_path(gpulib):
    from pyfe3d_gb300 import batch
    m, props, pid, bk, f = _plate(11)
    perm = np.random.default_rng(1).permutation(m.E)
    ik = (576 * perm).astype(np.int64)   # permuted slots: the device path handles them
    nk = 576 * m.E
    Kr = np.zeros(nk, np.int64); Kc = np.zeros(nk, np.int64); Kv = np.zeros(nk)
    batch.quad4_update_KC0(Kr, Kc, Kv, m.x, m.cdof, ik, props, pid=pid)
    Kr2 = np.zeros(nk, np.int64); Kc2 = np.zeros(nk, np.int64); Kv2 = np.zeros(nk)
    batch.quad4_update_KC0(Kr2, Kc2, Kv2, m.x, m.cdof, m.init_k(576), props, pid=pid)
    blocks = Kv.reshape(m.E, 576)
    assert np.array_equal(blocks[perm], Kv2.reshape(m.E, 576))


def test_host_offsets_out_of_range_raise(gpulib):
    from pyfe3d_gb300 import _lib, batch
    m, props, pid, bk, f = _plate(11)
    nk = 576 * m.E - 1
    Kr = np.zeros(nk, np.int64); Kc = np.zeros(nk, np.int64); Kv = np.zeros(nk)
    with pytest.raises(_lib.Fe3dError):
        batch.quad4_update_KC0(Kr, Kc, Kv, m.x, m.cdof, m.init_k(576), props, pid=pid)


def test_ramped_chunks_match_device_path(gpulib):
    """10,000 elements in chunks of 4,096: the sizes ramp 512, 1024, 2048,
    4096 then 2320 (five chunks over the three staging sets)."""
    from pyfe3d_gb300 import _lib
    m, props, pid, bk, f = _plate(101)
    k0 = 3
    nk = k0 + 576 * m.E
    Kv0 = np.random.default_rng(5).normal(size=nk)
    rr, cr, vr = _device_ref(m, props, pid, k0, nk, Kv0)
    Kr = np.full(nk, -7, dtype=np.int64)
    Kc = np.full(nk, -7, dtype=np.int64)
    Kv = Kv0.copy()
    err = ctypes.c_int(0)
    lib = _lib.load()
    ik = m.init_k(576, start=k0)
    P = np.ascontiguousarray(props)
    rc = lib.fe3d_quad4_kc0_host(m.E, m.cdof.ctypes.data, ik.ctypes.data, m.x.ctypes.data, m.x.size,
                                 P.ctypes.data, P.shape[0], pid.ctypes.data, Kr.ctypes.data, Kc.ctypes.data,
                                 Kv.ctypes.data, nk, 0, 4096, ctypes.byref(err), _lib.stream_ptr())
    assert rc == 0 and err.value == 0
    assert np.array_equal(Kr, rr) and np.array_equal(Kc, cr) and np.array_equal(Kv, vr)
