"""Loader of ``libfe3d_gb300.so`` and device-buffer plumbing.

The library is a plain C ABI (``include/fe3d_gb300.h``) loaded with ctypes.
PyTorch only provides device memory and the current CUDA stream.  There is no
CPU fallback: every entry point raises if the library or a GPU is missing.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, 'libfe3d_gb300.so')

FE3D_ERRORS = {
    -1: 'invalid argument',
    -2: 'kernel launch failed',
    -3: 'CUDA runtime error',
    -4: 'offset outside the caller\'s buffers',
    -5: 'device allocation failed',
    -6: 'object used in the wrong state',
    -7: 'size above the allocation-free maximum (FE3D_NOALLOC_MAX_ROWS rows)',
}

_lib = None
_err_words = {}

c_i64 = ctypes.c_int64
c_int = ctypes.c_int
c_dbl = ctypes.c_double
c_vp = ctypes.c_void_p

# argument signatures of the exported entry points (see include/fe3d_gb300.h)
_SIGS = {
    'fe3d_version': ([], c_int),
    'fe3d_quad4_frame': ([c_i64, c_vp, c_vp, c_i64, c_vp, c_int, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp], c_int),
    'fe3d_quad4_probe_xe': ([c_i64, c_vp, c_vp, c_i64, c_vp, c_vp, c_vp, c_vp, c_vp], c_int),
    'fe3d_quad4_probe_ue': ([c_i64, c_vp, c_vp, c_i64, c_vp, c_vp, c_vp, c_vp], c_int),
    'fe3d_quad4_kc0': ([c_i64, c_vp, c_vp, c_vp, c_i64, c_vp, c_int, c_vp, c_vp, c_vp, c_vp, c_vp, c_i64,
                        c_vp, c_vp, c_vp, c_vp, c_i64, c_int, c_vp, c_vp], c_int),
    'fe3d_quad4_kg': ([c_i64, c_vp, c_vp, c_vp, c_i64, c_vp, c_int, c_vp, c_i64, c_vp, c_vp, c_vp, c_vp,
                       c_vp, c_i64, c_vp, c_vp, c_vp, c_vp, c_i64, c_vp, c_vp], c_int),
    'fe3d_quad4_m': ([c_i64, c_vp, c_vp, c_vp, c_i64, c_vp, c_vp, c_vp, c_vp, c_i64, c_vp, c_vp, c_vp,
                      c_vp, c_i64, c_int, c_vp, c_vp], c_int),
    'fe3d_quad4_fint': ([c_i64, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_i64, c_vp, c_vp, c_i64,
                         c_vp, c_vp], c_int),
    'fe3d_beamc_frame': ([c_i64, c_vp, c_vp, c_i64, c_vp, c_int, c_vp, c_vp, c_vp, c_vp, c_vp], c_int),
    'fe3d_beamc_probe_xe': ([c_i64, c_vp, c_vp, c_i64, c_vp, c_vp, c_vp, c_vp, c_vp], c_int),
    'fe3d_beamc_probe_ue': ([c_i64, c_vp, c_vp, c_i64, c_vp, c_vp, c_vp, c_vp], c_int),
    'fe3d_beamc_kc0': ([c_i64, c_vp, c_vp, c_vp, c_vp, c_vp, c_i64, c_vp, c_vp, c_vp, c_vp, c_i64, c_int,
                        c_vp, c_vp], c_int),
    'fe3d_beamc_kg': ([c_i64, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_i64, c_vp, c_vp, c_vp, c_vp, c_i64,
                       c_int, c_vp, c_vp], c_int),
    'fe3d_beamc_m': ([c_i64, c_vp, c_vp, c_vp, c_vp, c_vp, c_i64, c_vp, c_vp, c_vp, c_vp, c_i64, c_int,
                      c_vp, c_vp], c_int),
    'fe3d_quad4_finte': ([c_i64, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_i64, c_vp, c_vp, c_i64, c_vp, c_vp,
                          c_vp], c_int),
    'fe3d_quad4_kg_given_stress': ([c_i64, c_vp, c_vp, c_vp, c_i64, c_vp, c_int, c_vp, c_vp, c_vp, c_int, c_vp,
                                    c_vp, c_vp, c_i64, c_vp, c_vp], c_int),
    'fe3d_tria3r_frame': ([c_i64, c_vp, c_vp, c_i64, c_vp, c_int, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp], c_int),
    'fe3d_tria3r_probe_xe': ([c_i64, c_vp, c_vp, c_i64, c_vp, c_vp, c_vp, c_vp, c_vp], c_int),
    'fe3d_tria3r_probe_ue': ([c_i64, c_vp, c_vp, c_i64, c_vp, c_vp, c_vp, c_vp], c_int),
    'fe3d_tria3r_kc0': ([c_i64, c_vp, c_vp, c_vp, c_i64, c_vp, c_int, c_vp, c_vp, c_vp, c_vp, c_vp, c_i64,
                         c_vp, c_vp, c_int, c_vp, c_int, c_vp, c_vp, c_vp, c_i64, c_int, c_vp, c_vp], c_int),
    'fe3d_quad4r_kc0': ([c_i64, c_vp, c_vp, c_vp, c_i64, c_vp, c_int, c_vp, c_vp, c_vp, c_vp, c_vp, c_i64,
                         c_vp, c_vp, c_int, c_vp, c_int, c_vp, c_vp, c_vp, c_i64, c_int, c_vp, c_vp], c_int),
    'fe3d_tria3r_finte': ([c_i64, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_i64, c_vp, c_vp, c_int, c_vp,
                           c_int, c_vp, c_i64, c_vp, c_vp, c_vp], c_int),
    'fe3d_quad4r_finte': ([c_i64, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_i64, c_vp, c_vp, c_int, c_vp,
                           c_int, c_vp, c_i64, c_vp, c_vp, c_vp], c_int),
    'fe3d_tria3r_kg': ([c_i64, c_vp, c_vp, c_vp, c_i64, c_vp, c_int, c_vp, c_i64, c_vp, c_vp, c_vp, c_vp, c_vp,
                        c_vp, c_i64, c_vp, c_vp, c_vp, c_vp, c_i64, c_int, c_vp, c_vp], c_int),
    'fe3d_tria3r_kg_given_stress': ([c_i64, c_vp, c_vp, c_vp, c_i64, c_vp, c_vp, c_vp, c_vp, c_int, c_vp, c_vp,
                                     c_vp, c_i64, c_int, c_vp, c_vp], c_int),
    'fe3d_tria3r_m': ([c_i64, c_vp, c_vp, c_vp, c_i64, c_vp, c_vp, c_vp, c_i64, c_vp, c_vp, c_vp, c_vp, c_i64,
                       c_int, c_vp, c_vp], c_int),
    'fe3d_beamc_fint': ([c_i64, c_vp, c_vp, c_vp, c_vp, c_vp, c_i64, c_vp, c_vp, c_i64, c_vp, c_vp, c_vp], c_int),
    'fe3d_isotropic_plate_records': ([c_i64, c_vp, c_int, c_vp, c_int, c_vp, c_int, c_vp, c_int, c_vp, c_int,
                                      c_int, c_vp, c_vp], c_int),
    'fe3d_laminate_records': ([c_i64, c_int, c_vp, c_i64, c_vp, c_i64, c_vp, c_i64, c_vp, c_i64, c_vp, c_i64,
                               c_int, c_vp, c_vp], c_int),
    'fe3d_spmm': ([c_vp, c_vp, c_vp, c_vp, c_int, c_vp], c_int),
    'fe3d_solver_precond_multi': ([c_vp, c_vp, c_vp, c_int, c_vp], c_int),
    'fe3d_dense_gram_scratch': ([c_int, c_int], c_i64),
    'fe3d_dense_gram': ([c_i64, c_int, c_int, c_vp, c_vp, c_vp, c_vp, c_vp], c_int),
    'fe3d_dense_gemm_tall': ([c_i64, c_int, c_int, c_vp, c_vp, c_dbl, c_dbl, c_vp, c_vp], c_int),
    'fe3d_quad4_kc0_host': ([c_i64, c_vp, c_vp, c_vp, c_i64, c_vp, c_i64, c_vp, c_vp, c_vp, c_vp, c_i64, c_int,
                             c_i64, c_vp, c_vp], c_int),
    'fe3d_pattern_build': ([c_vp, c_vp, c_i64, c_i64, c_vp, c_vp, c_vp, c_vp], c_int),
    'fe3d_pattern_free': ([c_vp], c_int),
    'fe3d_pattern_info': ([c_vp, c_vp, c_vp, c_vp], c_int),
    'fe3d_pattern_arrays': ([c_vp, c_vp, c_vp, c_vp, c_vp], c_int),
    'fe3d_pattern_copy': ([c_vp, c_vp, c_vp, c_vp, c_vp], c_int),
    'fe3d_assemble': ([c_vp, c_vp, c_vp, c_vp], c_int),
    'fe3d_spmv': ([c_vp, c_vp, c_vp, c_vp, c_vp], c_int),
    'fe3d_solver_create': ([c_vp, c_int, c_vp], c_int),
    'fe3d_solver_setup': ([c_vp, c_vp, c_int, c_vp, c_vp], c_int),
    'fe3d_solver_solve': ([c_vp, c_vp, c_vp, c_vp, c_vp, c_vp], c_int),
    'fe3d_solver_free': ([c_vp], c_int),
    'fe3d_solver_set_blocks': ([c_vp, c_vp, c_vp, c_vp, c_vp], c_int),
    'fe3d_lpc_features': ([c_vp, c_vp, c_vp, c_vp], c_int),
    'fe3d_lpc_features_set': ([c_vp, c_int, c_vp, c_vp, c_vp], c_int),
    'fe3d_lpc_forward': ([c_i64, c_vp, c_vp, c_vp, c_vp, c_vp], c_int),
    'fe3d_lpc_blocks': ([c_vp, c_vp, c_vp, ctypes.c_float, c_vp, c_vp], c_int),
    'fe3d_lpc_apply': ([c_vp, c_vp, c_vp, c_vp], c_int),
    'fe3d_lpc_loss_grad': ([c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, ctypes.c_double, ctypes.c_double,
                            ctypes.c_float, c_int, c_vp, c_vp, c_vp], c_int),
    'fe3d_lpc_backward': ([c_i64, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp], c_int),
    'fe3d_lpc_adam': ([c_i64, c_vp, c_vp, c_vp, c_vp, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                       ctypes.c_float, c_int, c_vp], c_int),
    'fe3d_bsolver_create': ([c_vp, c_int, c_i64, c_vp, c_vp], c_int),
    'fe3d_bsolver_setup': ([c_vp, c_vp, c_int, c_vp, c_vp], c_int),
    'fe3d_bsolver_info': ([c_vp, c_vp, c_vp], c_int),
    'fe3d_bsolver_set_split': ([c_vp, c_i64, c_vp], c_int),
    'fe3d_bsolver_solve': ([c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp], c_int),
    'fe3d_bsolver_free': ([c_vp], c_int),
    'fe3d_pattern_build_elements': ([c_vp, c_int, c_i64, c_vp, c_vp, c_vp, c_vp], c_int),
    'fe3d_fmap_build': ([c_vp, c_vp, c_int, c_vp, c_vp, c_vp], c_int),
    'fe3d_fmap_free': ([c_vp], c_int),
    'fe3d_fmap_info': ([c_vp, c_int, c_vp, c_vp], c_int),
    'fe3d_csr_scatter': ([c_vp, c_int, c_vp, c_vp, c_i64, c_vp, c_int, c_vp, c_vp], c_int),
    'fe3d_quad4_kc0_csr': ([c_vp, c_int, c_vp, c_i64, c_vp, c_int, c_vp, c_i64, c_vp, c_vp, c_int, c_vp, c_vp],
                           c_int),
    'fe3d_noalloc_max_rows': ([], c_i64),
    'fe3d_jacobi_pcg_noalloc': ([c_i64, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp], c_int),
}


class Fe3dError(RuntimeError):
    """Error reported by the CUDA library (negative status or device error word)."""


def declared_symbols():
    return dict(_SIGS)


def load(path=LIB_PATH):
    """Load the shared library (without touching the GPU)."""
    global _lib
    if _lib is None:
        if not os.path.exists(path):
            raise Fe3dError('%s is not built: run `python -m pyfe3d_gb300.build`' % path)
        lib = ctypes.CDLL(path)
        for name, (args, res) in _SIGS.items():
            f = getattr(lib, name)
            f.argtypes = args
            f.restype = res
        _lib = lib
    return _lib


def register(name, args, res=c_int):
    """Declare the signature of an additional entry point."""
    _SIGS[name] = (args, res)
    if _lib is not None:
        f = getattr(_lib, name)
        f.argtypes = args
        f.restype = res


def torch_mod():
    import torch
    return torch


def device():
    """The current CUDA device; raises when no GPU is available."""
    torch = torch_mod()
    if not torch.cuda.is_available():
        raise Fe3dError('pyfe3d_gb300 needs a CUDA device (GB300, sm_103a); none is available')
    return torch.device('cuda', torch.cuda.current_device())


def stream_ptr():
    torch = torch_mod()
    return c_vp(torch.cuda.current_stream().cuda_stream)


def err_word():
    """Per-device int32 error word the kernels OR their error bits into."""
    torch = torch_mod()
    dev = device()
    w = _err_words.get(dev.index)
    if w is None:
        w = torch.zeros(1, dtype=torch.int32, device=dev)
        _err_words[dev.index] = w
    return w


def ptr(t):
    if t is None:
        return None
    return c_vp(t.data_ptr())


_kept = []


def keep(t):
    """Pointer of a temporary device tensor that must outlive the launch it
    is passed to: the tensor is held until the next ``check`` has
    synchronised the stream (otherwise the caching allocator could hand its
    memory to the next temporary before the kernel has run)."""
    _kept.append(t)
    return ptr(t)


def check(rc, what='', err=None):
    """Raise on a negative status; with ``err``, synchronise and check the device word."""
    if _kept:
        torch_mod().cuda.current_stream().synchronize()
        del _kept[:]
    if rc != 0:
        raise Fe3dError('%s: %s (status %d)' % (what, FE3D_ERRORS.get(rc, 'unknown'), rc))
    if err is not None:
        v = int(err.item())
        if v:
            err.zero_()
            raise Fe3dError('%s: device reported error bits 0x%x (an offset outside the '
                            'caller\'s buffers)' % (what, v))


_NP_TO_TORCH = None


def to_device(a, dtype):
    """numpy array or torch tensor -> contiguous CUDA tensor of ``dtype`` (numpy dtype)."""
    torch = torch_mod()
    tdt = {np.float64: torch.float64, np.int64: torch.int64, np.int32: torch.int32,
           np.float32: torch.float32, np.uint8: torch.uint8}[np.dtype(dtype).type]
    dev = device()
    if isinstance(a, torch.Tensor):
        t = a
        if t.dtype != tdt:
            t = t.to(tdt)
        if t.device != dev:
            t = t.to(dev)
        return t.contiguous()
    arr = np.ascontiguousarray(a, dtype=dtype)
    return torch.from_numpy(arr).to(dev)


def is_cuda_tensor(a):
    try:
        torch = torch_mod()
    except ImportError:
        return False
    return isinstance(a, torch.Tensor) and a.is_cuda
