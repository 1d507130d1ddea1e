"""Per-element call plumbing shared by the Quad4 and BeamC classes.

A per-element method moves the element's few inputs to the GPU, runs the
batched kernel with E = 1 and copies the touched slots back.  When the
caller's COO arrays are CUDA tensors the kernel writes into them in place.
"""
import numpy as np

from . import _lib


def gather(arr, idx):
    """arr[idx] for a numpy array or a torch tensor (data movement only)."""
    if _lib.is_cuda_tensor(arr):
        torch = _lib.torch_mod()
        return arr[torch.as_tensor(idx, device=arr.device)]
    return np.asarray(arr)[idx]


def dev(a, dtype=np.float64):
    return _lib.to_device(a, dtype)


def host(t):
    return t.detach().cpu().numpy()


class CooTarget:
    """The [k0, k0+size) window of the caller's (r, c, v) arrays on the device."""

    def __init__(self, Kr, Kc, Kv, k0, size, write_idx):
        self.Kr, self.Kc, self.Kv = Kr, Kc, Kv
        self.k0, self.size, self.write_idx = int(k0), int(size), write_idx
        n = len(Kv)
        if self.k0 < 0 or self.k0 + self.size > n:
            raise IndexError('sparse slots [%d, %d) outside the value array of length %d'
                             % (self.k0, self.k0 + self.size, n))
        if write_idx and (len(Kr) < self.k0 + self.size or len(Kc) < self.k0 + self.size):
            raise IndexError('row/column arrays shorter than the value array window')
        self.inplace = (_lib.is_cuda_tensor(Kv) and (not write_idx or
                        (_lib.is_cuda_tensor(Kr) and _lib.is_cuda_tensor(Kc))))
        torch = _lib.torch_mod()
        if self.inplace:
            # values-only updates never write the index arrays: only Kv is checked then
            checked = ((Kv, torch.float64), (Kr, torch.int64), (Kc, torch.int64)) if write_idx \
                else ((Kv, torch.float64),)
            for t, dt in checked:
                if t is not None and (t.dtype != dt or not t.is_contiguous()):
                    raise TypeError('COO tensors must be contiguous int64/float64 CUDA tensors')
            self.r, self.c, self.v = Kr, Kc, Kv
            if not write_idx:
                # the kernels take null index arrays in values-only mode
                self.r = Kr if _lib.is_cuda_tensor(Kr) else None
                self.c = Kc if _lib.is_cuda_tensor(Kc) else None
            self.init_k = dev(np.array([self.k0], dtype=np.int64), np.int64)
            self.nk = n
        else:
            s = slice(self.k0, self.k0 + self.size)
            if not (isinstance(Kv, np.ndarray) and Kv.dtype == np.float64):
                raise TypeError('KC0v/KGv/Mv must be float64 arrays')
            self.v = dev(Kv[s])
            self.r = dev(np.zeros(self.size, np.int64), np.int64)
            self.c = dev(np.zeros(self.size, np.int64), np.int64)
            self.init_k = dev(np.zeros(1, np.int64), np.int64)
            self.nk = self.size

    def finish(self, touched=None):
        if self.inplace:
            return
        n = self.size if touched is None else touched
        s = slice(self.k0, self.k0 + n)
        self.Kv[s] = host(self.v)[:n]
        if self.write_idx:
            self.Kr[s] = host(self.r)[:n]
            self.Kc[s] = host(self.c)[:n]
