# cython: language_level=3
"""Cython binding of the C ABI (compiled module ``pyfe3d_gb300.fe3d_cy``).

The reference is Cython; its methods would reach this library through a
``cdef extern`` block like ``fe3d_gb300.pxd`` next to this file.  This module
is that binding, compiled: it calls the entry points with the GIL released
and takes device pointers as integers (``tensor.data_ptr()``), so Cython and
Python callers share one path with the ctypes layer.
"""
from libc.stdint cimport int64_t, int32_t, uintptr_t

from fe3d_gb300 cimport fe3d_version, fe3d_error_string, fe3d_quad4_kc0, fe3d_beamc_kc0


def version():
    return fe3d_version()


def error_string(int code):
    return fe3d_error_string(code).decode()


def quad4_kc0(int64_t E, uintptr_t cdof, uintptr_t init_k, uintptr_t x, int64_t nx,
              uintptr_t props, int64_t nprops, uintptr_t pid, uintptr_t Kr, uintptr_t Kc,
              uintptr_t Kv, int64_t nk, int values_only, uintptr_t err, uintptr_t stream):
    """Quad4.update_KC0 over E elements (pyfe3d/quad4.pyx:1204-1313), frames
    from the coordinates x, device pointers as integers; returns the status."""
    cdef int rc
    with nogil:
        rc = fe3d_quad4_kc0(E, <const int64_t *>cdof, <const int64_t *>init_k, <const double *>x, nx,
                            NULL, 0, NULL, NULL, NULL, NULL, <const double *>props, nprops,
                            <const int32_t *>pid, <int64_t *>Kr, <int64_t *>Kc, <double *>Kv, nk,
                            values_only, <int *>err, <void *>stream)
    return rc


def beamc_kc0(int64_t E, uintptr_t cdof, uintptr_t init_k, uintptr_t R, uintptr_t length, uintptr_t props,
              int64_t nprops, uintptr_t pid, uintptr_t Kr, uintptr_t Kc, uintptr_t Kv, int64_t nk,
              int values_only, uintptr_t err, uintptr_t stream):
    """BeamC.update_KC0 over E elements (pyfe3d/beamc.pyx:489-1352) from their
    frames R and lengths; returns the status."""
    cdef int rc
    with nogil:
        rc = fe3d_beamc_kc0(E, <const int64_t *>cdof, <const int64_t *>init_k, <const double *>R,
                            <const double *>length, <const double *>props, nprops, <const int32_t *>pid,
                            <int64_t *>Kr, <int64_t *>Kc, <double *>Kv, nk, values_only, <int *>err,
                            <void *>stream)
    return rc
