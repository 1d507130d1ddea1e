# Cython declarations of the C ABI (include/fe3d_gb300.h) for Cython callers,
# e.g. a Cython build of pyfe3d calling the GPU path from its own methods.
from libc.stdint cimport int64_t, int32_t, uint8_t

cdef extern from "fe3d_gb300.h" nogil:
    int fe3d_version()
    const char *fe3d_error_string(int code)
    int fe3d_quad4_kc0(int64_t E, const int64_t *cdof, const int64_t *init_k,
                       const double *x, int64_t nx, const double *xmat, int xmat_stride,
                       const double *R, const double *m, const double *xe, const double *area,
                       const double *props, int64_t nprops, const int32_t *pid,
                       int64_t *Kr, int64_t *Kc, double *Kv, int64_t nk, int values_only,
                       int *err, void *stream)
    int fe3d_beamc_kc0(int64_t E, const int64_t *cdof, const int64_t *init_k, const double *R,
                       const double *length, const double *props, int64_t nprops, const int32_t *pid,
                       int64_t *Kr, int64_t *Kc, double *Kv, int64_t nk, int values_only, int *err,
                       void *stream)
