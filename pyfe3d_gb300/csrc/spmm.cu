// Block kernels of the device eigensolver (LOBPCG) that stands in for the
// reference tests' `eigsh(A=K, M=M, sigma=..)` calls
// (tests/test_quad4_natural_freq.py:117-120,
// tests/test_quad4_linear_buckling_plate_rotated.py:129-131):
//   Y = A X  for a row-major n x k block X (CSR A, k <= 16), LPR lanes per
//            row, every lane carrying k partial sums;
//   Z = Dinv R  the 6x6 nodal block-Jacobi inverses of a solver applied to
//            every column of a block.
#include "common.cuh"
#include "fe3d_internal.h"

namespace fe3d {
namespace {

constexpr int SPMM_BS = 256;

template <int K, int LPR>
__global__ void __launch_bounds__(SPMM_BS) spmm_kernel(int64_t n, const int64_t *__restrict__ rowptr,
                                                       const int32_t *__restrict__ colind,
                                                       const double *__restrict__ vals,
                                                       const double *__restrict__ X, double *__restrict__ Y,
                                                       int k) {
    const int lane = threadIdx.x % LPR;
    const int64_t group = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) / LPR;
    const int64_t ngroups = (int64_t)gridDim.x * blockDim.x / LPR;
    const int64_t trips = (n + ngroups - 1) / ngroups;  // uniform: full-warp shuffles below
    for (int64_t t = 0; t < trips; t++) {
        const int64_t row = group + t * ngroups;
        const bool in = row < n;
        double acc[K];
#pragma unroll
        for (int j = 0; j < K; j++) acc[j] = 0.;
        if (in)
            for (int64_t p = rowptr[row] + lane; p < rowptr[row + 1]; p += LPR) {
                const double a = vals[p];
                const double *x = X + (int64_t)k * colind[p];
#pragma unroll
                for (int j = 0; j < K; j++)
                    if (j < k) acc[j] += a * x[j];
            }
#pragma unroll
        for (int j = 0; j < K; j++)
#pragma unroll
            for (int o = LPR / 2; o > 0; o >>= 1) acc[j] += __shfl_xor_sync(0xffffffffu, acc[j], o);
        if (in && lane == 0)
#pragma unroll
            for (int j = 0; j < K; j++)
                if (j < k) Y[(int64_t)k * row + j] = acc[j];
    }
}

// Z[:, j] = Dinv R[:, j] node by node (row-major n x k blocks).
__global__ void bjacobi_multi_kernel(int64_t nnodes, const int32_t *start, const int8_t *size, const double *Dinv,
                                     const double *R, double *Z, int k) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= nnodes * k) return;
    const int64_t j = t / k;
    const int col = (int)(t - j * k);
    const int s = start[j], b = size[j];
    double r[6];
    for (int i = 0; i < 6; i++) r[i] = i < b ? R[(int64_t)k * (s + i) + col] : 0.;
    for (int i = 0; i < b; i++) {
        double a = 0.;
        for (int q = 0; q < 6; q++) a += Dinv[36 * j + 6 * i + q] * r[q];
        Z[(int64_t)k * (s + i) + col] = a;
    }
}

}  // namespace
}  // namespace fe3d

using namespace fe3d;

extern "C" int fe3d_spmm(const fe3d_pattern *p, const double *vals, const double *X, double *Y, int k,
                         void *stream) {
    if (!p || k < 1 || k > 16 || (p->nrows > 0 && (!vals || !X || !Y))) return FE3D_ERR_ARG;
    if (p->nrows == 0) return FE3D_OK;
    constexpr int LPR = 4;
    int64_t g = (p->nrows * LPR + SPMM_BS - 1) / SPMM_BS;
    if (g > kSMs * 8) g = kSMs * 8;
    cudaStream_t st = as_stream(stream);
    if (k <= 4)
        spmm_kernel<4, LPR><<<(int)g, SPMM_BS, 0, st>>>(p->nrows, p->rowptr, p->colind, vals, X, Y, k);
    else if (k <= 8)
        spmm_kernel<8, LPR><<<(int)g, SPMM_BS, 0, st>>>(p->nrows, p->rowptr, p->colind, vals, X, Y, k);
    else
        spmm_kernel<16, LPR><<<(int)g, SPMM_BS, 0, st>>>(p->nrows, p->rowptr, p->colind, vals, X, Y, k);
    FE3D_CHECK_LAUNCH();
    return FE3D_OK;
}

extern "C" int fe3d_solver_precond_multi(const fe3d_solver *s, const double *R, double *Z, int k, void *stream) {
    if (!s || k < 1 || (s->n > 0 && (!R || !Z))) return FE3D_ERR_ARG;
    if (!s->ready) return FE3D_ERR_STATE;
    if (s->nnodes == 0) return FE3D_OK;
    const int64_t work = s->nnodes * k;
    bjacobi_multi_kernel<<<(unsigned)((work + 255) / 256), 256, 0, as_stream(stream)>>>(s->nnodes, s->start, s->size,
                                                                                       s->Dinv, R, Z, k);
    FE3D_CHECK_LAUNCH();
    return FE3D_OK;
}
