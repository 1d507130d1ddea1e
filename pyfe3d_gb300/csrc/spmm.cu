// Block kernels of the device eigensolver (LOBPCG) that stands in for the
// reference tests' `eigsh(A=K, M=M, sigma=..)` calls
// (tests/test_quad4_natural_freq.py:117-120,
// tests/test_quad4_linear_buckling_plate_rotated.py:129-131):
//   Y = A X  for a row-major n x k block X (CSR A, k <= 16), LPR lanes per
//            row, every lane carrying k partial sums;
//   Z = Dinv R  the 6x6 nodal block-Jacobi inverses of a solver applied to
//            every column of a block;
//   G = X^T Y  the Rayleigh-Ritz projections of tall-skinny row-major blocks
//            (k1, k2 <= 64): per block of the grid a partial product over a
//            contiguous range of rows (staged in shared memory), then the
//            partials summed in a fixed order (deterministic);
//   Y = beta Y + alpha X T  a tall-skinny block times a small k x m matrix.
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

constexpr int GRAM_PARTS = 2 * kSMs;  // blocks of the partial Gram products
constexpr int GRAM_MAXK = 64;
constexpr int GRAM_ROWS = 32;  // rows staged per tile

__global__ void __launch_bounds__(SPMM_BS) gram_partial_kernel(int64_t n, int k1, int k2,
                                                               const double *__restrict__ X,
                                                               const double *__restrict__ Y,
                                                               double *__restrict__ part) {
    __shared__ double xs[GRAM_ROWS][GRAM_MAXK];
    __shared__ double ys[GRAM_ROWS][GRAM_MAXK];
    const int np = k1 * k2;  // output entries, at most 4096: 16 per thread
    double acc[GRAM_MAXK * GRAM_MAXK / SPMM_BS];
#pragma unroll
    for (int q = 0; q < GRAM_MAXK * GRAM_MAXK / SPMM_BS; q++) acc[q] = 0.;
    const int64_t per = (n + gridDim.x - 1) / gridDim.x;
    const int64_t r0 = blockIdx.x * per, r1 = r0 + per < n ? r0 + per : n;
    for (int64_t t0 = r0; t0 < r1; t0 += GRAM_ROWS) {
        const int rows = (int)(r1 - t0 < GRAM_ROWS ? r1 - t0 : GRAM_ROWS);
        __syncthreads();
        for (int i = threadIdx.x; i < rows * k1; i += blockDim.x) xs[i / k1][i % k1] = X[(t0 + i / k1) * k1 + i % k1];
        for (int i = threadIdx.x; i < rows * k2; i += blockDim.x) ys[i / k2][i % k2] = Y[(t0 + i / k2) * k2 + i % k2];
        __syncthreads();
#pragma unroll
        for (int q = 0; q < GRAM_MAXK * GRAM_MAXK / SPMM_BS; q++) {
            const int e = threadIdx.x + q * SPMM_BS;
            if (e < np) {
                const int a = e / k2, b = e - a * k2;
                double v = acc[q];
                for (int r = 0; r < rows; r++) v += xs[r][a] * ys[r][b];
                acc[q] = v;
            }
        }
    }
#pragma unroll
    for (int q = 0; q < GRAM_MAXK * GRAM_MAXK / SPMM_BS; q++) {
        const int e = threadIdx.x + q * SPMM_BS;
        if (e < np) part[(int64_t)blockIdx.x * np + e] = acc[q];
    }
}

__global__ void gram_sum_kernel(int nparts, int np, const double *__restrict__ part, double *__restrict__ G) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= np) return;
    double v = 0.;
    for (int b = 0; b < nparts; b++) v += part[(int64_t)b * np + e];
    G[e] = v;
}

__global__ void __launch_bounds__(SPMM_BS) gemm_tall_kernel(int64_t n, int k, int m, const double *__restrict__ X,
                                                            const double *__restrict__ T, double alpha,
                                                            double beta, double *__restrict__ Y) {
    __shared__ double ts[GRAM_MAXK * GRAM_MAXK];
    for (int i = threadIdx.x; i < k * m; i += blockDim.x) ts[i] = T[i];
    __syncthreads();
    const int64_t total = n * m;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = e / m;
        const int c = (int)(e - r * m);
        const double *x = X + r * k;
        double v = 0.;
        for (int j = 0; j < k; j++) v += x[j] * ts[j * m + c];
        Y[e] = beta == 0. ? alpha * v : beta * Y[e] + alpha * v;
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

extern "C" int64_t fe3d_dense_gram_scratch(int k1, int k2) { return (int64_t)GRAM_PARTS * k1 * k2; }

extern "C" int fe3d_dense_gram(int64_t n, int k1, int k2, const double *X, const double *Y, double *G,
                               double *scratch, void *stream) {
    if (n < 0 || k1 < 1 || k2 < 1 || k1 > GRAM_MAXK || k2 > GRAM_MAXK || !G || !scratch ||
        (n > 0 && (!X || !Y)))
        return FE3D_ERR_ARG;
    cudaStream_t st = as_stream(stream);
    gram_partial_kernel<<<GRAM_PARTS, SPMM_BS, 0, st>>>(n, k1, k2, X, Y, scratch);
    const int np = k1 * k2;
    gram_sum_kernel<<<(np + 255) / 256, 256, 0, st>>>(GRAM_PARTS, np, scratch, G);
    FE3D_CHECK_LAUNCH();
    return FE3D_OK;
}

extern "C" int fe3d_dense_gemm_tall(int64_t n, int k, int m, const double *X, const double *T, double alpha,
                                    double beta, double *Y, void *stream) {
    if (n < 0 || k < 1 || m < 1 || k > GRAM_MAXK || m > GRAM_MAXK || !T || (n > 0 && (!X || !Y))) return FE3D_ERR_ARG;
    if (n == 0) return FE3D_OK;
    const int64_t blocks = (n * m + SPMM_BS - 1) / SPMM_BS;
    const unsigned grid = (unsigned)(blocks < kSMs * 8 ? blocks : kSMs * 8);
    gemm_tall_kernel<<<grid, SPMM_BS, 0, as_stream(stream)>>>(n, k, m, X, T, alpha, beta, Y);
    FE3D_CHECK_LAUNCH();
    return FE3D_OK;
}
