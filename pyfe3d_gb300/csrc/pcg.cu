// Preconditioned conjugate gradients on the reduced CSR system, standing in
// for the reference tests' `spsolve(Kuu, fu)` / `cg(Kuu, fu)`
// (tests/test_beamc_static_point_load.py:109, tests/test_quad4_static_point_load.py:102).
//
// Preconditioner: 6x6 nodal block Jacobi (the diagonal block of each node's
// free DOFs, inverted through its Cholesky factor in FP64).
//
// Iteration (3 launches, deterministic reductions):
//   K1  q = K p                          partial sums of p.q per block
//   K2  alpha = rz / p.q;  u += alpha p;  r -= alpha q;  z = Minv r
//                                        partial sums of r.z and r.r
//   K3  beta = rz_new / rz;  p = z + beta p
// Every block of a consumer kernel reduces the producer's per-block partial
// sums in the same order, so all blocks see identical scalars and the result
// does not depend on scheduling.
//
// The solution is held as a double-double base plus an FP64 increment that
// the iterations update; the residual r = f - K x is evaluated from the base
// with compensated (double-double) row sums whenever the recurrence residual
// is replaced, so the attainable residual is not limited by FP64 rounding of
// K x (which reaches ~1e-7 of ||f|| on the 1001 x 1001-node clamped plate).
// The caller receives the base rounded to FP64.
//
// precision 0: everything FP64 (the drop-in plain form).
// precision 1: the Krylov recurrence runs on the symmetrically scaled system
//   S^-1 K S^-1 (S = sqrt(diag K), so every FP32 row has unit diagonal and the
//   membrane, bending and drilling rows share one scale) with FP32 values and
//   block inverses (FP32 products and accumulation), while u, r and all
//   scalars stay FP64; every `replace_every` iterations the true residual
//   replaces the recurrence residual (reliable updates), and convergence is
//   decided on that residual only.
#include "common.cuh"
#include "fe3d_internal.h"

namespace fe3d {
namespace {

constexpr int RED_BS = 256;
constexpr int LANES_PER_ROW = 4;  // compensated residual kernel (FP64-pipe bound)

__device__ __forceinline__ double block_sum(double v, double *sh) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) sh[w] = v;
    __syncthreads();
    double s = 0.;
    if (threadIdx.x < 32) {
        s = (l < (int)(blockDim.x >> 5)) ? sh[l] : 0.;
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    }
    return s;  // valid in thread 0
}

// Sum of partials[0..n) in a fixed order, broadcast to the whole block.
__device__ __forceinline__ double reduce_partials(const double *partials, int n, double *sh) {
    double v = 0.;
    for (int i = threadIdx.x; i < n; i += blockDim.x) v += partials[i];
    // fixed-shape tree: identical in every block
    v = block_sum(v, sh);
    __syncthreads();
    if (threadIdx.x == 0) sh[32] = v;
    __syncthreads();
    return sh[32];
}

// Fixed-order sum of per-block partials read through L2 (written by other
// blocks of the same launch), broadcast to the block.
__device__ __forceinline__ double reduce_partials_l2(const double *partials, int n, double *sh) {
    double v = 0.;
    for (int i = threadIdx.x; i < n; i += blockDim.x) v += __ldcg(partials + i);
    v = block_sum(v, sh);
    __syncthreads();
    if (threadIdx.x == 0) sh[32] = v;
    __syncthreads();
    return sh[32];
}

// True in the block that finishes last (its partials are the last written).
// Thread 0 of every block must have stored its partials before the call.
__device__ __forceinline__ bool last_block(unsigned int *counter) {
    __shared__ bool am_last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) am_last = atomicAdd(counter, 1u) == gridDim.x - 1;
    __syncthreads();
    return am_last;
}

// y = K x over CSR rows, LPR lanes per row.  With partial_dot: per-block
// sums of x.y, and the last block to finish reduces them in a fixed order
// into alpha = rz / (x.y) (0 when x.y = 0) and resets the counter.
template <typename VT, typename XT, int LPR, bool C16>
__global__ void __launch_bounds__(RED_BS) spmv_kernel(int64_t n, const int64_t *__restrict__ rowptr,
                                                      const int32_t *__restrict__ colind,
                                                      const int32_t *__restrict__ colbase,
                                                      const uint16_t *__restrict__ col16,
                                                      const VT *__restrict__ vals,
                                                      const XT *__restrict__ x, XT *__restrict__ y,
                                                      double *partial_dot, unsigned int *counter,
                                                      const double *rz, double *alpha_out) {
    __shared__ double sh[34];
    const int lane = threadIdx.x % LPR;
    const int64_t group = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) / LPR;
    const int64_t ngroups = (int64_t)gridDim.x * blockDim.x / LPR;
    double dot = 0.;
    // every lane runs the same number of trips: the full-warp shuffles below
    // must never wait for lanes that have left the loop
    const int64_t trips = (n + ngroups - 1) / ngroups;
    for (int64_t t = 0; t < trips; t++) {
        const int64_t row = group + t * ngroups;
        const bool in = row < n;
        VT acc = 0;
        if (in) {
            const int32_t base = C16 ? colbase[row] : 0;
            for (int64_t k = rowptr[row] + lane; k < rowptr[row + 1]; k += LPR)
                acc += vals[k] * (VT)x[C16 ? base + (int32_t)col16[k] : colind[k]];
        }
#pragma unroll
        for (int o = LPR / 2; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (in && lane == 0) {
            y[row] = (XT)acc;
            dot += (double)x[row] * (double)acc;
        }
    }
    if (partial_dot) {
        const double s = block_sum(dot, sh);
        if (threadIdx.x == 0) partial_dot[blockIdx.x] = s;
        if (last_block(counter)) {
            const double pq = reduce_partials_l2(partial_dot, gridDim.x, sh);
            if (threadIdx.x == 0) {
                *alpha_out = pq != 0. ? *rz / pq : 0.;
                *counter = 0u;
            }
        }
    }
}

// y = K x with the products on the FP32 pipe: values and x are held as
// float pairs (hi + lo, ~48 significant bits), each product is split exactly
// with an FMA plus the two cross terms, and the row sums are carried in
// float-float (TwoSum); y is rounded to FP64 once per row.  The FP64 pipe,
// which bounds the FP64 SpMV on GB300, is left with one conversion per row,
// so the kernel runs at the HBM bound (8 bytes per value as in FP64).
// Otherwise as spmv_kernel (p.q partials, alpha by the last block).
#ifndef FE3D_SPLIT_UNROLL
#define FE3D_SPLIT_UNROLL 2
#endif
constexpr int SPLIT_U = FE3D_SPLIT_UNROLL;

template <int LPR, bool C16>
__global__ void __launch_bounds__(RED_BS) spmv_split_kernel(int64_t n, const int64_t *__restrict__ rowptr,
                                                            const int32_t *__restrict__ colind,
                                                            const int32_t *__restrict__ colbase,
                                                            const uint16_t *__restrict__ col16,
                                                            const float2 *__restrict__ vals,
                                                            const float2 *__restrict__ x2,
                                                            const double *__restrict__ x, double *__restrict__ y,
                                                            double *partial_dot, unsigned int *counter,
                                                            const double *rz, double *alpha_out) {
    __shared__ double sh[34];
    const int lane = threadIdx.x % LPR;
    const int64_t group = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) / LPR;
    const int64_t ngroups = (int64_t)gridDim.x * blockDim.x / LPR;
    double dot = 0.;
    const int64_t trips = (n + ngroups - 1) / ngroups;  // uniform: full-warp shuffles below
    for (int64_t t = 0; t < trips; t++) {
        const int64_t row = group + t * ngroups;
        const bool in = row < n;
        float hi = 0.f, lo = 0.f;
        const int32_t base = (C16 && in) ? colbase[row] : 0;
        if (in) {
            // SPLIT_U entries per lane per trip, their loads issued before the
            // float-float sums (entries past the row end are zeros, which leave
            // hi and lo unchanged)
            const int64_t ke = rowptr[row + 1];
            for (int64_t k = rowptr[row] + lane; k < ke; k += SPLIT_U * LPR) {
                float2 a[SPLIT_U], b[SPLIT_U];
#pragma unroll
                for (int t = 0; t < SPLIT_U; t++) {
                    const int64_t kt = k + t * LPR;
                    const bool ok = t == 0 || kt < ke;
                    a[t] = ok ? vals[kt] : make_float2(0.f, 0.f);
                    b[t] = ok ? x2[C16 ? base + (int32_t)col16[kt] : colind[kt]] : make_float2(0.f, 0.f);
                }
#pragma unroll
                for (int t = 0; t < SPLIT_U; t++) {
                    const float ph = a[t].x * b[t].x;
                    const float pe = fmaf(a[t].x, b[t].x, -ph);
                    const float pc = fmaf(a[t].x, b[t].y, a[t].y * b[t].x);
                    const float sm = hi + ph;
                    const float bb = sm - hi;
                    const float er = (hi - (sm - bb)) + (ph - bb);
                    hi = sm;
                    lo += er + (pe + pc);
                }
            }
        }
#pragma unroll
        for (int o = LPR / 2; o > 0; o >>= 1) {
            const float oh = __shfl_xor_sync(0xffffffffu, hi, o);
            const float ol = __shfl_xor_sync(0xffffffffu, lo, o);
            const float sm = hi + oh;
            const float bb = sm - hi;
            const float er = (hi - (sm - bb)) + (oh - bb);
            hi = sm;
            lo += ol + er;
        }
        if (in && lane == 0) {
            const double v = (double)hi + (double)lo;
            y[row] = v;
            dot += x[row] * v;
        }
    }
    if (partial_dot) {
        const double s = block_sum(dot, sh);
        if (threadIdx.x == 0) partial_dot[blockIdx.x] = s;
        if (last_block(counter)) {
            const double pq = reduce_partials_l2(partial_dot, gridDim.x, sh);
            if (threadIdx.x == 0) {
                *alpha_out = pq != 0. ? *rz / pq : 0.;
                *counter = 0u;
            }
        }
    }
}

__device__ __forceinline__ float2 split_double(double v) {
    const float h = (float)v;
    return make_float2(h, (float)(v - (double)h));
}

__global__ void split_kernel(int64_t n, const double *a, float2 *b) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        b[i] = split_double(a[i]);
}

// Node blocks: rows [start, start + size) of the reduced system.
// Dinv: 36 entries per node (row-major, padded with zeros beyond size).

// Inverse of the symmetric b x b block A through its Cholesky factor, into
// D (36, zero padded).  Returns false, leaving D untouched, when A is not
// positive definite.
__device__ bool chol_inverse(const double (&A)[6][6], int b, double (&D)[36]) {
    double L[6][6];
    for (int i = 0; i < 6; i++)
        for (int k = 0; k < 6; k++) L[i][k] = 0.;
    for (int i = 0; i < b; i++) {
        for (int k = 0; k <= i; k++) {
            double sum = A[i][k];
            for (int m = 0; m < k; m++) sum -= L[i][m] * L[k][m];
            if (i == k) {
                if (!(sum > 0.)) return false;
                L[i][i] = sqrt(sum);
            } else {
                L[i][k] = sum / L[k][k];
            }
        }
    }
    double Li[6][6];  // L^-1
    for (int i = 0; i < 6; i++)
        for (int k = 0; k < 6; k++) Li[i][k] = 0.;
    for (int i = 0; i < b; i++) {
        Li[i][i] = 1. / L[i][i];
        for (int k = 0; k < i; k++) {
            double sum = 0.;
            for (int m = k; m < i; m++) sum -= L[i][m] * Li[m][k];
            Li[i][k] = sum / L[i][i];
        }
    }
    for (int i = 0; i < 6; i++)
        for (int k = 0; k < 6; k++) {
            double v = 0.;
            if (i < b && k < b)
                for (int m = (i > k ? i : k); m < b; m++) v += Li[m][i] * Li[m][k];
            D[6 * i + k] = v;
        }
    return true;
}

__device__ void gather_diag_block(int s, int b, const int64_t *rowptr, const int32_t *colind,
                                  const double *vals, double (&A)[6][6]) {
    for (int i = 0; i < 6; i++)
        for (int k = 0; k < 6; k++) A[i][k] = 0.;
    for (int i = 0; i < b; i++) {
        const int64_t rb = rowptr[s + i], re = rowptr[s + i + 1];
        for (int64_t k = rb; k < re; k++) {
            const int c = colind[k] - s;
            if (c >= 0 && c < b) A[i][c] = vals[k];
        }
    }
}

// Block-Jacobi inverse of node j's diagonal block; a block that is not
// positive definite falls back to the scalar Jacobi inverse (counted).
__device__ void bjacobi_node(int64_t j, int s, int b, const int64_t *rowptr, const int32_t *colind,
                             const double *vals, double (&D)[36], int *nonpos) {
    double A[6][6];
    gather_diag_block(s, b, rowptr, colind, vals, A);
    if (!chol_inverse(A, b, D)) {
        atomicAdd(nonpos, 1);
        for (int i = 0; i < 36; i++) D[i] = 0.;
        for (int i = 0; i < b; i++) D[7 * i] = A[i][i] != 0. ? 1. / A[i][i] : 0.;
    }
}

// Row scales sc = sqrt(K_ii) of the node's rows (1 where not positive) and
// the FP32 block inverse of the scaled system S^-1 K S^-1: S Dinv S.
__device__ void store_inverses(int64_t j, int s, int b, const int64_t *rowptr, const int32_t *colind,
                               const double *vals, const double (&D)[36], double *Dinv, float *Dinv32,
                               double *sc, int64_t n_rows) {
    double sv[6];
    for (int i = 0; i < 6; i++) sv[i] = 1.;
    for (int i = 0; i < b; i++) {
        double d = 0.;
        for (int64_t k = rowptr[s + i]; k < rowptr[s + i + 1]; k++)
            if (colind[k] == s + i) d = vals[k];
        sv[i] = d > 0. ? sqrt(d) : 1.;
        sc[s + i] = sv[i];
        sc[n_rows + s + i] = 1. / sv[i];  // inverse scales follow the scales
    }
    for (int i = 0; i < 6; i++)
        for (int k = 0; k < 6; k++) {
            Dinv[36 * j + 6 * i + k] = D[6 * i + k];
            Dinv32[36 * j + 6 * i + k] = (float)(sv[i] * D[6 * i + k] * sv[k]);
        }
}

__global__ void bjacobi_setup_kernel(int64_t nnodes, const int32_t *start, const int8_t *size,
                                     const int64_t *rowptr, const int32_t *colind,
                                     const double *vals, double *Dinv, float *Dinv32, double *sc,
                                     int64_t n_rows, int *nonpos) {
    const int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (j >= nnodes) return;
    double D[36];
    bjacobi_node(j, start[j], size[j], rowptr, colind, vals, D, nonpos);
    store_inverses(j, start[j], size[j], rowptr, colind, vals, D, Dinv, Dinv32, sc, n_rows);
}

// Caller-given blocks (36 per node over the free DOFs): inverted when
// positive definite, else the block-Jacobi inverse of the diagonal block.
__global__ void blocks_setup_kernel(int64_t nnodes, const int32_t *start, const int8_t *size,
                                    const int64_t *rowptr, const int32_t *colind, const double *vals,
                                    const double *blocks, double *Dinv, float *Dinv32, double *sc,
                                    int64_t n_rows, int8_t *fallback, int *nfallback, int *nonpos) {
    const int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (j >= nnodes) return;
    const int s = start[j], b = size[j];
    double A[6][6], D[36];
    for (int i = 0; i < 6; i++)
        for (int k = 0; k < 6; k++) A[i][k] = (i < b && k < b) ? blocks[36 * j + 6 * i + k] : 0.;
    const bool ok = chol_inverse(A, b, D);
    if (!ok) {
        atomicAdd(nfallback, 1);
        bjacobi_node(j, s, b, rowptr, colind, vals, D, nonpos);
    }
    if (fallback) fallback[j] = ok ? 0 : 1;
    store_inverses(j, s, b, rowptr, colind, vals, D, Dinv, Dinv32, sc, n_rows);
}

// FP32 values of the scaled matrix S^-1 K S^-1 (row per thread).
__global__ void cast_scaled_kernel(int64_t n, const int64_t *rowptr, const int32_t *colind, const double *vals,
                                   const double *sc, float *vals32) {
    const int64_t row = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (row >= n) return;
    const double sr = sc[row];
    for (int64_t k = rowptr[row]; k < rowptr[row + 1]; k++) vals32[k] = (float)(vals[k] / (sr * sc[colind[k]]));
}

// z = Minv r for all nodes, with partial r.z and r.r (no update).
// With sc (the FP32 recurrence of the scaled system): z~ = (S Dinv S) (r / sc).
template <typename ZT, typename DT>
__global__ void __launch_bounds__(RED_BS) precond_kernel(int64_t nnodes, const int32_t *start,
                                                         const int8_t *size, const DT *Dinv,
                                                         const double *r, ZT *z, double *prz,
                                                         double *prr, const double *sc, const double *isc) {
    __shared__ double sh[33];
    double rz = 0., rr = 0.;
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < nnodes;
         j += (int64_t)gridDim.x * blockDim.x) {
        const int s = start[j], b = size[j];
        double rl[6], rs[6];
#pragma unroll
        for (int i = 0; i < 6; i++) {
            rl[i] = i < b ? r[s + i] : 0.;
            rs[i] = (i < b && sc) ? rl[i] * isc[s + i] : rl[i];
        }
        const DT *D = Dinv + 36 * j;
        // static indices (unrolled, predicated on the block size): registers
#pragma unroll
        for (int i = 0; i < 6; i++) {
            if (i < b) {
                DT acc = 0;
#pragma unroll
                for (int k = 0; k < 6; k++) acc += D[6 * i + k] * (DT)rs[k];
                z[s + i] = (ZT)acc;
                rz += rs[i] * (double)acc;
                rr += rl[i] * rl[i];
            }
        }
    }
    double s1 = block_sum(rz, sh);
    __syncthreads();
    if (threadIdx.x == 0) prz[blockIdx.x] = s1;
    double s2 = block_sum(rr, sh);
    if (threadIdx.x == 0) prr[blockIdx.x] = s2;
}

// K2: alpha = rz / pq; u += alpha p; r -= alpha q; z = Minv r; partial rz, rr.
template <typename PT, typename DT>
__global__ void __launch_bounds__(RED_BS) update_kernel(int64_t nnodes, const int32_t *start,
                                                        const int8_t *size, const DT *Dinv,
                                                        const double *alpha_in, const double *rz_cur,
                                                        const PT *p, const PT *q, double *u, double *r, PT *z,
                                                        double *prz, double *prr, double *prf, const double *sc,
                                                        const double *isc, unsigned int *counter, double *rz_new, double *rr_out,
                                                        double *beta_out) {
    __shared__ double sh[34];
    // alpha = rz / p.q from the SpMV's last block (0 when p.q = 0: r = 0 met
    // between host checks leaves the iterate unchanged)
    const double alpha = *alpha_in;
    double rz = 0., rr = 0., rzo = 0.;
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < nnodes;
         j += (int64_t)gridDim.x * blockDim.x) {
        const int s = start[j], b = size[j];
        // rl: the FP64 residual; rs: the residual of the system the
        // recurrence runs on (r / sc when scaled: p~ = sc p, q~ = K p / sc)
        double rl[6], rs[6];
        for (int i = 0; i < 6; i++) {
            if (i < b) {
                double pi = (double)p[s + i], qi = (double)q[s + i];
                const double iv = sc ? isc[s + i] : 1.;
                if (sc) {
                    pi *= iv;
                    qi *= sc[s + i];
                }
                u[s + i] += alpha * pi;
                const double ri = r[s + i] - alpha * qi;
                r[s + i] = ri;
                rl[i] = ri;
                rs[i] = sc ? ri * iv : ri;
            } else {
                rl[i] = 0.;
                rs[i] = 0.;
            }
        }
        const DT *D = Dinv + 36 * j;
        // flexible CG: the previous z, all six loads issued before any store
        double zo[6];
        if (prf) {
#pragma unroll
            for (int i = 0; i < 6; i++) zo[i] = i < b ? (double)z[s + i] : 0.;
        }
        // static indices throughout (unrolled, predicated on the block
        // size): rl, rs and zo stay in registers
#pragma unroll
        for (int i = 0; i < 6; i++) {
            if (i < b) {
                DT acc = 0;
#pragma unroll
                for (int k = 0; k < 6; k++) acc += D[6 * i + k] * (DT)rs[k];
                if (prf) rzo += rs[i] * zo[i];
                z[s + i] = (PT)acc;
                rz += rs[i] * (double)acc;
                rr += rl[i] * rl[i];
            }
        }
    }
    __syncthreads();
    double s1 = block_sum(rz, sh);
    __syncthreads();
    if (threadIdx.x == 0) prz[blockIdx.x] = s1;
    double s2 = block_sum(rr, sh);
    if (threadIdx.x == 0) prr[blockIdx.x] = s2;
    if (prf) {
        __syncthreads();
        double s3 = block_sum(rzo, sh);
        if (threadIdx.x == 0) prf[blockIdx.x] = s3;
    }
    // the last block reduces rz, rr (and r.z_old) in a fixed order:
    // beta = rz_new / rz (flexible: (rz_new - r.z_old) / rz)
    if (last_block(counter)) {
        const double rzn = reduce_partials_l2(prz, gridDim.x, sh);
        const double rrn = reduce_partials_l2(prr, gridDim.x, sh);
        const double rzo_t = prf ? reduce_partials_l2(prf, gridDim.x, sh) : 0.;
        if (threadIdx.x == 0) {
            const double rzc = *rz_cur;
            *rz_new = rzn;
            *rr_out = rrn;
            *beta_out = rzc != 0. ? (rzn - rzo_t) / rzc : 0.;
            *counter = 0u;
        }
    }
}

// K3: p = z + beta p (beta from the update kernel's last block; a restart
// sets p = z without reading p: fresh allocations hold garbage).
template <typename PT>
__global__ void __launch_bounds__(RED_BS) direction_kernel(int64_t n, const double *beta_in, int restart,
                                                           const PT *__restrict__ z, PT *__restrict__ p,
                                                           float2 *__restrict__ p2) {
    const double beta = restart ? 0. : *beta_in;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const PT v = beta == 0. ? z[i] : (PT)((double)z[i] + beta * (double)p[i]);
        p[i] = v;
        if (p2) p2[i] = split_double((double)v);  // the split SpMV's operand
    }
}

__device__ __forceinline__ void two_sum(double a, double b, double &s, double &e) {
    s = a + b;
    const double bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

// Solution base in double-double: (xhi, xlo) += d exactly up to the
// double-double rounding, then d = 0.
__global__ void fold_kernel(int64_t n, double *xhi, double *xlo, double *d) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double sh, e;
        two_sum(xhi[i], d[i], sh, e);
        e += xlo[i];
        const double h = sh + e;
        xlo[i] = e - (h - sh);
        xhi[i] = h;
        d[i] = 0.;
    }
}

// r = f - K (xhi + xlo) with compensated row sums (products split exactly
// with an FMA, sums carried in double-double); partial sums of r.r.
__global__ void __launch_bounds__(RED_BS) dd_residual_kernel(int64_t n, const int64_t *__restrict__ rowptr,
                                                             const int32_t *__restrict__ colind,
                                                             const double *__restrict__ vals,
                                                             const double *__restrict__ xhi,
                                                             const double *__restrict__ xlo,
                                                             const double *__restrict__ f, double *__restrict__ r,
                                                             double *partial_rr) {
    __shared__ double sh[33];
    const int lane = threadIdx.x % LANES_PER_ROW;
    const int64_t group = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) / LANES_PER_ROW;
    const int64_t ngroups = (int64_t)gridDim.x * blockDim.x / LANES_PER_ROW;
    double rr = 0.;
    const int64_t trips = (n + ngroups - 1) / ngroups;  // uniform: full-warp shuffles below
    for (int64_t t = 0; t < trips; t++) {
        const int64_t row = group + t * ngroups;
        const bool in = row < n;
        double hi = 0., lo = 0.;
        const int64_t kb = in ? rowptr[row] + lane : 0, ke = in ? rowptr[row + 1] : 0;
        for (int64_t k = kb; k < ke; k += LANES_PER_ROW) {
            const double a = vals[k];
            const int c = colind[k];
            const double xh = xhi[c];
            const double pr = a * xh;
            const double pe = fma(a, xh, -pr);
            double e;
            two_sum(hi, pr, hi, e);
            lo = fma(a, xlo[c], lo + (e + pe));
        }
#pragma unroll
        for (int o = LANES_PER_ROW / 2; o > 0; o >>= 1) {
            const double oh = __shfl_xor_sync(0xffffffffu, hi, o);
            const double ol = __shfl_xor_sync(0xffffffffu, lo, o);
            double e;
            two_sum(hi, oh, hi, e);
            lo += ol + e;
        }
        if (in && lane == 0) {
            double sm, e;
            two_sum(f[row], -hi, sm, e);
            const double ri = sm + (e - lo);
            r[row] = ri;
            rr += ri * ri;
        }
    }
    const double s = block_sum(rr, sh);
    if (threadIdx.x == 0) partial_rr[blockIdx.x] = s;
}

__global__ void combine_kernel(int64_t n, const double *xhi, const double *xlo, double *u) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        u[i] = xhi[i] + xlo[i];
}

__global__ void finalize_sum_kernel(const double *partials, int n, double *out) {
    __shared__ double sh[34];
    const double v = reduce_partials(partials, n, sh);
    if (threadIdx.x == 0) *out = v;
}

}  // namespace
}  // namespace fe3d


using namespace fe3d;

namespace fe3d {
namespace {

__global__ void node_blocks_kernel(int64_t nnodes, int64_t N, const int32_t *row_of_dof,
                                   int32_t *start, int8_t *size, int bs) {
    const int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (j >= nnodes) return;
    int s = -1, b = 0;
    for (int d = 0; d < bs; d++) {
        const int64_t dof = (int64_t)bs * j + d;
        if (dof < N) {
            const int32_t r = row_of_dof[dof];
            if (r >= 0) {
                if (s < 0) s = r;
                b++;
            }
        }
    }
    start[j] = s < 0 ? 0 : s;
    size[j] = (int8_t)b;
}

template <typename T>
int alloc(T **p, size_t n) {
    if (n == 0) n = 1;
    return cudaMalloc((void **)p, n * sizeof(T)) == cudaSuccess ? 0 : FE3D_ERR_NOMEM;
}

int grid_cap(int64_t work, int per_block, int cap) {
    int64_t g = (work + per_block - 1) / per_block;
    if (g < 1) g = 1;
    return (int)(g < cap ? g : cap);
}

int spmv_grid_for(int64_t n, int lanes) { return grid_cap(n * lanes, RED_BS, kSMs * 8); }

template <typename VT, typename XT>
void launch_spmv(int lanes, cudaStream_t st, int64_t n, const fe3d_pattern *pat, const VT *vals, const XT *x, XT *y,
                 double *partial, unsigned int *counter, const double *rz, double *alpha) {
    const int g = spmv_grid_for(n, lanes);
#define FE3D_SPMV(L, C)                                                                                  \
    spmv_kernel<VT, XT, L, C><<<g, RED_BS, 0, st>>>(n, pat->rowptr, pat->colind, pat->colbase, pat->col16, \
                                                    vals, x, y, partial, counter, rz, alpha)
    if (pat->col16) {
        switch (lanes) {
            case 2: FE3D_SPMV(2, true); break;
            case 8: FE3D_SPMV(8, true); break;
            case 16: FE3D_SPMV(16, true); break;
            default: FE3D_SPMV(4, true); break;
        }
    } else {
        switch (lanes) {
            case 2: FE3D_SPMV(2, false); break;
            case 8: FE3D_SPMV(8, false); break;
            case 16: FE3D_SPMV(16, false); break;
            default: FE3D_SPMV(4, false); break;
        }
    }
#undef FE3D_SPMV
}

void launch_spmv_split(int lanes, cudaStream_t st, int64_t n, const fe3d_pattern *pat, const float2 *vals,
                       const float2 *x2, const double *x, double *y, double *partial, unsigned int *counter,
                       const double *rz, double *alpha) {
    const int g = spmv_grid_for(n, lanes);
#define FE3D_SPMV2(L, C)                                                                                    \
    spmv_split_kernel<L, C><<<g, RED_BS, 0, st>>>(n, pat->rowptr, pat->colind, pat->colbase, pat->col16, vals, \
                                                  x2, x, y, partial, counter, rz, alpha)
    if (pat->col16) {
        switch (lanes) {
            case 2: FE3D_SPMV2(2, true); break;
            case 8: FE3D_SPMV2(8, true); break;
            case 16: FE3D_SPMV2(16, true); break;
            default: FE3D_SPMV2(4, true); break;
        }
    } else {
        switch (lanes) {
            case 2: FE3D_SPMV2(2, false); break;
            case 8: FE3D_SPMV2(8, false); break;
            case 16: FE3D_SPMV2(16, false); break;
            default: FE3D_SPMV2(4, false); break;
        }
    }
#undef FE3D_SPMV2
}

int tune_spmv_split(fe3d_solver *s, cudaStream_t st, int *best) {
    *best = 4;
    const int64_t n = s->pat->nrows;
    if (n == 0) return FE3D_OK;
    FE3D_CUDA(cudaMemsetAsync(s->p, 0, sizeof(double) * n, st));
    FE3D_CUDA(cudaMemsetAsync(s->p2, 0, sizeof(float2) * n, st));
    cudaEvent_t e0, e1;
    FE3D_CUDA(cudaEventCreate(&e0));
    FE3D_CUDA(cudaEventCreate(&e1));
    const int cand[4] = {2, 4, 8, 16};
    float bestms = 1e30f;
    int rc = FE3D_OK;
    for (int c = 0; c < 4; c++) {
        launch_spmv_split(cand[c], st, n, s->pat, s->vals2, s->p2, s->p, s->q, nullptr, nullptr, nullptr, nullptr);
        cudaEventRecord(e0, st);
        for (int w = 0; w < 5; w++)
            launch_spmv_split(cand[c], st, n, s->pat, s->vals2, s->p2, s->p, s->q, nullptr, nullptr, nullptr,
                              nullptr);
        cudaEventRecord(e1, st);
        if (cudaGetLastError() != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess) {
            rc = FE3D_ERR_CUDA;
            break;
        }
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms < bestms) {
            bestms = ms;
            *best = cand[c];
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return rc;
}

// Times the lanes-per-row candidates of the SpMV on this matrix (x = 0) and
// returns the fastest.
template <typename VT, typename XT>
int tune_spmv(const fe3d_pattern *pat, const VT *vals, XT *x, XT *y, cudaStream_t st, int *best) {
    *best = 4;
    if (pat->nrows == 0) return FE3D_OK;
    FE3D_CUDA(cudaMemsetAsync(x, 0, sizeof(XT) * pat->nrows, st));
    cudaEvent_t e0, e1;
    FE3D_CUDA(cudaEventCreate(&e0));
    FE3D_CUDA(cudaEventCreate(&e1));
    const int cand[4] = {2, 4, 8, 16};
    float bestms = 1e30f;
    int rc = FE3D_OK;
    for (int c = 0; c < 4; c++) {
        launch_spmv<VT, XT>(cand[c], st, pat->nrows, pat, vals, x, y, nullptr, nullptr, nullptr, nullptr);
        cudaEventRecord(e0, st);
        for (int w = 0; w < 5; w++)
            launch_spmv<VT, XT>(cand[c], st, pat->nrows, pat, vals, x, y, nullptr, nullptr, nullptr, nullptr);
        cudaEventRecord(e1, st);
        if (cudaGetLastError() != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess) {
            rc = FE3D_ERR_CUDA;
            break;
        }
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms < bestms) {
            bestms = ms;
            *best = cand[c];
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return rc;
}

}  // namespace
}  // namespace fe3d

extern "C" int fe3d_solver_free(fe3d_solver *s) {
    if (!s) return FE3D_OK;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 2; j++)
            if (s->graph[i][j]) cudaGraphExecDestroy(s->graph[i][j]);
    if (s->ev_in) cudaEventDestroy(s->ev_in);
    if (s->ev_out) cudaEventDestroy(s->ev_out);
    if (s->stream) cudaStreamDestroy(s->stream);
    cudaFree(s->uin); cudaFree(s->fin); cudaFree(s->xhi); cudaFree(s->xlo); cudaFree(s->sc); cudaFree(s->counter);
    cudaFree(s->start); cudaFree(s->size); cudaFree(s->Dinv); cudaFree(s->Dinv32);
    cudaFree(s->vals32); cudaFree(s->r); cudaFree(s->z); cudaFree(s->p); cudaFree(s->q);
    cudaFree(s->z32); cudaFree(s->p32); cudaFree(s->q32); cudaFree(s->ppq); cudaFree(s->prz);
    cudaFree(s->prr); cudaFree(s->prf); cudaFree(s->scal); cudaFree(s->nonpos);
    cudaFree(s->vals2); cudaFree(s->p2);
    delete s;
    return FE3D_OK;
}

extern "C" int fe3d_solver_create(const fe3d_pattern *pat, int block_size, fe3d_solver **out) {
    if (!pat || !out || block_size < 1 || block_size > 6) return FE3D_ERR_ARG;
    *out = nullptr;
    fe3d_solver *s = new fe3d_solver();
    s->pat = pat;
    s->n = pat->nrows;
    s->nnodes = (pat->N + block_size - 1) / block_size;
    s->bs = block_size;
    int rc = 0;
    const int64_t n = s->n;
    s->spmv_grid = grid_cap(n * LANES_PER_ROW, RED_BS, kSMs * 8);
    s->node_grid = grid_cap(s->nnodes, RED_BS, kSMs * 8);
    s->vec_grid = grid_cap(n, RED_BS, kSMs * 8);
    s->nparts = kSMs * 8;
    if ((rc = alloc(&s->start, s->nnodes)) || (rc = alloc(&s->size, s->nnodes)) ||
        (rc = alloc(&s->Dinv, 36 * (size_t)s->nnodes)) || (rc = alloc(&s->Dinv32, 36 * (size_t)s->nnodes)) ||
        (rc = alloc(&s->r, n)) || (rc = alloc(&s->z, n)) || (rc = alloc(&s->p, n)) ||
        (rc = alloc(&s->q, n)) || (rc = alloc(&s->ppq, s->nparts)) || (rc = alloc(&s->prz, s->nparts)) ||
        (rc = alloc(&s->prr, s->nparts)) || (rc = alloc(&s->prf, s->nparts)) || (rc = alloc(&s->scal, 8)) ||
        (rc = alloc(&s->nonpos, 2)) ||
        (rc = alloc(&s->uin, n)) || (rc = alloc(&s->fin, n)) || (rc = alloc(&s->xhi, n)) ||
        (rc = alloc(&s->xlo, n)) || (rc = alloc(&s->sc, 2 * n)) || (rc = alloc(&s->counter, 1))) {
        fe3d_solver_free(s);
        return rc;
    }
    if (cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&s->ev_in, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&s->ev_out, cudaEventDisableTiming) != cudaSuccess) {
        fe3d_solver_free(s);
        return FE3D_ERR_CUDA;
    }
    cudaMemset(s->counter, 0, sizeof(unsigned int));
    node_blocks_kernel<<<grid_cap(s->nnodes, 256, 1 << 30), 256>>>(s->nnodes, pat->N, pat->row_of_dof,
                                                                 s->start, s->size, block_size);
    if (cudaDeviceSynchronize() != cudaSuccess) {
        fe3d_solver_free(s);
        return FE3D_ERR_CUDA;
    }
    *out = s;
    return FE3D_OK;
}

extern "C" int fe3d_solver_setup(fe3d_solver *s, const double *vals, int mixed, int *nonpos_blocks,
                                 void *stream) {
    if (!s || (s->pat->nnz > 0 && !vals)) return FE3D_ERR_ARG;
    cudaStream_t st = as_stream(stream);
    // captured iteration graphs embed the value pointers: rebuild them
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 2; j++)
            if (s->graph[i][j]) {
                cudaGraphExecDestroy(s->graph[i][j]);
                s->graph[i][j] = nullptr;
            }
    s->vals = vals;
    s->ready = 1;
    FE3D_CUDA(cudaMemsetAsync(s->nonpos, 0, sizeof(int), st));
    bjacobi_setup_kernel<<<grid_cap(s->nnodes, 128, 1 << 30), 128, 0, st>>>(
        s->nnodes, s->start, s->size, s->pat->rowptr, s->pat->colind, vals, s->Dinv, s->Dinv32, s->sc, s->n,
        s->nonpos);
    FE3D_CHECK_LAUNCH();
    if (mixed & 2) {
        if (!s->have2) {
            if (alloc(&s->vals2, s->pat->nnz) || alloc(&s->p2, s->n)) return FE3D_ERR_NOMEM;
            s->have2 = 1;
        }
        split_kernel<<<grid_cap(s->pat->nnz, 256, kSMs * 16), 256, 0, st>>>(s->pat->nnz, vals, s->vals2);
        FE3D_CHECK_LAUNCH();
    }
    if (mixed & 1) {
        if (!s->have32) {
            if (alloc(&s->vals32, s->pat->nnz) || alloc(&s->z32, s->n) || alloc(&s->p32, s->n) ||
                alloc(&s->q32, s->n))
                return FE3D_ERR_NOMEM;
            s->have32 = 1;
        }
        if (s->n > 0)
            cast_scaled_kernel<<<grid_cap(s->n, 256, 1 << 30), 256, 0, st>>>(s->n, s->pat->rowptr, s->pat->colind,
                                                                             vals, s->sc, s->vals32);
        FE3D_CHECK_LAUNCH();
    }
    int h = 0;
    FE3D_CUDA(cudaMemcpyAsync(&h, s->nonpos, sizeof(int), cudaMemcpyDeviceToHost, st));
    FE3D_CUDA(cudaStreamSynchronize(st));
    if (nonpos_blocks) *nonpos_blocks = h;
    int rc = FE3D_OK;
    if (!s->lanes[0]) rc = tune_spmv<double, double>(s->pat, vals, s->p, s->q, st, &s->lanes[0]);
    if (!rc && (mixed & 1) && !s->lanes[1])
        rc = tune_spmv<float, float>(s->pat, s->vals32, s->p32, s->q32, st, &s->lanes[1]);
    if (!rc && (mixed & 2) && !s->lanes[2]) rc = tune_spmv_split(s, st, &s->lanes[2]);
    return rc;
}

extern "C" int fe3d_solver_set_blocks(fe3d_solver *s, const double *blocks, int8_t *fallback, int *nfallback,
                                      void *stream) {
    if (!s || (s->nnodes > 0 && !blocks)) return FE3D_ERR_ARG;
    if (!s->ready) return FE3D_ERR_STATE;
    cudaStream_t st = as_stream(stream);
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 2; j++)
            if (s->graph[i][j]) {
                cudaGraphExecDestroy(s->graph[i][j]);
                s->graph[i][j] = nullptr;
            }
    // counters: [0] fallbacks, [1] not positive definite diagonal blocks
    FE3D_CUDA(cudaMemsetAsync(s->nonpos, 0, 2 * sizeof(int), st));
    if (s->nnodes > 0) {
        blocks_setup_kernel<<<grid_cap(s->nnodes, 128, 1 << 30), 128, 0, st>>>(
            s->nnodes, s->start, s->size, s->pat->rowptr, s->pat->colind, s->vals, blocks, s->Dinv, s->Dinv32,
            s->sc, s->n, fallback, s->nonpos, s->nonpos + 1);
        FE3D_CHECK_LAUNCH();
    }
    int h[2] = {0, 0};
    FE3D_CUDA(cudaMemcpyAsync(h, s->nonpos, 2 * sizeof(int), cudaMemcpyDeviceToHost, st));
    FE3D_CUDA(cudaStreamSynchronize(st));
    if (nfallback) *nfallback = h[0];
    return FE3D_OK;
}

extern "C" int fe3d_spmv(const fe3d_pattern *p, const double *vals, const double *x, double *y,
                         void *stream) {
    if (!p || (p->nrows > 0 && (!vals || !x || !y))) return FE3D_ERR_ARG;
    if (p->nrows == 0) return FE3D_OK;
    launch_spmv<double, double>(4, as_stream(stream), p->nrows, p, vals, x, y, nullptr, nullptr, nullptr, nullptr);
    FE3D_CHECK_LAUNCH();
    return FE3D_OK;
}

namespace {

// FP64 residual r = f - K u; returns ||r||^2 (synchronises).
int true_residual(fe3d_solver *s, const double *f, double *u, cudaStream_t st, double *rr) {
    // the increment u since the last replacement joins the double-double
    // base, whose residual is evaluated with compensated sums
    fold_kernel<<<s->vec_grid, RED_BS, 0, st>>>(s->n, s->xhi, s->xlo, u);
    dd_residual_kernel<<<s->spmv_grid, RED_BS, 0, st>>>(s->n, s->pat->rowptr, s->pat->colind, s->vals, s->xhi,
                                                         s->xlo, f, s->r, s->prr);
    finalize_sum_kernel<<<1, RED_BS, 0, st>>>(s->prr, s->spmv_grid, s->scal + 2);
    FE3D_CHECK_LAUNCH();
    FE3D_CUDA(cudaMemcpyAsync(rr, s->scal + 2, sizeof(double), cudaMemcpyDeviceToHost, st));
    FE3D_CUDA(cudaStreamSynchronize(st));
    return FE3D_OK;
}

template <typename PT, typename VT>
int run_cg(fe3d_solver *s, const double *f, double *u, const fe3d_solve_opts *o, fe3d_solve_stats *stats,
           cudaStream_t st, const VT *vals_k, const PT *Dk, PT *z, PT *p, PT *q, int prec) {
    // prec 0: FP64; 1: FP32 recurrence on the scaled system; 2: FP64 vectors
    // with the split-FP32 SpMV; 3: nested iterative refinement -- inner FP32
    // PCG on the scaled system (FP32 values, block inverses, directions and
    // products) run from a fresh direction until its recurrence residual has
    // dropped by inner_tol, then the outer FP64 step: the increment joins the
    // double-double iterate and r = f - K x is recomputed in FP64
    const int nested = prec == 3;
    const int mixed = prec == 1 || nested;
    float2 *p2 = prec == 2 ? s->p2 : nullptr;
    const int64_t n = s->n;
    const double *sck = mixed ? s->sc : nullptr;  // the FP32 recurrence runs on S^-1 K S^-1
    const double *isck = mixed ? s->sc + n : nullptr;
    double ff = 0.;
    {
        // ||f||
        precond_kernel<double, double><<<s->node_grid, RED_BS, 0, st>>>(
            s->nnodes, s->start, s->size, s->Dinv, f, s->z, s->prz, s->prr, nullptr, nullptr);
        finalize_sum_kernel<<<1, RED_BS, 0, st>>>(s->prr, s->node_grid, s->scal + 4);
        FE3D_CHECK_LAUNCH();
        FE3D_CUDA(cudaMemcpyAsync(&ff, s->scal + 4, sizeof(double), cudaMemcpyDeviceToHost, st));
        FE3D_CUDA(cudaStreamSynchronize(st));
    }
    stats->iterations = 0;
    stats->replacements = 0;
    stats->status = 1;
    if (ff == 0.) {
        if (n) FE3D_CUDA(cudaMemsetAsync(u, 0, sizeof(double) * n, st));
        stats->relres = 0.;
        stats->status = 0;
        return FE3D_OK;
    }
    const double target = o->tol * o->tol * ff;
    // solution = (xhi + xlo) + u: the base starts at the initial guess and
    // the iterations accumulate the increment u
    if (n) {
        FE3D_CUDA(cudaMemcpyAsync(s->xhi, u, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
        FE3D_CUDA(cudaMemsetAsync(s->xlo, 0, sizeof(double) * n, st));
        FE3D_CUDA(cudaMemsetAsync(u, 0, sizeof(double) * n, st));
    }
    double rr = 0.;
    int rc = true_residual(s, f, u, st, &rr);
    if (rc) return rc;
    if (!(rr == rr)) {
        combine_kernel<<<s->vec_grid, RED_BS, 0, st>>>(n, s->xhi, s->xlo, u);
        FE3D_CHECK_LAUNCH();
        stats->status = 3;
        stats->relres = rr;
        return FE3D_OK;
    }
    const int check = o->check_every > 0 ? o->check_every : 50;
    // nested: replace_every caps the iterations of one inner solve (0: none)
    const int replace = nested ? (o->replace_every > 0 ? o->replace_every : 0)
                               : mixed ? (o->replace_every > 0 ? o->replace_every : 100) : 0;
    const double inner2 = nested ? (o->inner_tol > 0. && o->inner_tol < 1. ? o->inner_tol * o->inner_tol : 1e-4)
                                 : 1e-4;
    int64_t it = 0;
    int par = 0;  // rz double buffer index
    // restart: z = Minv r; p = z; rz
    auto restart = [&]() -> int {
        precond_kernel<PT, PT><<<s->node_grid, RED_BS, 0, st>>>(s->nnodes, s->start, s->size, Dk, s->r, z,
                                                               s->prz, s->prr, sck, isck);
        finalize_sum_kernel<<<1, RED_BS, 0, st>>>(s->prz, s->node_grid, s->scal + (par ^ 1));
        direction_kernel<PT><<<s->vec_grid, RED_BS, 0, st>>>(n, nullptr, 1, z, p, p2);
        par ^= 1;
        FE3D_CHECK_LAUNCH();
        return FE3D_OK;
    };
    if ((rc = restart())) return rc;
    double relres = sqrt(rr / ff);
    // iterations run in chunks of an even length, each chunk one CUDA graph
    // replay (the rz double-buffer parity is the same at every chunk start)
    int chunk = check < 2 ? 2 : (check & ~1);
    const int pidx = prec == 3 ? 1 : prec;  // the nested inner iterations are the precision-1 graphs
    double *prf = o->flexible ? s->prf : nullptr;
    const int gflex = o->flexible ? 1 : 0;
    const int lanes = s->lanes[pidx] ? s->lanes[pidx] : 4;
    auto launch_iteration = [&](int pr) {
        // scal: [pr] rz, [pr ^ 1] rz_new, [2] r.r, [3] alpha, [5] beta
        if (prec == 2)
            launch_spmv_split(lanes, st, n, s->pat, s->vals2, p2, (const double *)p, (double *)q, s->ppq, s->counter,
                              s->scal + pr, s->scal + 3);
        else
            launch_spmv<VT, PT>(lanes, st, n, s->pat, vals_k, p, q, s->ppq, s->counter, s->scal + pr, s->scal + 3);
        update_kernel<PT, PT><<<s->node_grid, RED_BS, 0, st>>>(s->nnodes, s->start, s->size, Dk, s->scal + 3,
                                                               s->scal + pr, p, q, u, s->r, z, s->prz, s->prr, prf,
                                                               sck, isck, s->counter, s->scal + (pr ^ 1), s->scal + 2,
                                                               s->scal + 5);
        direction_kernel<PT><<<s->vec_grid, RED_BS, 0, st>>>(n, s->scal + 5, 0, z, p, p2);
    };
    auto run_chunk = [&](int len) -> int {
        if (len == chunk) {
            cudaGraphExec_t &ge = s->graph[pidx][par];
            if (!ge || s->graph_chunk[pidx][par] != chunk || s->graph_flex[pidx][par] != gflex ||
                s->graph_lanes[pidx][par] != lanes) {
                if (ge) {
                    cudaGraphExecDestroy(ge);
                    ge = nullptr;
                }
                cudaGraph_t g = nullptr;
                FE3D_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
                int pr = par;
                for (int i = 0; i < chunk; i++) {
                    launch_iteration(pr);
                    pr ^= 1;
                }
                FE3D_CUDA(cudaStreamEndCapture(st, &g));
                const cudaError_t e = cudaGraphInstantiate(&ge, g, 0);
                cudaGraphDestroy(g);
                if (e != cudaSuccess) {
                    ge = nullptr;
                    return FE3D_ERR_CUDA;
                }
                s->graph_chunk[pidx][par] = chunk;
                s->graph_flex[pidx][par] = gflex;
                s->graph_lanes[pidx][par] = lanes;
            }
            FE3D_CUDA(cudaGraphLaunch(ge, st));
        } else {
            int pr = par;
            for (int i = 0; i < len; i++) {
                launch_iteration(pr);
                pr ^= 1;
            }
        }
        if (len & 1) par ^= 1;
        FE3D_CHECK_LAUNCH();
        return FE3D_OK;
    };
    // residual replacement (reliable updates): r = f - K x from the
    // double-double base, z = Minv r and r.z rebuilt, the direction p kept.
    // Triggered every `replace` iterations (mixed precision), when the
    // recurrence residual has dropped 100-fold since the last replacement,
    // and when the recurrence reports convergence (the FP64 residual decides).
    auto replace_residual = [&](double *rt) -> int {
        int e = true_residual(s, f, u, st, rt);
        if (e) return e;
        stats->replacements++;
        precond_kernel<PT, PT><<<s->node_grid, RED_BS, 0, st>>>(s->nnodes, s->start, s->size, Dk, s->r, z,
                                                               s->prz, s->prr, sck, isck);
        finalize_sum_kernel<<<1, RED_BS, 0, st>>>(s->prz, s->node_grid, s->scal + par);
        FE3D_CHECK_LAUNCH();
        return FE3D_OK;
    };
    int64_t since_replace = 0;
    double rr_replaced = rr;
    int stalls = 0;
    while (it < o->maxiter) {
        const int len = (int)((o->maxiter - it) < chunk ? (o->maxiter - it) : chunk);
        if ((rc = run_chunk(len))) return rc;
        it += len;
        since_replace += len;
        FE3D_CUDA(cudaMemcpyAsync(&rr, s->scal + 2, sizeof(double), cudaMemcpyDeviceToHost, st));
        FE3D_CUDA(cudaStreamSynchronize(st));
        if (!(rr == rr) || isinf(rr)) {
            stats->status = 3;
            break;
        }
        const bool periodic = replace && since_replace >= replace;
        if (periodic || rr <= target || rr <= inner2 * rr_replaced) {
            double rt = 0.;
            if (nested) {
                // outer step: FP64 residual of the refined iterate, and a new
                // inner solve from a fresh direction
                if ((rc = true_residual(s, f, u, st, &rt))) return rc;
                stats->replacements++;
                if ((rc = restart())) return rc;
            } else if ((rc = replace_residual(&rt))) {
                return rc;
            }
            since_replace = 0;
            relres = sqrt(rt / ff);
            if (rt <= target) {
                stats->status = 0;
                break;
            }
            if (nested) {
                // no 10 % progress over three outer steps in a row: the FP32
                // inner solves can no longer reduce the FP64 residual
                stalls = rt > 0.81 * rr_replaced ? stalls + 1 : 0;
                if (stalls >= 3) {
                    stats->status = 4;
                    break;
                }
            }
            // mixed precision: no 10 % progress of the FP64 residual over
            // three periodic replacements in a row means FP32 directions can
            // no longer reduce it (kappa * eps32 too large): status 4
            if (periodic && !nested) {
                stalls = rt > 0.81 * rr_replaced ? stalls + 1 : 0;
                if (stalls >= 3) {
                    stats->status = 4;
                    break;
                }
            }
            rr_replaced = rt;
        }
    }
    double rt = 0.;
    if ((rc = true_residual(s, f, u, st, &rt))) return rc;
    // the caller gets the base rounded to FP64
    combine_kernel<<<s->vec_grid, RED_BS, 0, st>>>(n, s->xhi, s->xlo, u);
    FE3D_CHECK_LAUNCH();
    relres = sqrt(rt / ff);
    if (stats->status != 3 && stats->status != 4) stats->status = (rt <= target) ? 0 : 1;
    stats->iterations = it;
    stats->relres = relres;
    return FE3D_OK;
}

}  // namespace

extern "C" int fe3d_solver_solve(fe3d_solver *s, const double *f, double *u, const fe3d_solve_opts *o,
                                 fe3d_solve_stats *stats, void *stream) {
    if (!s || !o || !stats || (s->n > 0 && (!f || !u))) return FE3D_ERR_ARG;
    if (!s->ready) return FE3D_ERR_STATE;
    if (o->precision < 0 || o->precision > 3) return FE3D_ERR_ARG;
    if (((o->precision == 1 || o->precision == 3) && !s->have32) || (o->precision == 2 && !s->have2))
        return FE3D_ERR_STATE;
    if (o->tol <= 0 || o->maxiter < 0) return FE3D_ERR_ARG;
    cudaStream_t caller = as_stream(stream), st = s->stream;
    const size_t bytes = sizeof(double) * (size_t)s->n;
    FE3D_CUDA(cudaEventRecord(s->ev_in, caller));
    FE3D_CUDA(cudaStreamWaitEvent(st, s->ev_in, 0));
    if (s->n) {
        FE3D_CUDA(cudaMemcpyAsync(s->fin, f, bytes, cudaMemcpyDeviceToDevice, st));
        FE3D_CUDA(cudaMemcpyAsync(s->uin, u, bytes, cudaMemcpyDeviceToDevice, st));
    }
    int rc;
    if (o->precision == 1 || o->precision == 3)
        rc = run_cg<float, float>(s, s->fin, s->uin, o, stats, st, s->vals32, s->Dinv32, s->z32, s->p32, s->q32,
                                  o->precision);
    else
        rc = run_cg<double, double>(s, s->fin, s->uin, o, stats, st, s->vals, s->Dinv, s->z, s->p, s->q,
                                    o->precision);
    if (rc) return rc;
    if (s->n) FE3D_CUDA(cudaMemcpyAsync(u, s->uin, bytes, cudaMemcpyDeviceToDevice, st));
    FE3D_CUDA(cudaEventRecord(s->ev_out, st));
    FE3D_CUDA(cudaStreamWaitEvent(caller, s->ev_out, 0));
    return FE3D_OK;
}

