// Learned block preconditioner for the PCG of the static solve (no
// counterpart in the reference, whose tests call spsolve/cg directly:
// tests/test_quad4_static_point_load.py:102).
//
// Per node j (6 DOFs) a small MLP (FP32, inputs -> 64 -> 64 -> 21, tanh)
// reads features of the node's diagonal block D_j and of its couplings and
// predicts a symmetric 6x6 correction C_j in the scaled coordinates
// S^-1 D S^-1 (S = sqrt(diag K)).  The preconditioner block is
//     B_j = D_j + scale * S_j C_j S_j        (free DOFs of the node)
// inverted through its Cholesky factor; a block that is not positive
// definite falls back to the block-Jacobi inverse (fe3d_solver_set_blocks).
// Flexible CG with these blocks converges to the FP64 tolerance whatever the
// prediction: a poor network costs iterations only.
//
// Features (35 floats per node, zero for a node without free DOFs):
//   [0, 15)   off-diagonal entries of S^-1 D S^-1 over the 6 local DOFs,
//             upper triangle row-major (0 for constrained DOFs)
//   [15, 21)  (log D_ii - mean over the node's free DOFs) / 10
//   [21, 27)  1 for a free DOF, 0 for a constrained one
//   [27, 35)  Frobenius norms of the scaled coupling blocks S_j^-1 K_jk S_k^-1
//             to the neighbour nodes k, largest first (zero padded)
//
// Training (all on the GPU with the kernels below): for residuals r that the
// FP64 solver produced, z = B^-1 r and, with w = 1 / (e.r), e = K^-1 r,
//   mode 0: L = w (z.Kz - 2 z.r) = w ||z - e||_K^2 - 1, the squared
//           energy-norm error of z as an approximation of the error,
//           relative to ||e||_K^2, minus one;
//   mode 1: L = 1 - w (z.r)^2 / (z.Kz) = min_t ||t z - e||_K^2 / ||e||_K^2,
//           the same after the optimal step along z (invariant to the scale
//           of B, as CG is).
// With g = dL/dz and z_j = B_j^-1 r_j, dL/dB_j = -(B_j^-1 g_j) z_j^T and
// dL/dC_j = scale * S dL/dB_j S.
#include <math.h>

#include "common.cuh"
#include "fe3d_internal.h"

namespace fe3d {
namespace {

constexpr int NF = FE3D_LPC_NFEAT, NH = FE3D_LPC_NHID, NO = FE3D_LPC_NOUT;
constexpr int OW1 = 0, OB1 = OW1 + NH * NF, OW2 = OB1 + NH, OB2 = OW2 + NH * NH, OW3 = OB2 + NH,
              OB3 = OW3 + NO * NH, NW = OB3 + NO;
static_assert(NW == FE3D_LPC_NWEIGHTS, "weight layout");
constexpr int ND = NO + 2 * NH;  // per-node deltas: [dL/do | dL/da2 | dL/da1]

__host__ __device__ constexpr int ut_index(int i, int k) { return i * 6 - i * (i - 1) / 2 + (k - i); }  // i <= k
__host__ __device__ constexpr int off_index(int i, int k) { return i * 5 - i * (i - 1) / 2 + (k - i - 1); }  // i < k

int lgrid(int64_t work, int per_block) {
    int64_t g = (work + per_block - 1) / per_block;
    if (g < 1) g = 1;
    return (int)(g < (1 << 30) ? g : (1 << 30));
}

// sdiag[row] = sqrt(K_rr) (1 where the diagonal is not positive)
__global__ void lpc_sdiag_kernel(int64_t n, const int64_t *rowptr, const int32_t *colind, const double *vals,
                                 double *sdiag) {
    const int64_t row = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (row >= n) return;
    double d = 0.;
    for (int64_t k = rowptr[row]; k < rowptr[row + 1]; k++)
        if (colind[k] == row) d = vals[k];
    sdiag[row] = d > 0. ? sqrt(d) : 1.;
}

__device__ void gather_block(int s, int b, const int64_t *rowptr, const int32_t *colind, const double *vals,
                             double (&A)[6][6]) {
    for (int i = 0; i < 6; i++)
        for (int k = 0; k < 6; k++) A[i][k] = 0.;
    for (int i = 0; i < b; i++)
        for (int64_t k = rowptr[s + i]; k < rowptr[s + i + 1]; k++) {
            const int c = colind[k] - s;
            if (c >= 0 && c < b) A[i][c] = vals[k];
        }
}

__global__ void lpc_features_kernel(int64_t nnodes, const int32_t *start, const int8_t *size,
                                    const int64_t *dof_of_row, const int64_t *rowptr, const int32_t *colind,
                                    const double *vals, const double *sdiag, float *feat) {
    const int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (j >= nnodes) return;
    float *f = feat + NF * j;
    for (int i = 0; i < NF; i++) f[i] = 0.f;
    const int b = size[j], s = start[j];
    if (b == 0) return;
    double A[6][6];
    int li[6];
    long long nid[16];
    double nsum[16];
    int nn = 0;
    for (int i = 0; i < 6; i++)
        for (int k = 0; k < 6; k++) A[i][k] = 0.;
    for (int i = 0; i < b; i++) {
        const int64_t row = s + i;
        li[i] = (int)(dof_of_row[row] - 6 * j);
        const double di = sdiag[row];
        for (int64_t k = rowptr[row]; k < rowptr[row + 1]; k++) {
            const int c = colind[k];
            if (c >= s && c < s + b) {
                A[i][c - s] = vals[k];
                continue;
            }
            const long long nd = dof_of_row[c] / 6;
            double v = vals[k] / (di * sdiag[c]);
            v *= v;
            int slot = -1;
            for (int t = 0; t < nn; t++)
                if (nid[t] == nd) slot = t;
            if (slot < 0 && nn < 16) {
                slot = nn++;
                nid[slot] = nd;
                nsum[slot] = 0.;
            }
            if (slot >= 0) nsum[slot] += v;
        }
    }
    double mean = 0.;
    for (int i = 0; i < b; i++) mean += 2. * log(sdiag[s + i]);
    mean /= b;
    for (int i = 0; i < b; i++) {
        f[15 + li[i]] = (float)((2. * log(sdiag[s + i]) - mean) / 10.);
        f[21 + li[i]] = 1.f;
        for (int k = i + 1; k < b; k++)
            f[off_index(li[i], li[k])] = (float)(A[i][k] / (sdiag[s + i] * sdiag[s + k]));
    }
    for (int t = 0; t < 8 && t < nn; t++) {
        int best = t;
        for (int q = t + 1; q < nn; q++)
            if (nsum[q] > nsum[best]) best = q;
        const double v = nsum[best];
        nsum[best] = nsum[t];
        nsum[t] = v;
        f[27 + t] = (float)sqrt(v);
    }
}

// Feature set 1 (29 inputs, slots 29..34 zero): the 21 unique entries of
// the node's diagonal block normalised by the block diagonal, S^-1 D S^-1
// (upper triangle row-major over the 6 local DOFs; 1 on the diagonal of a
// free DOF, 0 for constrained DOFs), then the Frobenius norms of the
// normalised coupling blocks S_j^-1 K_jk S_k^-1 to the neighbour nodes k,
// largest first (8, zero padded).  Zero inputs leave their first-layer
// weights without gradient, so the network is a 29-input MLP.
__global__ void lpc_features29_kernel(int64_t nnodes, const int32_t *start, const int8_t *size,
                                      const int64_t *dof_of_row, const int64_t *rowptr, const int32_t *colind,
                                      const double *vals, const double *sdiag, float *feat) {
    const int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (j >= nnodes) return;
    float *f = feat + NF * j;
    for (int i = 0; i < NF; i++) f[i] = 0.f;
    const int b = size[j], s = start[j];
    if (b == 0) return;
    int li[6];
    long long nid[16];
    double nsum[16];
    int nn = 0;
    for (int i = 0; i < b; i++) li[i] = (int)(dof_of_row[s + i] - 6 * j);
    for (int i = 0; i < b; i++) {
        const int64_t row = s + i;
        const double di = sdiag[row];
        for (int64_t k = rowptr[row]; k < rowptr[row + 1]; k++) {
            const int c = colind[k];
            const double v = vals[k] / (di * sdiag[c]);
            if (c >= s && c < s + b) {
                const int a = li[i], bb = li[c - s];
                if (a <= bb) f[ut_index(a, bb)] = (float)v;
                continue;
            }
            const long long nd = dof_of_row[c] / 6;
            int slot = -1;
            for (int t = 0; t < nn; t++)
                if (nid[t] == nd) slot = t;
            if (slot < 0 && nn < 16) {
                slot = nn++;
                nid[slot] = nd;
                nsum[slot] = 0.;
            }
            if (slot >= 0) nsum[slot] += v * v;
        }
    }
    for (int t = 0; t < 8 && t < nn; t++) {
        int best = t;
        for (int q = t + 1; q < nn; q++)
            if (nsum[q] > nsum[best]) best = q;
        const double v = nsum[best];
        nsum[best] = nsum[t];
        nsum[t] = v;
        f[21 + t] = (float)sqrt(v);
    }
}

// out = MLP(feat); act (optional) keeps tanh outputs [h1 | h2] per node.
// Shared memory: the weights, then one column of 64 hidden values per
// thread (column-major across the block, so the accesses are conflict-free).
constexpr int MLP_THREADS = 128;
constexpr int MLP_SMEM = (NW + NH * MLP_THREADS) * (int)sizeof(float);
__global__ void __launch_bounds__(MLP_THREADS) lpc_forward_kernel(int64_t nnodes, const float *__restrict__ feat,
                                                                  const float *__restrict__ W,
                                                                  float *__restrict__ out,
                                                                  float *__restrict__ act) {
    extern __shared__ float sw[];
    float *hs = sw + NW;
    const int t = threadIdx.x;
    for (int i = t; i < NW; i += blockDim.x) sw[i] = W[i];
    __syncthreads();
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + t; j < nnodes; j += (int64_t)gridDim.x * blockDim.x) {
        float x[NF];
#pragma unroll
        for (int i = 0; i < NF; i++) x[i] = feat[NF * j + i];
#pragma unroll 1
        for (int h = 0; h < NH; h++) {
            float a = sw[OB1 + h];
#pragma unroll
            for (int i = 0; i < NF; i++) a = fmaf(sw[OW1 + h * NF + i], x[i], a);
            const float v = tanhf(a);
            hs[h * MLP_THREADS + t] = v;
            if (act) act[2 * NH * j + h] = v;
        }
        float o[NO];
#pragma unroll
        for (int m = 0; m < NO; m++) o[m] = sw[OB3 + m];
#pragma unroll 1
        for (int k = 0; k < NH; k++) {
            float a = sw[OB2 + k];
#pragma unroll
            for (int i = 0; i < NH; i++) a = fmaf(sw[OW2 + k * NH + i], hs[i * MLP_THREADS + t], a);
            const float h2 = tanhf(a);
            if (act) act[2 * NH * j + NH + k] = h2;
#pragma unroll
            for (int m = 0; m < NO; m++) o[m] = fmaf(sw[OW3 + m * NH + k], h2, o[m]);
        }
#pragma unroll
        for (int m = 0; m < NO; m++) out[NO * j + m] = o[m];
    }
}

// blocks[36 j] = D_j + scale S C_j S over the node's free DOFs.
__global__ void lpc_blocks_kernel(int64_t nnodes, const int32_t *start, const int8_t *size,
                                  const int64_t *dof_of_row, const int64_t *rowptr, const int32_t *colind,
                                  const double *vals, const double *sdiag, const float *out, float scale,
                                  double *blocks) {
    const int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (j >= nnodes) return;
    const int b = size[j], s = start[j];
    double A[6][6];
    gather_block(s, b, rowptr, colind, vals, A);
    int li[6];
    for (int i = 0; i < b; i++) li[i] = (int)(dof_of_row[s + i] - 6 * j);
    const float *o = out + NO * j;
    for (int i = 0; i < 6; i++)
        for (int k = 0; k < 6; k++) {
            double v = 0.;
            if (i < b && k < b) {
                const int p = li[i] < li[k] ? li[i] : li[k], q = li[i] < li[k] ? li[k] : li[i];
                v = A[i][k] + (double)scale * sdiag[s + i] * sdiag[s + k] * (double)o[ut_index(p, q)];
            }
            blocks[36 * j + 6 * i + k] = v;
        }
}

// z = Minv r with the solver's current block inverses (FP64).
__global__ void lpc_apply_kernel(int64_t nnodes, const int32_t *start, const int8_t *size, const double *Dinv,
                                 const double *r, double *z) {
    const int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (j >= nnodes) return;
    const int b = size[j], s = start[j];
    double rl[6];
    for (int i = 0; i < 6; i++) rl[i] = i < b ? r[s + i] : 0.;
    for (int i = 0; i < b; i++) {
        double a = 0.;
        for (int k = 0; k < 6; k++) a += Dinv[36 * j + 6 * i + k] * rl[k];
        z[s + i] = a;
    }
}

__device__ __forceinline__ double warp_sum(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// dots[0] += z.r, dots[1] += z.Kz over the rows.
__global__ void lpc_dots_kernel(int64_t n, const double *r, const double *z, const double *Kz, double *dots) {
    const int64_t nth = (int64_t)gridDim.x * blockDim.x;
    const int64_t trips = (n + nth - 1) / nth;
    double a = 0., b = 0.;
    for (int64_t t = 0; t < trips; t++) {
        const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x + t * nth;
        if (i < n) {
            a += z[i] * r[i];
            b += z[i] * Kz[i];
        }
    }
    a = warp_sum(a);
    b = warp_sum(b);
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(dots, a);
        atomicAdd(dots + 1, b);
    }
}

// One residual sample r (w = 1 / (e.r), e = K^-1 r; factor scales the
// sample's share of the batch).  gout[21 j] += dL/do_j, acc[0] += L.
//   mode 0: L = factor w (z.Kz - 2 z.r) = factor (w ||z - e||_K^2 - 1),
//           dL/dz = 2 factor w (Kz - r)
//   mode 1: the same error after the optimal step t = a / b along z
//           (a = z.r, b = z.Kz, from acc[1], acc[2]):
//           L = factor (1 - w a^2 / b),
//           dL/dz = factor (2 w a / b) (t Kz - r)
__global__ void lpc_grad_kernel(int64_t nnodes, const int32_t *start, const int8_t *size,
                                const int64_t *dof_of_row, const double *Dinv, const double *sdiag,
                                const double *r, const double *z, const double *Kz, const int8_t *fallback,
                                double w, double factor, float scale, int mode, float *gout, double *acc) {
    const int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    double cg = 2. * factor * w, t = 1.;
    if (mode == 1) {
        const double a = acc[1], b = acc[2];
        t = b != 0. ? a / b : 0.;
        cg = b != 0. ? 2. * factor * w * a / b : 0.;
    }
    double l = 0.;
    if (j < nnodes) {
        const int b = size[j], s = start[j];
        double g[6], zl[6], wv[6], sd[6];
        int li[6];
        for (int i = 0; i < 6; i++) g[i] = zl[i] = wv[i] = sd[i] = 0.;
        for (int i = 0; i < b; i++) {
            const double kz = Kz[s + i], ri = r[s + i], zi = z[s + i];
            l += zi * kz - 2. * zi * ri;
            g[i] = cg * (t * kz - ri);
            zl[i] = zi;
            sd[i] = sdiag[s + i];
            li[i] = (int)(dof_of_row[s + i] - 6 * j);
        }
        if (b > 0 && !(fallback && fallback[j])) {
            for (int i = 0; i < b; i++)
                for (int k = 0; k < b; k++) wv[i] += Dinv[36 * j + 6 * i + k] * g[k];
            float *go = gout + NO * j;
            for (int i = 0; i < b; i++)
                for (int k = i; k < b; k++) {
                    // G = -scale (S w)(S z)^T; a symmetric parameter collects G_ik + G_ki
                    double v = -(double)scale * sd[i] * sd[k] * (wv[i] * zl[k] + (i == k ? 0. : wv[k] * zl[i]));
                    const int p = li[i] < li[k] ? li[i] : li[k], q = li[i] < li[k] ? li[k] : li[i];
                    go[ut_index(p, q)] += (float)v;
                }
        }
    }
    if (mode == 0) {
        l = warp_sum(l * factor * w);
        if ((threadIdx.x & 31) == 0 && l != 0.) atomicAdd(acc, l);
    } else if (j == 0) {
        const double a = acc[1], b = acc[2];
        atomicAdd(acc, factor * (1. - (b != 0. ? w * a * a / b : 0.)));
    }
}

// Per-node deltas of the backward pass: [dL/do | dL/da2 | dL/da1].
__global__ void __launch_bounds__(MLP_THREADS) lpc_delta_kernel(int64_t nnodes, const float *__restrict__ W,
                                                                const float *__restrict__ act,
                                                                const float *__restrict__ gout,
                                                                float *__restrict__ delta) {
    extern __shared__ float sw[];
    float *ds = sw + NW;
    const int t = threadIdx.x;
    for (int i = t; i < NW; i += blockDim.x) sw[i] = W[i];
    __syncthreads();
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + t; j < nnodes; j += (int64_t)gridDim.x * blockDim.x) {
        float go[NO];
#pragma unroll
        for (int m = 0; m < NO; m++) {
            go[m] = gout[NO * j + m];
            delta[ND * j + m] = go[m];
        }
        const float *h = act + 2 * NH * j;
#pragma unroll 1
        for (int k = 0; k < NH; k++) {
            float a = 0.f;
#pragma unroll
            for (int m = 0; m < NO; m++) a = fmaf(sw[OW3 + m * NH + k], go[m], a);
            const float h2 = h[NH + k];
            const float d2 = a * (1.f - h2 * h2);
            ds[k * MLP_THREADS + t] = d2;
            delta[ND * j + NO + k] = d2;
        }
#pragma unroll 1
        for (int i = 0; i < NH; i++) {
            float a = 0.f;
#pragma unroll
            for (int k = 0; k < NH; k++) a = fmaf(sw[OW2 + k * NH + i], ds[k * MLP_THREADS + t], a);
            const float h1 = h[i];
            delta[ND * j + NO + NH + i] = a * (1.f - h1 * h1);
        }
    }
}

// gW[r][c] += sum_n d[n][r] x[n][c] and gb[r] += sum_n d[n][r] over a chunk
// of nodes per block (R, C <= 64).
constexpr int OS_THREADS = 256, OS_SUB = 32, OS_CHUNK = 1024, OS_PER = 16;
__global__ void __launch_bounds__(OS_THREADS) lpc_outer_kernel(int64_t N, int R, int C, const float *d, int ldd,
                                                               const float *x, int ldx, float *gW, float *gb) {
    __shared__ float ds[OS_SUB][64];
    __shared__ float xs[OS_SUB][64];
    const int t = threadIdx.x;
    float acc[OS_PER];
    int rr[OS_PER], cc[OS_PER];
#pragma unroll
    for (int q = 0; q < OS_PER; q++) {
        acc[q] = 0.f;
        const int w = t + OS_THREADS * q;
        rr[q] = w < R * C ? w / C : 0;
        cc[q] = w < R * C ? w - (w / C) * C : 0;
    }
    float bacc = 0.f;
    const int64_t n0 = (int64_t)blockIdx.x * OS_CHUNK;
    for (int64_t sub = n0; sub < n0 + OS_CHUNK && sub < N; sub += OS_SUB) {
        __syncthreads();
        for (int i = t; i < OS_SUB * 64; i += OS_THREADS) {
            const int n = i / 64, c = i - n * 64;
            const int64_t node = sub + n;
            ds[n][c] = (node < N && c < R) ? d[node * ldd + c] : 0.f;
            xs[n][c] = (node < N && c < C) ? x[node * ldx + c] : 0.f;
        }
        __syncthreads();
#pragma unroll 4
        for (int n = 0; n < OS_SUB; n++) {
#pragma unroll
            for (int q = 0; q < OS_PER; q++) acc[q] = fmaf(ds[n][rr[q]], xs[n][cc[q]], acc[q]);
            if (t < R) bacc += ds[n][t];
        }
    }
#pragma unroll
    for (int q = 0; q < OS_PER; q++) {
        const int w = t + OS_THREADS * q;
        if (w < R * C) atomicAdd(gW + w, acc[q]);
    }
    if (t < R) atomicAdd(gb + t, bacc);
}

__global__ void lpc_adam_kernel(int64_t nw, float *w, const float *g, float *m, float *v, float lr, float b1,
                                float b2, float eps, float c1, float c2) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= nw) return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    w[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

int check_solver(const fe3d_solver *s) {
    if (!s || !s->pat) return FE3D_ERR_ARG;
    if (s->bs != 6) return FE3D_ERR_ARG;
    if (!s->ready) return FE3D_ERR_STATE;
    return FE3D_OK;
}

}  // namespace
}  // namespace fe3d

using namespace fe3d;

extern "C" int fe3d_lpc_features(const fe3d_solver *s, float *feat, double *sdiag, void *stream) {
    return fe3d_lpc_features_set(s, 0, feat, sdiag, stream);
}

extern "C" int fe3d_lpc_features_set(const fe3d_solver *s, int set, float *feat, double *sdiag, void *stream) {
    if (set != 0 && set != 1) return FE3D_ERR_ARG;
    int rc = check_solver(s);
    if (rc) return rc;
    if (!feat || (s->n > 0 && !sdiag)) return FE3D_ERR_ARG;
    cudaStream_t st = as_stream(stream);
    const fe3d_pattern *p = s->pat;
    if (s->n > 0) {
        lpc_sdiag_kernel<<<lgrid(s->n, 256), 256, 0, st>>>(s->n, p->rowptr, p->colind, s->vals, sdiag);
        FE3D_CHECK_LAUNCH();
    }
    if (s->nnodes > 0) {
        if (set == 1)
            lpc_features29_kernel<<<lgrid(s->nnodes, 128), 128, 0, st>>>(s->nnodes, s->start, s->size, p->dof_of_row,
                                                                        p->rowptr, p->colind, s->vals, sdiag, feat);
        else
            lpc_features_kernel<<<lgrid(s->nnodes, 128), 128, 0, st>>>(s->nnodes, s->start, s->size, p->dof_of_row,
                                                                      p->rowptr, p->colind, s->vals, sdiag, feat);
        FE3D_CHECK_LAUNCH();
    }
    return FE3D_OK;
}

extern "C" int fe3d_lpc_forward(int64_t nnodes, const float *feat, const float *weights, float *out, float *act,
                                void *stream) {
    if (nnodes < 0 || (nnodes > 0 && (!feat || !weights || !out))) return FE3D_ERR_ARG;
    if (nnodes == 0) return FE3D_OK;
    if (cudaFuncSetAttribute(lpc_forward_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, MLP_SMEM) !=
        cudaSuccess)
        return FE3D_ERR_CUDA;
    const int64_t blocks = (nnodes + MLP_THREADS - 1) / MLP_THREADS;
    const int grid = (int)(blocks < kSMs * 8 ? blocks : kSMs * 8);
    lpc_forward_kernel<<<grid, MLP_THREADS, MLP_SMEM, as_stream(stream)>>>(nnodes, feat, weights, out, act);
    FE3D_CHECK_LAUNCH();
    return FE3D_OK;
}

extern "C" int fe3d_lpc_blocks(const fe3d_solver *s, const double *sdiag, const float *out, float out_scale,
                               double *blocks, void *stream) {
    int rc = check_solver(s);
    if (rc) return rc;
    if (s->nnodes > 0 && (!out || !blocks || (s->n > 0 && !sdiag))) return FE3D_ERR_ARG;
    if (s->nnodes == 0) return FE3D_OK;
    const fe3d_pattern *p = s->pat;
    lpc_blocks_kernel<<<lgrid(s->nnodes, 128), 128, 0, as_stream(stream)>>>(
        s->nnodes, s->start, s->size, p->dof_of_row, p->rowptr, p->colind, s->vals, sdiag, out, out_scale, blocks);
    FE3D_CHECK_LAUNCH();
    return FE3D_OK;
}

extern "C" int fe3d_lpc_apply(const fe3d_solver *s, const double *r, double *z, void *stream) {
    if (!s) return FE3D_ERR_ARG;
    if (s->n > 0 && (!r || !z)) return FE3D_ERR_ARG;
    if (s->nnodes == 0) return FE3D_OK;
    lpc_apply_kernel<<<lgrid(s->nnodes, 128), 128, 0, as_stream(stream)>>>(s->nnodes, s->start, s->size, s->Dinv,
                                                                            r, z);
    FE3D_CHECK_LAUNCH();
    return FE3D_OK;
}

extern "C" int fe3d_lpc_loss_grad(const fe3d_solver *s, const double *sdiag, const double *r, const double *z,
                                  const double *Kz, const int8_t *fallback, double inv_er, double factor,
                                  float out_scale, int mode, float *gout, double *acc, void *stream) {
    int rc = check_solver(s);
    if (rc) return rc;
    if (mode != 0 && mode != 1) return FE3D_ERR_ARG;
    if (s->n > 0 && (!sdiag || !r || !z || !Kz || !gout || !acc)) return FE3D_ERR_ARG;
    if (s->nnodes == 0) return FE3D_OK;
    cudaStream_t st = as_stream(stream);
    if (mode == 1) {
        FE3D_CUDA(cudaMemsetAsync(acc + 1, 0, 2 * sizeof(double), st));
        const int64_t g = (s->n + 255) / 256;
        lpc_dots_kernel<<<(int)(g < kSMs * 8 ? g : kSMs * 8), 256, 0, st>>>(s->n, r, z, Kz, acc + 1);
    }
    lpc_grad_kernel<<<lgrid(s->nnodes, 128), 128, 0, st>>>(s->nnodes, s->start, s->size, s->pat->dof_of_row,
                                                          s->Dinv, sdiag, r, z, Kz, fallback, inv_er, factor,
                                                          out_scale, mode, gout, acc);
    FE3D_CHECK_LAUNCH();
    return FE3D_OK;
}

extern "C" int fe3d_lpc_backward(int64_t nnodes, const float *feat, const float *weights, const float *act,
                                 const float *gout, float *delta, float *grad, void *stream) {
    if (nnodes < 0 || (nnodes > 0 && (!feat || !weights || !act || !gout || !delta || !grad))) return FE3D_ERR_ARG;
    if (nnodes == 0) return FE3D_OK;
    cudaStream_t st = as_stream(stream);
    if (cudaFuncSetAttribute(lpc_delta_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, MLP_SMEM) !=
        cudaSuccess)
        return FE3D_ERR_CUDA;
    const int64_t blocks = (nnodes + MLP_THREADS - 1) / MLP_THREADS;
    lpc_delta_kernel<<<(int)(blocks < kSMs * 8 ? blocks : kSMs * 8), MLP_THREADS, MLP_SMEM, st>>>(
        nnodes, weights, act, gout, delta);
    FE3D_CHECK_LAUNCH();
    const int og = lgrid(nnodes, OS_CHUNK);
    // layer 3: d = dL/do, x = h2; layer 2: d = dL/da2, x = h1; layer 1: d = dL/da1, x = features
    lpc_outer_kernel<<<og, OS_THREADS, 0, st>>>(nnodes, NO, NH, delta, ND, act + NH, 2 * NH, grad + OW3, grad + OB3);
    lpc_outer_kernel<<<og, OS_THREADS, 0, st>>>(nnodes, NH, NH, delta + NO, ND, act, 2 * NH, grad + OW2, grad + OB2);
    lpc_outer_kernel<<<og, OS_THREADS, 0, st>>>(nnodes, NH, NF, delta + NO + NH, ND, feat, NF, grad + OW1,
                                                grad + OB1);
    FE3D_CHECK_LAUNCH();
    return FE3D_OK;
}

extern "C" int fe3d_lpc_adam(int64_t nw, float *w, const float *g, float *m, float *v, float lr, float beta1,
                             float beta2, float eps, int step, void *stream) {
    if (nw < 0 || step < 1 || (nw > 0 && (!w || !g || !m || !v))) return FE3D_ERR_ARG;
    if (nw == 0) return FE3D_OK;
    const float c1 = 1.f - powf(beta1, (float)step), c2 = 1.f - powf(beta2, (float)step);
    lpc_adam_kernel<<<lgrid(nw, 256), 256, 0, as_stream(stream)>>>(nw, w, g, m, v, lr, beta1, beta2, eps, c1, c2);
    FE3D_CHECK_LAUNCH();
    return FE3D_OK;
}
