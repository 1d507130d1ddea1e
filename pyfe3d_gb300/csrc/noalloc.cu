// Allocation-free Jacobi-preconditioned CG on a caller-provided CSR matrix.
//
// For callers that cannot allocate device memory themselves -- for example a
// host application whose device memory is owned by another runtime's pool,
// or code that runs where a cudaMalloc would synchronise or fail -- this
// entry point solves K u = f with the caller's CSR arrays and vectors only.
// Its working vectors live in one file-scope __device__ array of fixed size
// (FE3D_NOALLOC_MAX_ROWS rows), which every GPU that loads the library keeps
// until the process exits.  No cudaMalloc, cudaFree or allocating library
// routine is called.
//
// Shared-state rules: every call uses the same array, so calls that overlap
// on the GPU (concurrent streams, or several host threads) race and must be
// serialised by the caller.  The array keeps the last call's contents; each
// call initialises everything it reads (the scalars are cleared, the
// vectors are written before they are read).  The first call on a device
// looks up the array's device address with cudaGetSymbolAddress while that
// device is current and keeps it for the life of the process; make that first
// call before any stream capture, and do not use this entry point after a
// cudaDeviceReset (the kept address would be stale).
#include "common.cuh"

namespace fe3d {
namespace {

constexpr int64_t kMaxRows = FE3D_NOALLOC_MAX_ROWS;
constexpr int kParts = 1216;  // per-block partial sums (grid cap)
constexpr int kBS = 256;
constexpr int kLanes = 16;    // lanes per CSR row

// r, z, p, q, dinv [kMaxRows] | partials pq, rz (two buffers), rr [kParts] | scalars [8]
constexpr size_t kScratch = 5 * (size_t)kMaxRows + 4 * (size_t)kParts + 8;
static __device__ __align__(256) double g_noalloc_scratch[kScratch];

double *g_scratch_addr[64] = {nullptr};

__device__ __forceinline__ double nblock_sum(double v, double *sh) {
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
    return s;
}

__device__ __forceinline__ double nreduce(const double *partials, int n, double *sh) {
    double v = 0.;
    for (int i = threadIdx.x; i < n; i += blockDim.x) v += partials[i];
    v = nblock_sum(v, sh);
    __syncthreads();
    if (threadIdx.x == 0) sh[32] = v;
    __syncthreads();
    return sh[32];
}

// r = f - K u, dinv = 1 / diag(K); partial r.r
__global__ void __launch_bounds__(kBS) na_residual(int64_t n, const int64_t *rowptr, const int32_t *colind,
                                                    const double *vals, const double *u, const double *f,
                                                    double *r, double *dinv, double *prr) {
    __shared__ double sh[34];
    const int lane = threadIdx.x % kLanes;
    const int64_t g = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) / kLanes;
    const int64_t ng = (int64_t)gridDim.x * blockDim.x / kLanes;
    double rr = 0.;
    // every lane runs the same number of trips: the full-warp shuffles below
    // must never wait for lanes that have left the loop
    const int64_t trips = (n + ng - 1) / ng;
    for (int64_t t = 0; t < trips; t++) {
        const int64_t row = g + t * ng;
        const bool in = row < n;
        double acc = 0., d = 0.;
        if (in)
            for (int64_t k = rowptr[row] + lane; k < rowptr[row + 1]; k += kLanes) {
                const int32_t c = colind[k];
                acc += vals[k] * u[c];
                if (c == row) d += vals[k];  // duplicate diagonal entries are summed like the SpMV sums them
            }
        for (int o = kLanes / 2; o > 0; o >>= 1) {
            acc += __shfl_xor_sync(0xffffffffu, acc, o);
            d += __shfl_xor_sync(0xffffffffu, d, o);
        }
        if (in && lane == 0) {
            const double ri = f[row] - acc;
            r[row] = ri;
            dinv[row] = d != 0. ? 1. / d : 1.;
            rr += ri * ri;
        }
    }
    const double s = nblock_sum(rr, sh);
    if (threadIdx.x == 0) prr[blockIdx.x] = s;
}

// z = dinv r; p = z (restart); partial r.z
__global__ void __launch_bounds__(kBS) na_restart(int64_t n, const double *r, const double *dinv, double *z,
                                                   double *p, double *prz) {
    __shared__ double sh[34];
    double rz = 0.;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double zi = dinv[i] * r[i];
        z[i] = zi;
        p[i] = zi;
        rz += r[i] * zi;
    }
    const double s = nblock_sum(rz, sh);
    if (threadIdx.x == 0) prz[blockIdx.x] = s;
}

// q = K p; partial p.q
__global__ void __launch_bounds__(kBS) na_spmv(int64_t n, const int64_t *rowptr, const int32_t *colind,
                                                const double *vals, const double *p, double *q, double *ppq) {
    __shared__ double sh[34];
    const int lane = threadIdx.x % kLanes;
    const int64_t g = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) / kLanes;
    const int64_t ng = (int64_t)gridDim.x * blockDim.x / kLanes;
    double dot = 0.;
    const int64_t trips = (n + ng - 1) / ng;  // uniform: full-warp shuffles below
    for (int64_t t = 0; t < trips; t++) {
        const int64_t row = g + t * ng;
        const bool in = row < n;
        double acc = 0.;
        if (in)
            for (int64_t k = rowptr[row] + lane; k < rowptr[row + 1]; k += kLanes) acc += vals[k] * p[colind[k]];
        for (int o = kLanes / 2; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (in && lane == 0) {
            q[row] = acc;
            dot += p[row] * acc;
        }
    }
    const double s = nblock_sum(dot, sh);
    if (threadIdx.x == 0) ppq[blockIdx.x] = s;
}

// alpha = rz / pq; u += alpha p; r -= alpha q; z = dinv r; partial r.z, r.r
__global__ void __launch_bounds__(kBS) na_update(int64_t n, const double *ppq, int npq, const double *prz_old,
                                                  int nrz, double *u, double *r, double *z, const double *p,
                                                  const double *q, const double *dinv, double *prz, double *prr,
                                                  double *scal) {
    __shared__ double sh[34];
    const double pq = nreduce(ppq, npq, sh);
    const double rz = nreduce(prz_old, nrz, sh);
    // p.q = 0 only when p = 0 (r reached exactly zero): no step
    const double alpha = pq != 0. ? rz / pq : 0.;
    if (blockIdx.x == 0 && threadIdx.x == 0) scal[0] = rz;
    __syncthreads();
    double rzn = 0., rrn = 0.;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        u[i] += alpha * p[i];
        const double ri = r[i] - alpha * q[i];
        r[i] = ri;
        const double zi = dinv[i] * ri;
        z[i] = zi;
        rzn += ri * zi;
        rrn += ri * ri;
    }
    double s1 = nblock_sum(rzn, sh);
    __syncthreads();
    double s2 = nblock_sum(rrn, sh);
    if (threadIdx.x == 0) {
        prz[blockIdx.x] = s1;
        prr[blockIdx.x] = s2;
    }
}

// beta = rz_new / rz_old; p = z + beta p; scal[1] = r.r
__global__ void __launch_bounds__(kBS) na_direction(int64_t n, const double *prz, const double *prr, int np,
                                                     const double *scal_in, double *p, const double *z,
                                                     double *rr_out) {
    __shared__ double sh[34];
    const double rzn = nreduce(prz, np, sh);
    const double rrn = nreduce(prr, np, sh);
    const double beta = scal_in[0] != 0. ? rzn / scal_in[0] : 0.;
    if (blockIdx.x == 0 && threadIdx.x == 0) *rr_out = rrn;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        p[i] = z[i] + beta * p[i];
}

// partial a.b
__global__ void __launch_bounds__(kBS) na_dot(int64_t n, const double *a, const double *b, double *part) {
    __shared__ double sh[34];
    double v = 0.;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        v += a[i] * b[i];
    const double t = nblock_sum(v, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = t;
}

__global__ void na_sum(const double *partials, int n, double *out) {
    __shared__ double sh[34];
    const double v = nreduce(partials, n, sh);
    if (threadIdx.x == 0) *out = v;
}

int grid_of(int64_t work) {
    int64_t g = (work + kBS - 1) / kBS;
    if (g < 1) g = 1;
    return (int)(g < kParts ? g : kParts);
}

}  // namespace
}  // namespace fe3d

using namespace fe3d;

extern "C" int64_t fe3d_noalloc_max_rows(void) { return FE3D_NOALLOC_MAX_ROWS; }

extern "C" int fe3d_jacobi_pcg_noalloc(int64_t n, const int64_t *rowptr, const int32_t *colind,
                                       const double *vals, const double *f, double *u,
                                       const fe3d_solve_opts *o, fe3d_solve_stats *stats, void *stream) {
    if (!o || !stats || n < 0) return FE3D_ERR_ARG;
    if (n > FE3D_NOALLOC_MAX_ROWS) return FE3D_ERR_TOO_LARGE;
    if (n > 0 && (!rowptr || !colind || !vals || !f || !u)) return FE3D_ERR_ARG;
    if (!(o->tol > 0) || o->maxiter < 0) return FE3D_ERR_ARG;
    stats->iterations = 0;
    stats->replacements = 0;
    stats->relres = 0.;
    stats->status = 0;
    if (n == 0) return FE3D_OK;
    // one-time set-up per device: device address of the file-scope array
    int dev = 0;
    FE3D_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) return FE3D_ERR_ARG;
    if (!g_scratch_addr[dev]) {
        void *ptr = nullptr;
        if (cudaGetSymbolAddress(&ptr, g_noalloc_scratch) != cudaSuccess || !ptr) return FE3D_ERR_CUDA;
        g_scratch_addr[dev] = static_cast<double *>(ptr);
    }
    double *base = g_scratch_addr[dev];
    double *r = base, *z = r + kMaxRows, *p = z + kMaxRows, *q = p + kMaxRows, *dinv = q + kMaxRows;
    double *ppq = dinv + kMaxRows, *prz_a = ppq + kParts, *prz_b = prz_a + kParts, *prr = prz_b + kParts;
    double *scal = prr + kParts;  // [0] rz, [1] r.r (recurrence), [2] r.r (true), [3] f.f
    cudaStream_t st = as_stream(stream);
    FE3D_CUDA(cudaMemsetAsync(scal, 0, 8 * sizeof(double), st));
    const int gs = grid_of(n * kLanes), gv = grid_of(n);
    double ff = 0., rr = 0.;
    na_dot<<<gv, kBS, 0, st>>>(n, f, f, prr);
    na_sum<<<1, kBS, 0, st>>>(prr, gv, scal + 3);
    FE3D_CHECK_LAUNCH();
    FE3D_CUDA(cudaMemcpyAsync(&ff, scal + 3, sizeof(double), cudaMemcpyDeviceToHost, st));
    FE3D_CUDA(cudaStreamSynchronize(st));
    if (ff == 0.) {
        if (n) FE3D_CUDA(cudaMemsetAsync(u, 0, sizeof(double) * n, st));
        FE3D_CUDA(cudaStreamSynchronize(st));
        return FE3D_OK;
    }
    const double target = o->tol * o->tol * ff;
    // true residual and Jacobi inverse; returns ||r||^2 on the host
    auto true_residual = [&](double *out) -> int {
        na_residual<<<gs, kBS, 0, st>>>(n, rowptr, colind, vals, u, f, r, dinv, prr);
        na_sum<<<1, kBS, 0, st>>>(prr, gs, scal + 2);
        FE3D_CHECK_LAUNCH();
        FE3D_CUDA(cudaMemcpyAsync(out, scal + 2, sizeof(double), cudaMemcpyDeviceToHost, st));
        FE3D_CUDA(cudaStreamSynchronize(st));
        return FE3D_OK;
    };
    int rc = true_residual(&rr);
    if (rc) return rc;
    double *prz_old = prz_a, *prz_new = prz_b;
    na_restart<<<gv, kBS, 0, st>>>(n, r, dinv, z, p, prz_old);
    FE3D_CHECK_LAUNCH();
    const int check = o->check_every > 0 ? o->check_every : 50;
    int64_t it = 0;
    stats->status = 1;
    if (!(rr == rr)) stats->status = 3;
    else if (rr <= target) stats->status = 0;
    while (stats->status == 1 && it < o->maxiter) {
        const int64_t end = it + check < o->maxiter ? it + check : o->maxiter;
        for (; it < end; it++) {
            na_spmv<<<gs, kBS, 0, st>>>(n, rowptr, colind, vals, p, q, ppq);
            na_update<<<gv, kBS, 0, st>>>(n, ppq, gs, prz_old, gv, u, r, z, p, q, dinv, prz_new, prr, scal);
            na_direction<<<gv, kBS, 0, st>>>(n, prz_new, prr, gv, scal, p, z, scal + 1);
            double *t = prz_old;
            prz_old = prz_new;
            prz_new = t;
        }
        FE3D_CHECK_LAUNCH();
        FE3D_CUDA(cudaMemcpyAsync(&rr, scal + 1, sizeof(double), cudaMemcpyDeviceToHost, st));
        FE3D_CUDA(cudaStreamSynchronize(st));
        if (!(rr == rr) || isinf(rr)) {
            stats->status = 3;
            break;
        }
        if (rr <= target) {
            // confirm on the true residual; restart from it if it drifted
            double rt = 0.;
            if ((rc = true_residual(&rt))) return rc;
            if (rt <= target) {
                stats->status = 0;
                break;
            }
            stats->replacements++;
            na_restart<<<gv, kBS, 0, st>>>(n, r, dinv, z, p, prz_old);
            FE3D_CHECK_LAUNCH();
        }
    }
    double rt = 0.;
    if ((rc = true_residual(&rt))) return rc;
    stats->iterations = it;
    stats->relres = sqrt(rt / ff);
    if (stats->status != 3) stats->status = (rt <= target) ? 0 : 1;
    return FE3D_OK;
}
