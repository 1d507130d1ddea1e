// Batched block-Jacobi PCG: many independent systems (instances, e.g. one
// plate each) stored together as one block-diagonal reduced CSR matrix, as a
// user of the reference would otherwise solve them one at a time with
// `spsolve(Kuu, fu)` / `cg(Kuu, fu)` (tests/test_quad4_static_point_load.py:102).
//
// Every instance runs its own CG recurrence (own alpha, beta and convergence
// test) in lockstep with the others over one launch per kernel per iteration;
// converged instances are frozen.  Per-instance dot products are accumulated
// with warp-aggregated FP64 atomics, so their summation order (and the last
// bits of the iterates) can differ from run to run.  Iteration chunks are
// captured as CUDA graphs; the host reads the per-instance residuals between
// chunks and confirms convergence on the FP64 residual f - K u.
//
// precision 1: FP32 values of the scaled matrix S^-1 K S^-1 (S = sqrt(diag K)),
// scaled block inverses and search directions with FP64 u and r; every
// `replace_every` iterations the FP64 residual replaces the recurrence
// residual (reliable updates) for every active instance.
//
// The SpMV lanes-per-row count is chosen at setup by timing the candidates
// (4, 8, 16, 32 lanes) on the actual matrix.  The iteration kernels walk
// lists of the rows and nodes of the active instances (in memory order, one
// contiguous chunk per block, per-instance sums kept in registers until the
// instance changes), rebuilt between chunks whenever a quarter of the listed
// instances has finished, so converged plates stop costing bandwidth.
//
// Work split (precision 0): instances whose rows are contiguous and at most
// `split_rows` in number are instead solved each by one thread block of a
// block-resident kernel (bcta_kernel) on a second stream, concurrently with
// the lockstep iterations of the others: the whole PCG recurrence of a small
// plate runs inside one block (block-level reductions in a fixed order, no
// host round trips, no launches per iteration), and the block moves on to
// the next small instance when its plate has converged.
#include <limits.h>
#include <math.h>

#include <type_traits>
#include <vector>

#include "common.cuh"
#include "fe3d_internal.h"

namespace fe3d {
namespace {

constexpr int BS = 256;

template <typename T>
int balloc(T **p, size_t n) {
    if (n == 0) n = 1;
    return cudaMalloc((void **)p, n * sizeof(T)) == cudaSuccess ? 0 : FE3D_ERR_NOMEM;
}

int bgrid(int64_t work, int per_block, int cap) {
    int64_t g = (work + per_block - 1) / per_block;
    if (g < 1) g = 1;
    return (int)(g < cap ? g : cap);
}

// base[inst] += v over the lanes with valid set.  Must be reached by all 32
// lanes of the warp.  Lanes of one instance are summed in the warp first
// (tree when the whole warp belongs to one instance, else a loop over the
// peer group) and one lane per instance commits an FP64 atomic.
__device__ __forceinline__ void warp_atomic_add(double *base, int inst, double v, bool valid) {
    const int key = valid ? inst : -1;
    const unsigned peers = __match_any_sync(0xffffffffu, key);
    if (!valid) return;
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(peers) - 1;
    double acc = v;
    if (peers == 0xffffffffu) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    } else {
        unsigned rest = peers & ~(1u << leader);
        while (rest) {
            const int src = __ffs(rest) - 1;
            rest &= rest - 1;
            const double o = __shfl_sync(peers, v, src);
            if (lane == leader) acc += o;
        }
    }
    if (lane == leader) atomicAdd(base + inst, acc);
}

// Running sum of one instance's contributions per lane, committed with
// warp_atomic_add when any lane of the warp moves on to another instance, and
// by flush() at the end: over contiguous chunks of rows or nodes (every
// instance is a contiguous range of them) a warp commits about one atomic per
// instance it touches instead of one per trip.  Must be reached by whole warps.
struct InstAcc {
    int cur = -1;
    double sum = 0.;
    __device__ __forceinline__ void add(double *base, int inst, double v, bool valid) {
        const bool change = valid && cur >= 0 && inst != cur;
        if (__any_sync(0xffffffffu, change)) {
            warp_atomic_add(base, cur, sum, cur >= 0);
            cur = -1;
            sum = 0.;
        }
        if (valid) {
            cur = inst;
            sum += v;
        }
    }
    __device__ __forceinline__ void flush(double *base) {
        warp_atomic_add(base, cur, sum, cur >= 0);
        cur = -1;
        sum = 0.;
    }
};

// q = K p for rows of active instances; pq[inst] += p.q.  Also clears the
// accumulators the following update kernel fills.  Every thread runs the
// same number of trips so the warp-level reductions see whole warps.
template <typename VT, typename PT, int LPR, bool C16>
__global__ void __launch_bounds__(BS) bspmv_kernel(int64_t n, const int64_t *__restrict__ rowptr,
                                                   const int32_t *__restrict__ colind,
                                                   const int32_t *__restrict__ colbase,
                                                   const uint16_t *__restrict__ col16,
                                                   const VT *__restrict__ vals, const int32_t *__restrict__ inst,
                                                   const int *__restrict__ active, const PT *__restrict__ p,
                                                   PT *__restrict__ q, double *pq, double *clear_a,
                                                   double *clear_b, int64_t ninst, const int32_t *__restrict__ rows,
                                                   const int *__restrict__ nrows) {
    const int64_t gt = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t nth = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = gt; i < ninst; i += nth) {
        clear_a[i] = 0.;
        clear_b[i] = 0.;
    }
    // rows of the instances active at the last compaction, one contiguous
    // chunk per block (the same number of trips in every block)
    const int64_t cnt = *nrows;
    const int lane = threadIdx.x % LPR;
    const int G = blockDim.x / LPR;
    const int64_t per = (cnt + gridDim.x - 1) / gridDim.x;
    const int64_t c0 = blockIdx.x * per, c1 = c0 + per < cnt ? c0 + per : cnt;
    const int64_t trips = (per + G - 1) / G;
    InstAcc apq;
    for (int64_t t = 0; t < trips; t++) {
        const int64_t idx = c0 + t * G + threadIdx.x / LPR;
        const bool in = idx < c1;
        const int64_t row = in ? rows[idx] : 0;
        const int ii = in ? inst[row] : -1;
        const bool act = in && active[ii];
        VT acc = 0;
        if (act) {
            const int32_t base = C16 ? colbase[row] : 0;
            for (int64_t k = rowptr[row] + lane; k < rowptr[row + 1]; k += LPR)
                acc += vals[k] * (VT)p[C16 ? base + (int32_t)col16[k] : colind[k]];
        }
#pragma unroll
        for (int o = LPR / 2; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        const bool lead = act && lane == 0;
        double contrib = 0.;
        if (lead) {
            q[row] = (PT)acc;
            contrib = (double)p[row] * (double)acc;
        }
        apq.add(pq, ii, contrib, lead);
    }
    apq.flush(pq);
}

// Per node of an active instance: alpha = rz/pq; u += alpha p; r -= alpha q;
// z = Dinv r; rz_new[inst] += r.z; rr[inst] += r.r.
template <typename PT>
__global__ void __launch_bounds__(BS) bupdate_kernel(int64_t nnodes, const int32_t *__restrict__ start,
                                                     const int8_t *__restrict__ size,
                                                     const int32_t *__restrict__ node_inst,
                                                     const int *__restrict__ active, const PT *__restrict__ Dinv,
                                                     const double *pq, const double *rz_cur,
                                                     const PT *__restrict__ p, const PT *__restrict__ q, double *u,
                                                     double *r, PT *z, double *rz_new, double *rr,
                                                     const double *__restrict__ sc, const double *__restrict__ isc,
                                                     const int32_t *__restrict__ nodes, const int *__restrict__ nlist) {
    // nodes of the active instances, one contiguous chunk per block
    const int64_t cnt = *nlist;
    const int64_t per = (cnt + gridDim.x - 1) / gridDim.x;
    const int64_t c0 = blockIdx.x * per, c1 = c0 + per < cnt ? c0 + per : cnt;
    const int64_t trips = (per + blockDim.x - 1) / blockDim.x;
    InstAcc arz, arr;
    for (int64_t t = 0; t < trips; t++) {
        const int64_t idx = c0 + t * blockDim.x + threadIdx.x;
        const bool in = idx < c1;
        const int64_t j = in ? nodes[idx] : 0;
        const int ii = in ? node_inst[j] : -1;
        const bool act = ii >= 0 && active[ii];
        double lrz = 0., lrr = 0.;
        if (act) {
            const int s = start[j], b = size[j];
            // a zero p.q (r = 0 met between host checks) leaves the instance unchanged
            const double pqi = pq[ii];
            const double alpha = pqi != 0. ? rz_cur[ii] / pqi : 0.;
            // with sc the recurrence runs on S^-1 K S^-1: p~ = sc p, q~ = K p / sc
            double rl[6], rs[6];
#pragma unroll
            for (int i = 0; i < 6; i++) {
                rl[i] = 0.;
                rs[i] = 0.;
                if (i < b) {
                    double pi = (double)p[s + i], qi = (double)q[s + i];
                    const double iv = sc ? isc[s + i] : 1.;
                    if (sc) {
                        pi *= iv;
                        qi *= sc[s + i];
                    }
                    u[s + i] += alpha * pi;
                    rl[i] = r[s + i] - alpha * qi;
                    r[s + i] = rl[i];
                    rs[i] = sc ? rl[i] * iv : rl[i];
                }
            }
            const PT *D = Dinv + 36 * j;
#pragma unroll
            for (int i = 0; i < 6; i++) {
                if (i < b) {
                    PT acc = 0;
#pragma unroll
                    for (int k = 0; k < 6; k++) acc += D[6 * i + k] * (PT)rs[k];
                    z[s + i] = acc;
                    lrz += rs[i] * (double)acc;
                    lrr += rl[i] * rl[i];
                }
            }
        }
        arz.add(rz_new, ii, lrz, act);
        arr.add(rr, ii, lrr, act);
    }
    arz.flush(rz_new);
    arr.flush(rr);
}

// p = z + (rz_new/rz_old) p for rows of active instances; clears pq.
template <typename PT>
__global__ void __launch_bounds__(BS) bdirection_kernel(int64_t n, const int32_t *__restrict__ inst,
                                                        const int *__restrict__ active, const double *rz_new,
                                                        const double *rz_old, const PT *__restrict__ z, PT *p,
                                                        double *pq_clear, int64_t ninst,
                                                        const int32_t *__restrict__ rows,
                                                        const int *__restrict__ nrows) {
    const int64_t nth = (int64_t)gridDim.x * blockDim.x;
    const int64_t cnt = *nrows;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < cnt; idx += nth) {
        const int64_t i = rows[idx];
        const int ii = inst[i];
        if (!active[ii]) continue;
        const double ro = rz_old[ii];
        const double beta = ro != 0. ? rz_new[ii] / ro : 0.;
        p[i] = beta == 0. ? z[i] : (PT)((double)z[i] + beta * (double)p[i]);
    }
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < ninst; i += nth) pq_clear[i] = 0.;
}

// For flagged instances: z = Dinv r, rz[inst] = r.z (rz cleared first by the
// caller), and p = z when set_p (a restart) or p kept (a residual
// replacement).
template <typename PT>
__global__ void __launch_bounds__(BS) brestart_kernel(int64_t nnodes, const int32_t *__restrict__ start,
                                                      const int8_t *__restrict__ size,
                                                      const int32_t *__restrict__ node_inst,
                                                      const int *__restrict__ flag, const PT *__restrict__ Dinv,
                                                      const double *__restrict__ r, PT *z, PT *p, int set_p,
                                                      double *rz, const double *__restrict__ sc,
                                                      const double *__restrict__ isc) {
    const int64_t nth = (int64_t)gridDim.x * blockDim.x;
    const int64_t trips = (nnodes + nth - 1) / nth;
    for (int64_t t = 0; t < trips; t++) {
        const int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x + t * nth;
        const bool in = j < nnodes;
        const int ii = in ? node_inst[j] : -1;
        const bool act = ii >= 0 && flag[ii];
        double lrz = 0.;
        if (act) {
            const int s = start[j], b = size[j];
            double rl[6];
#pragma unroll
            for (int i = 0; i < 6; i++) rl[i] = i < b ? (sc ? r[s + i] * isc[s + i] : r[s + i]) : 0.;
            const PT *D = Dinv + 36 * j;
            for (int i = 0; i < b; i++) {
                PT acc = 0;
#pragma unroll
                for (int k = 0; k < 6; k++) acc += D[6 * i + k] * (PT)rl[k];
                z[s + i] = acc;
                if (set_p) p[s + i] = acc;
                lrz += rl[i] * (double)acc;
            }
        }
        warp_atomic_add(rz, ii, lrz, act);
    }
}

// r = f - K u (FP64) for rows of flagged instances; rr[inst] += r.r.
template <int LPR>
__global__ void __launch_bounds__(BS) bresidual_kernel(int64_t n, const int64_t *__restrict__ rowptr,
                                                       const int32_t *__restrict__ colind,
                                                       const double *__restrict__ vals,
                                                       const int32_t *__restrict__ inst, const int *__restrict__ flag,
                                                       const double *__restrict__ u, const double *__restrict__ f,
                                                       double *r, double *rr) {
    const int lane = threadIdx.x % LPR;
    const int64_t gt = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t ngroups = (int64_t)gridDim.x * blockDim.x / LPR;
    const int64_t trips = (n + ngroups - 1) / ngroups;
    for (int64_t t = 0; t < trips; t++) {
        const int64_t row = gt / LPR + t * ngroups;
        const bool in = row < n;
        const int ii = in ? inst[row] : -1;
        const bool act = in && flag[ii];
        double acc = 0.;
        if (act)
            for (int64_t k = rowptr[row] + lane; k < rowptr[row + 1]; k += LPR) acc += vals[k] * u[colind[k]];
#pragma unroll
        for (int o = LPR / 2; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        const bool lead = act && lane == 0;
        double contrib = 0.;
        if (lead) {
            const double ri = f[row] - acc;
            r[row] = ri;
            contrib = ri * ri;
        }
        warp_atomic_add(rr, ii, contrib, lead);
    }
}

// ff[inst] += f.f over all rows.
__global__ void __launch_bounds__(BS) bnorm_kernel(int64_t n, const int32_t *__restrict__ inst, const double *f,
                                                   double *ff) {
    const int64_t nth = (int64_t)gridDim.x * blockDim.x;
    const int64_t trips = (n + nth - 1) / nth;
    for (int64_t t = 0; t < trips; t++) {
        const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x + t * nth;
        const bool in = i < n;
        const double v = in ? f[i] : 0.;
        warp_atomic_add(ff, in ? inst[i] : -1, v * v, in);
    }
}

// x[i] = 0 for rows of flagged instances; clear[inst] = 0 for flagged ones.
__global__ void bzero_kernel(int64_t n, const int32_t *inst, const int *flag, double *x, int64_t ninst,
                             double *clear) {
    const int64_t nth = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += nth)
        if (x && flag[inst[i]]) x[i] = 0.;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < ninst; i += nth)
        if (clear && flag[i]) clear[i] = 0.;
}

// list[..] = the indices i < n whose instance is active, in increasing order
// (so the iteration kernels walk rows and nodes in memory order and an
// instance stays contiguous), *count = their number.  Block g owns the items
// [g per, (g + 1) per): pass 1 counts its kept items, one block scans the
// counts, pass 2 writes each block's items at its offset in order.
constexpr int kCompactGrid = kSMs * 8;

__global__ void __launch_bounds__(BS) bcount_kernel(int64_t n, const int32_t *__restrict__ inst,
                                                    const int *__restrict__ active, int *blockcount) {
    __shared__ int wsum[BS / 32];
    const int64_t per = (n + gridDim.x - 1) / gridDim.x;
    const int64_t c0 = blockIdx.x * per, c1 = c0 + per < n ? c0 + per : n;
    int cnt = 0;
    for (int64_t i = c0 + threadIdx.x; i < c1; i += blockDim.x) cnt += active[inst[i]] != 0;
    for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
    if ((threadIdx.x & 31) == 0) wsum[threadIdx.x >> 5] = cnt;
    __syncthreads();
    if (threadIdx.x == 0) {
        int t = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += wsum[w];
        blockcount[blockIdx.x] = t;
    }
}

// exclusive scan of blockcount[0..nb) in place (one block), total into *count
__global__ void __launch_bounds__(BS) bscan_kernel(int nb, int *blockcount, int *count) {
    __shared__ int part[BS];
    const int per = (nb + BS - 1) / BS;
    const int i0 = threadIdx.x * per;
    int s = 0;
    for (int i = i0; i < i0 + per && i < nb; i++) s += blockcount[i];
    part[threadIdx.x] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        int run = 0;
        for (int t = 0; t < BS; t++) {
            const int v = part[t];
            part[t] = run;
            run += v;
        }
        *count = run;
    }
    __syncthreads();
    int run = part[threadIdx.x];
    for (int i = i0; i < i0 + per && i < nb; i++) {
        const int v = blockcount[i];
        blockcount[i] = run;
        run += v;
    }
}

__global__ void __launch_bounds__(BS) bscatter_kernel(int64_t n, const int32_t *__restrict__ inst,
                                                      const int *__restrict__ active, const int *blockoff,
                                                      int32_t *__restrict__ list) {
    __shared__ int wsum[BS / 32];
    const int64_t per = (n + gridDim.x - 1) / gridDim.x;
    const int64_t c0 = blockIdx.x * per, c1 = c0 + per < n ? c0 + per : n;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int base = blockoff[blockIdx.x];
    for (int64_t t0 = c0; t0 < c1; t0 += blockDim.x) {
        const int64_t i = t0 + threadIdx.x;
        const bool keep = i < c1 && active[inst[i]] != 0;
        const unsigned m = __ballot_sync(0xffffffffu, keep);
        if (lane == 0) wsum[warp] = __popc(m);
        __syncthreads();
        int before = 0, total = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) {
            if (w < warp) before += wsum[w];
            total += wsum[w];
        }
        if (keep) list[base + before + __popc(m & ((1u << lane) - 1u))] = (int32_t)i;
        base += total;
        __syncthreads();
    }
}

__global__ void node_inst_kernel(int64_t nnodes, const int32_t *start, const int8_t *size, const int32_t *inst,
                                 int64_t ninst, int32_t *node_inst, int *bad) {
    const int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (j >= nnodes) return;
    const int b = size[j];
    if (b == 0) {
        node_inst[j] = -1;
        return;
    }
    const int s = start[j];
    const int i0 = inst[s];
    int nb = 0;
    for (int i = 0; i < b; i++)
        if (inst[s + i] != i0 || inst[s + i] < 0 || inst[s + i] >= ninst) nb++;
    node_inst[j] = (i0 >= 0 && i0 < ninst) ? i0 : -1;
    if (nb) atomicAdd(bad, nb);
}

// lo[k] / hi[k]: the smallest / largest index i with key[i] = k; cnt[k]:
// how many (keys < 0 are skipped).  lo, hi, cnt start at INT_MAX, -1, 0.
__global__ void inst_range_kernel(int64_t n, const int32_t *key, int32_t *lo, int32_t *hi, int32_t *cnt) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int k = key[i];
    if (k < 0) return;
    atomicMin(lo + k, (int32_t)i);
    atomicMax(hi + k, (int32_t)i);
    atomicAdd(cnt + k, 1);
}

__global__ void inst_range_init_kernel(int64_t k, int32_t *lo, int32_t *hi, int32_t *cnt) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= k) return;
    lo[i] = INT_MAX;
    hi[i] = -1;
    cnt[i] = 0;
}

// ---- block-resident solver of one small instance per block -------------
constexpr int CT = 256;     // threads per block
constexpr int CT_LPR = 4;   // lanes per matrix row

// Block sum in a fixed order (lane 0's warp tree, then the warps in order);
// every thread returns the same total.  Must be reached by the whole block.
__device__ __forceinline__ double cta_sum(double v, double *red) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    __syncthreads();  // the previous use of red is over
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    double t = 0.;
#pragma unroll
    for (int w = 0; w < CT / 32; w++) t += red[w];
    return t;
}

struct CtaArgs {
    const int32_t *list;  // the instances solved here
    int nlist;
    const int32_t *rlo, *rhi, *nlo, *nhi;  // row and node ranges per instance
    const int64_t *rowptr;
    const int32_t *colind;
    const double *vals;
    const int32_t *start;
    const int8_t *size;
    const int32_t *node_inst;
    const double *Dinv;
    const double *f;
    double *u, *r, *z;
    const double *ff;  // f.f per instance
    double tol2;
    int64_t maxiter;
    int *status;
    int64_t *iters;
    int64_t max_rows;  // rows of the largest listed instance (shared-memory vectors)
};

// y = K x over rows [r0, r1]; returns sum(x.y) (or, with f, y = f - K x and
// sum(y.y)).  x and y are indexed from xo and yo (r0 for the instance's
// shared-memory vectors, 0 for the global ones).  Every thread runs the same
// trips (the row groups' shuffles).
__device__ __forceinline__ double cta_rows(const CtaArgs &a, int64_t r0, int64_t r1, const double *x, int64_t xo,
                                           double *y, int64_t yo, const double *f, double *red) {
    const int lane = threadIdx.x % CT_LPR, grp = threadIdx.x / CT_LPR;
    constexpr int NG = CT / CT_LPR;
    double part = 0.;
    for (int64_t b0 = r0; b0 <= r1; b0 += NG) {
        const int64_t row = b0 + grp;
        const bool in = row <= r1;
        double acc = 0.;
        if (in)
            for (int64_t k = a.rowptr[row] + lane; k < a.rowptr[row + 1]; k += CT_LPR)
                acc += a.vals[k] * x[a.colind[k] - xo];
#pragma unroll
        for (int o = CT_LPR / 2; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (in && lane == 0) {
            if (f) {
                const double v = f[row] - acc;
                y[row - yo] = v;
                part += v * v;
            } else {
                y[row - yo] = acc;
                part += x[row - xo] * acc;
            }
        }
    }
    return cta_sum(part, red);
}

// Per node of the instance: u += alpha p, r -= alpha q (when step), then
// z = Dinv r (and p = z when set_p); returns r.z, and r.r into *rr.
__device__ __forceinline__ double cta_nodes(const CtaArgs &a, int inst, int64_t r0, int64_t n0, int64_t n1,
                                            bool step, double alpha, bool set_p, double *ps, const double *qs,
                                            double *rr, double *red) {
    double lrz = 0., lrr = 0.;
    for (int64_t j = n0 + threadIdx.x; j <= n1; j += CT) {
        if (a.node_inst[j] != inst) continue;
        const int s = a.start[j], b = a.size[j];
        double rl[6];
#pragma unroll
        for (int i = 0; i < 6; i++) {
            rl[i] = 0.;
            if (i < b) {
                if (step) {
                    a.u[s + i] += alpha * ps[s + i - r0];
                    a.r[s + i] -= alpha * qs[s + i - r0];
                }
                rl[i] = a.r[s + i];
            }
        }
        const double *D = a.Dinv + 36 * j;
#pragma unroll
        for (int i = 0; i < 6; i++) {
            if (i < b) {
                double acc = 0.;
#pragma unroll
                for (int k = 0; k < 6; k++) acc += D[6 * i + k] * rl[k];
                a.z[s + i] = acc;
                if (set_p) ps[s + i - r0] = acc;
                lrz += rl[i] * acc;
                lrr += rl[i] * rl[i];
            }
        }
    }
    const double rz = cta_sum(lrz, red);
    *rr = cta_sum(lrr, red);
    return rz;
}

// One block per listed instance (the blocks then take the next ones): FP64
// block-Jacobi PCG from the instance's u, convergence confirmed on the FP64
// residual f - K u (a false convergence restarts from it).  status: 0
// converged, 1 iteration cap, 3 non-finite residual.
__global__ void __launch_bounds__(CT) bcta_kernel(CtaArgs a) {
    __shared__ double red[CT / 32];
    // the search direction p and K p of the current instance (rows r0..r1)
    extern __shared__ double vec[];
    double *ps = vec, *qs = vec + a.max_rows;
    for (int li = blockIdx.x; li < a.nlist; li += gridDim.x) {
        const int inst = a.list[li];
        const int64_t r0 = a.rlo[inst], r1 = a.rhi[inst], n0 = a.nlo[inst], n1 = a.nhi[inst];
        const double lim = a.tol2 * a.ff[inst];
        double rr = cta_rows(a, r0, r1, a.u, 0, a.r, 0, a.f, red);
        int status = 1;
        int64_t it = 0;
        if (!(rr == rr) || isinf(rr)) {
            status = 3;
        } else if (rr <= lim) {
            status = 0;
        } else {
            double rr_r;
            double rz = cta_nodes(a, inst, r0, n0, n1, false, 0., true, ps, qs, &rr_r, red);
            while (it < a.maxiter) {
                const double pq = cta_rows(a, r0, r1, ps, r0, qs, r0, nullptr, red);
                const double alpha = pq != 0. ? rz / pq : 0.;
                const double rzn = cta_nodes(a, inst, r0, n0, n1, true, alpha, false, ps, qs, &rr, red);
                it++;
                if (!(rr == rr) || isinf(rr)) {
                    status = 3;
                    break;
                }
                if (rr <= lim) {
                    const double rt = cta_rows(a, r0, r1, a.u, 0, a.r, 0, a.f, red);
                    if (rt <= lim) {
                        status = 0;
                        break;
                    }
                    rz = cta_nodes(a, inst, r0, n0, n1, false, 0., true, ps, qs, &rr_r, red);
                    continue;
                }
                const double beta = rz != 0. ? rzn / rz : 0.;
                rz = rzn;
                for (int64_t i = r0 + threadIdx.x; i <= r1; i += CT) ps[i - r0] = a.z[i] + beta * ps[i - r0];
                __syncthreads();
            }
        }
        if (threadIdx.x == 0) {
            a.status[inst] = status;
            a.iters[inst] = it;
        }
    }
}

// Counts entries that couple two different instances.
__global__ void coupling_kernel(int64_t n, const int64_t *rowptr, const int32_t *colind, const int32_t *inst,
                                int *bad) {
    const int64_t row = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (row >= n) return;
    int nb = 0;
    for (int64_t k = rowptr[row]; k < rowptr[row + 1]; k++) nb += inst[colind[k]] != inst[row];
    if (nb) atomicAdd(bad, nb);
}

}  // namespace
}  // namespace fe3d

using namespace fe3d;

struct fe3d_bsolver {
    fe3d_solver *base = nullptr;  // node blocks, block inverses, work vectors, stream
    int64_t ninst = 0;
    int32_t *inst = nullptr;       // [nrows] instance of each reduced row
    int32_t *node_inst = nullptr;  // [nnodes]
    int *active = nullptr, *flag = nullptr;
    int *bad = nullptr;
    double *pq = nullptr, *rz = nullptr /* [2][ninst] */, *rr = nullptr, *ff = nullptr, *rt = nullptr;
    int lanes[2] = {0, 0};  // autotuned lanes per row [precision]
    int32_t *rowlist = nullptr, *nodelist = nullptr;  // rows / nodes of active instances
    int *lcount = nullptr;                            // [0] rows, [1] nodes in the lists
    int *blockcount = nullptr;                        // compaction scratch [2][kCompactGrid]
    cudaGraphExec_t graph[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};  // [precision][parity]
    int graph_chunk[2][2] = {{0, 0}, {0, 0}};
    // work split: row and node ranges per instance, the rows of the
    // instances whose rows are contiguous (0 otherwise), the size limit, and
    // the block-resident solver's list, results and stream
    int32_t *rlo = nullptr, *rhi = nullptr, *nlo = nullptr, *nhi = nullptr, *rcnt = nullptr, *ncnt = nullptr;
    std::vector<int64_t> contig_rows;
    int64_t split_rows = 0;
    int32_t *cta_list = nullptr;
    int *cta_status = nullptr;
    int64_t *cta_iters = nullptr;
    cudaStream_t cta_stream = nullptr;
    cudaEvent_t cta_start = nullptr, cta_done = nullptr;
};

namespace {

void drop_graphs(fe3d_bsolver *b) {
    for (int i = 0; i < 2; i++)
        for (int j = 0; j < 2; j++)
            if (b->graph[i][j]) {
                cudaGraphExecDestroy(b->graph[i][j]);
                b->graph[i][j] = nullptr;
            }
}

template <typename VT, typename PT>
void launch_bspmv(int lanes, int grid, cudaStream_t st, int64_t n, const fe3d_bsolver *b, const VT *vals,
                  const PT *p, PT *q, double *clear_a, double *clear_b) {
    const fe3d_pattern *pat = b->base->pat;
#define FE3D_BSPMV(L, C)                                                                                      \
    bspmv_kernel<VT, PT, L, C><<<grid, BS, 0, st>>>(n, pat->rowptr, pat->colind, pat->colbase, pat->col16, vals, \
                                                    b->inst, b->active, p, q, b->pq, clear_a, clear_b, b->ninst,   \
                                                    b->rowlist, b->lcount)
    if (pat->col16) {
        switch (lanes) {
            case 4: FE3D_BSPMV(4, true); break;
            case 8: FE3D_BSPMV(8, true); break;
            case 32: FE3D_BSPMV(32, true); break;
            default: FE3D_BSPMV(16, true); break;
        }
    } else {
        switch (lanes) {
            case 4: FE3D_BSPMV(4, false); break;
            case 8: FE3D_BSPMV(8, false); break;
            case 32: FE3D_BSPMV(32, false); break;
            default: FE3D_BSPMV(16, false); break;
        }
    }
#undef FE3D_BSPMV
}

void launch_bresidual(int lanes, int grid, cudaStream_t st, const fe3d_bsolver *b, const double *u,
                      const double *f) {
    const fe3d_solver *s = b->base;
    const fe3d_pattern *pat = s->pat;
#define FE3D_BRES(L) \
    bresidual_kernel<L><<<grid, BS, 0, st>>>(s->n, pat->rowptr, pat->colind, s->vals, b->inst, b->flag, u, f, s->r, b->rt)
    switch (lanes) {
        case 4: FE3D_BRES(4); break;
        case 8: FE3D_BRES(8); break;
        case 32: FE3D_BRES(32); break;
        default: FE3D_BRES(16); break;
    }
#undef FE3D_BRES
}

int spmv_grid_for(int64_t n, int lanes) { return bgrid(n * lanes, BS, kSMs * 8); }

// Lists of the rows and nodes of the instances active now (b->active).
int compact(fe3d_bsolver *b, cudaStream_t st) {
    fe3d_solver *s = b->base;
    FE3D_CUDA(cudaMemsetAsync(b->lcount, 0, 2 * sizeof(int), st));
    const int64_t len[2] = {s->n, s->nnodes};
    const int32_t *key[2] = {b->inst, b->node_inst};
    int32_t *list[2] = {b->rowlist, b->nodelist};
    for (int k = 0; k < 2; k++) {
        if (len[k] <= 0) continue;
        const int g = bgrid(len[k], BS, kCompactGrid);
        int *bc = b->blockcount + k * kCompactGrid;
        bcount_kernel<<<g, BS, 0, st>>>(len[k], key[k], b->active, bc);
        bscan_kernel<<<1, BS, 0, st>>>(g, bc, b->lcount + k);
        bscatter_kernel<<<g, BS, 0, st>>>(len[k], key[k], b->active, bc, list[k]);
    }
    FE3D_CHECK_LAUNCH();
    return FE3D_OK;
}

// Times each lanes-per-row candidate on the matrix (all instances active)
// and keeps the fastest.
template <typename VT, typename PT>
int autotune(fe3d_bsolver *b, const VT *vals, PT *p, PT *q, int *best) {
    fe3d_solver *s = b->base;
    cudaStream_t st = s->stream;
    const int64_t n = s->n, K = b->ninst;
    FE3D_CUDA(cudaMemsetAsync(p, 0, sizeof(PT) * (n ? n : 1), st));
    std::vector<int> ones(K, 1);
    FE3D_CUDA(cudaMemcpyAsync(b->active, ones.data(), sizeof(int) * K, cudaMemcpyHostToDevice, st));
    if (int e = compact(b, st)) return e;
    cudaEvent_t e0, e1;
    FE3D_CUDA(cudaEventCreate(&e0));
    FE3D_CUDA(cudaEventCreate(&e1));
    const int cand[4] = {4, 8, 16, 32};
    float bestms = 1e30f;
    *best = 16;
    int rc = FE3D_OK;
    for (int c = 0; c < 4 && rc == FE3D_OK; c++) {
        const int L = cand[c], g = spmv_grid_for(n, L);
        for (int w = 0; w < 2; w++) launch_bspmv<VT, PT>(L, g, st, n, b, vals, p, q, b->rr, b->rt);
        cudaEventRecord(e0, st);
        for (int w = 0; w < 8; w++) launch_bspmv<VT, PT>(L, g, st, n, b, vals, p, q, b->rr, b->rt);
        cudaEventRecord(e1, st);
        if (cudaGetLastError() != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess) {
            rc = FE3D_ERR_CUDA;
            break;
        }
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms < bestms) {
            bestms = ms;
            *best = L;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return rc;
}

}  // namespace

extern "C" int fe3d_bsolver_free(fe3d_bsolver *b) {
    if (!b) return FE3D_OK;
    drop_graphs(b);
    cudaFree(b->inst); cudaFree(b->node_inst); cudaFree(b->active); cudaFree(b->flag); cudaFree(b->bad);
    cudaFree(b->pq); cudaFree(b->rz); cudaFree(b->rr); cudaFree(b->ff); cudaFree(b->rt);
    cudaFree(b->rowlist); cudaFree(b->nodelist); cudaFree(b->lcount); cudaFree(b->blockcount);
    cudaFree(b->rlo); cudaFree(b->rhi); cudaFree(b->nlo); cudaFree(b->nhi); cudaFree(b->rcnt); cudaFree(b->ncnt);
    cudaFree(b->cta_list); cudaFree(b->cta_status); cudaFree(b->cta_iters);
    if (b->cta_start) cudaEventDestroy(b->cta_start);
    if (b->cta_done) cudaEventDestroy(b->cta_done);
    if (b->cta_stream) cudaStreamDestroy(b->cta_stream);
    fe3d_solver_free(b->base);
    delete b;
    return FE3D_OK;
}

extern "C" int fe3d_bsolver_create(const fe3d_pattern *pat, int block_size, int64_t ninst,
                                   const int32_t *inst_of_row, fe3d_bsolver **out) {
    if (!pat || !out || ninst <= 0 || ninst > INT32_MAX || (pat->nrows > 0 && !inst_of_row)) return FE3D_ERR_ARG;
    *out = nullptr;
    fe3d_bsolver *b = new fe3d_bsolver();
    int rc = fe3d_solver_create(pat, block_size, &b->base);
    if (rc) {
        delete b;
        return rc;
    }
    b->ninst = ninst;
    fe3d_solver *s = b->base;
    const int64_t n = s->n;
    if (balloc(&b->inst, n) || balloc(&b->node_inst, s->nnodes) || balloc(&b->active, ninst) ||
        balloc(&b->flag, ninst) || balloc(&b->bad, 1) || balloc(&b->pq, ninst) || balloc(&b->rz, 2 * ninst) ||
        balloc(&b->rr, ninst) || balloc(&b->ff, ninst) || balloc(&b->rt, ninst) || balloc(&b->rowlist, n) ||
        balloc(&b->nodelist, s->nnodes) || balloc(&b->lcount, 2) || balloc(&b->blockcount, 2 * kCompactGrid) ||
        balloc(&b->rlo, ninst) || balloc(&b->rhi, ninst) || balloc(&b->nlo, ninst) || balloc(&b->nhi, ninst) ||
        balloc(&b->rcnt, ninst) || balloc(&b->ncnt, ninst) || balloc(&b->cta_list, ninst) ||
        balloc(&b->cta_status, ninst) || balloc(&b->cta_iters, ninst)) {
        fe3d_bsolver_free(b);
        return FE3D_ERR_NOMEM;
    }
    cudaStream_t st = s->stream;
    int hbad[2] = {0, 0};
    bool ok = cudaMemsetAsync(b->bad, 0, sizeof(int), st) == cudaSuccess &&
              (n == 0 || cudaMemcpyAsync(b->inst, inst_of_row, sizeof(int32_t) * n, cudaMemcpyDefault, st) ==
                             cudaSuccess);
    if (ok && s->nnodes > 0) {
        node_inst_kernel<<<bgrid(s->nnodes, 256, 1 << 30), 256, 0, st>>>(s->nnodes, s->start, s->size, b->inst,
                                                                         ninst, b->node_inst, b->bad);
        ok = cudaGetLastError() == cudaSuccess;
    }
    ok = ok && cudaMemcpyAsync(&hbad[0], b->bad, sizeof(int), cudaMemcpyDeviceToHost, st) == cudaSuccess &&
         cudaMemsetAsync(b->bad, 0, sizeof(int), st) == cudaSuccess;
    if (ok && n > 0) {
        coupling_kernel<<<bgrid(n, 256, 1 << 30), 256, 0, st>>>(n, pat->rowptr, pat->colind, b->inst, b->bad);
        ok = cudaGetLastError() == cudaSuccess;
    }
    ok = ok && cudaMemcpyAsync(&hbad[1], b->bad, sizeof(int), cudaMemcpyDeviceToHost, st) == cudaSuccess &&
         cudaStreamSynchronize(st) == cudaSuccess;
    if (!ok) {
        fe3d_bsolver_free(b);
        return FE3D_ERR_CUDA;
    }
    if (hbad[0]) {  // instance out of range, or a node split between instances
        fe3d_bsolver_free(b);
        return FE3D_ERR_BOUNDS;
    }
    if (hbad[1]) {  // the matrix couples two instances
        fe3d_bsolver_free(b);
        return FE3D_ERR_ARG;
    }
    // row and node ranges per instance; an instance whose rows are contiguous
    // can go to the block-resident solver (the free rows of a node are
    // consecutive and follow the node order, so its nodes then span a range
    // that holds no node of another instance)
    {
        const int g = bgrid(ninst, 256, 1 << 30);
        inst_range_init_kernel<<<g, 256, 0, st>>>(ninst, b->rlo, b->rhi, b->rcnt);
        inst_range_init_kernel<<<g, 256, 0, st>>>(ninst, b->nlo, b->nhi, b->ncnt);
        if (n > 0) inst_range_kernel<<<bgrid(n, 256, 1 << 30), 256, 0, st>>>(n, b->inst, b->rlo, b->rhi, b->rcnt);
        if (s->nnodes > 0)
            inst_range_kernel<<<bgrid(s->nnodes, 256, 1 << 30), 256, 0, st>>>(s->nnodes, b->node_inst, b->nlo,
                                                                              b->nhi, b->ncnt);
        std::vector<int32_t> lo(ninst), hi(ninst), cnt(ninst);
        ok = cudaGetLastError() == cudaSuccess &&
             cudaMemcpyAsync(lo.data(), b->rlo, sizeof(int32_t) * ninst, cudaMemcpyDeviceToHost, st) == cudaSuccess &&
             cudaMemcpyAsync(hi.data(), b->rhi, sizeof(int32_t) * ninst, cudaMemcpyDeviceToHost, st) == cudaSuccess &&
             cudaMemcpyAsync(cnt.data(), b->rcnt, sizeof(int32_t) * ninst, cudaMemcpyDeviceToHost, st) ==
                 cudaSuccess &&
             cudaStreamSynchronize(st) == cudaSuccess &&
             cudaStreamCreateWithFlags(&b->cta_stream, cudaStreamNonBlocking) == cudaSuccess &&
             cudaEventCreateWithFlags(&b->cta_start, cudaEventDisableTiming) == cudaSuccess &&
             cudaEventCreateWithFlags(&b->cta_done, cudaEventDisableTiming) == cudaSuccess;
        if (!ok) {
            fe3d_bsolver_free(b);
            return FE3D_ERR_CUDA;
        }
        b->contig_rows.assign(ninst, 0);
        for (int64_t i = 0; i < ninst; i++)
            if (cnt[i] > 0 && (int64_t)hi[i] - lo[i] + 1 == cnt[i]) b->contig_rows[i] = cnt[i];
    }
    *out = b;
    return FE3D_OK;
}

extern "C" int fe3d_bsolver_setup(fe3d_bsolver *b, const double *vals, int mixed, int *nonpos_blocks,
                                  void *stream) {
    if (!b) return FE3D_ERR_ARG;
    drop_graphs(b);
    int rc = fe3d_solver_setup(b->base, vals, mixed, nonpos_blocks, stream);
    if (rc) return rc;
    fe3d_solver *s = b->base;
    if (s->n == 0) return FE3D_OK;
    // the private stream must see the block inverses written on the caller's stream
    FE3D_CUDA(cudaEventRecord(s->ev_in, as_stream(stream)));
    FE3D_CUDA(cudaStreamWaitEvent(s->stream, s->ev_in, 0));
    if ((rc = autotune<double, double>(b, s->vals, s->p, s->q, &b->lanes[0]))) return rc;
    if (mixed && (rc = autotune<float, float>(b, s->vals32, s->p32, s->q32, &b->lanes[1]))) return rc;
    return FE3D_OK;
}

extern "C" int fe3d_bsolver_info(const fe3d_bsolver *b, int *lanes_fp64, int *lanes_fp32) {
    if (!b) return FE3D_ERR_ARG;
    if (lanes_fp64) *lanes_fp64 = b->lanes[0];
    if (lanes_fp32) *lanes_fp32 = b->lanes[1];
    return FE3D_OK;
}

extern "C" int fe3d_bsolver_set_split(fe3d_bsolver *b, int64_t max_rows, int64_t *eligible) {
    // the block keeps the instance's p and K p in shared memory
    if (!b || max_rows < 0 || max_rows > FE3D_BSPLIT_MAX_ROWS) return FE3D_ERR_ARG;
    b->split_rows = max_rows;
    if (eligible) {
        int64_t c = 0;
        for (int64_t i = 0; i < b->ninst; i++) c += b->contig_rows[i] > 0 && b->contig_rows[i] <= max_rows;
        *eligible = c;
    }
    return FE3D_OK;
}

namespace {

template <typename VT, typename PT>
int bsolve(fe3d_bsolver *b, double *fu, double *uu, const fe3d_solve_opts *o, int prec, const VT *vals,
           const PT *Dinv, PT *z, PT *p, PT *q, int *status, int64_t *iters, double *relres,
           fe3d_solve_stats *total) {
    // prec 3: nested iterative refinement -- each instance runs inner FP32
    // PCG (the precision-1 data and graphs) from a fresh direction until its
    // recurrence residual has dropped by inner_tol (or replace_every
    // iterations), then an outer FP64 residual and a restart
    const bool nested = prec == 3;
    if (nested) prec = 1;
    const double inner2 = (o->inner_tol > 0. && o->inner_tol < 1.) ? o->inner_tol * o->inner_tol : 1e-4;
    fe3d_solver *s = b->base;
    const int64_t n = s->n, K = b->ninst;
    cudaStream_t st = s->stream;
    const int lanes = b->lanes[prec] ? b->lanes[prec] : 16;
    const double *sck = prec == 1 ? s->sc : nullptr;  // FP32 data hold S^-1 K S^-1 and S Dinv S
    const double *isck = prec == 1 ? s->sc + n : nullptr;
    const int sg = spmv_grid_for(n, lanes), ng = s->node_grid, vg = s->vec_grid;
    std::vector<double> hff(K), hrr(K), hrt(K);
    std::vector<int> hact(K, 0), hflag(K, 0);
    for (int64_t i = 0; i < K; i++) {
        status[i] = 1;
        iters[i] = 0;
    }
    auto upload = [&](int *dst, const std::vector<int> &v) -> int {
        FE3D_CUDA(cudaMemcpyAsync(dst, v.data(), sizeof(int) * K, cudaMemcpyHostToDevice, st));
        return FE3D_OK;
    };
    // FP64 residual of flagged instances into r and rt
    auto true_res = [&](const std::vector<int> &fl) -> int {
        int rc = upload(b->flag, fl);
        if (rc) return rc;
        bzero_kernel<<<vg, BS, 0, st>>>(0, b->inst, b->flag, nullptr, K, b->rt);
        launch_bresidual(b->lanes[0] ? b->lanes[0] : 16, spmv_grid_for(n, b->lanes[0] ? b->lanes[0] : 16), st,
                         b, uu, fu);
        FE3D_CHECK_LAUNCH();
        FE3D_CUDA(cudaMemcpyAsync(hrt.data(), b->rt, sizeof(double) * K, cudaMemcpyDeviceToHost, st));
        FE3D_CUDA(cudaStreamSynchronize(st));
        return FE3D_OK;
    };
    int par = 0;
    // z = Dinv r and rz[par] for flagged instances (already in b->flag);
    // p = z on a restart
    auto precondition = [&](int set_p) -> int {
        bzero_kernel<<<vg, BS, 0, st>>>(0, b->inst, b->flag, nullptr, K, b->rz + par * K);
        brestart_kernel<PT><<<ng, BS, 0, st>>>(s->nnodes, s->start, s->size, b->node_inst, b->flag, Dinv, s->r, z,
                                               p, set_p, b->rz + par * K, sck, isck);
        FE3D_CHECK_LAUNCH();
        return FE3D_OK;
    };
    const double tol2 = o->tol * o->tol;
    // right-hand-side norms; instances with f = 0 get u = 0
    FE3D_CUDA(cudaMemsetAsync(b->ff, 0, sizeof(double) * K, st));
    bnorm_kernel<<<vg, BS, 0, st>>>(n, b->inst, fu, b->ff);
    FE3D_CHECK_LAUNCH();
    FE3D_CUDA(cudaMemcpyAsync(hff.data(), b->ff, sizeof(double) * K, cudaMemcpyDeviceToHost, st));
    FE3D_CUDA(cudaStreamSynchronize(st));
    int rc;
    for (int64_t i = 0; i < K; i++) hflag[i] = hff[i] == 0.;
    if ((rc = upload(b->flag, hflag))) return rc;
    bzero_kernel<<<vg, BS, 0, st>>>(n, b->inst, b->flag, uu, 0, nullptr);
    FE3D_CHECK_LAUNCH();
    int nactive = 0;
    for (int64_t i = 0; i < K; i++) {
        hflag[i] = hff[i] != 0.;
        if (!hflag[i]) status[i] = 0;
    }
    if ((rc = true_res(hflag))) return rc;
    for (int64_t i = 0; i < K; i++) {
        if (!hflag[i]) continue;
        if (!(hrt[i] == hrt[i]) || isinf(hrt[i])) {
            status[i] = 3;
            hflag[i] = 0;
        } else if (hrt[i] <= tol2 * hff[i]) {
            status[i] = 0;  // the initial guess already meets the tolerance
            hflag[i] = 0;
        } else {
            hact[i] = 1;
            nactive++;
        }
    }
    // work split: small contiguous instances to the block-resident solver on
    // its own stream (FP64 only), the rest stay in the lockstep recurrence
    std::vector<int32_t> ctal;
    int64_t cta_rows_max = 0;
    if (prec == 0 && !nested && b->split_rows > 0 && std::is_same<VT, double>::value) {
        for (int64_t i = 0; i < K; i++)
            if (hact[i] && b->contig_rows[i] > 0 && b->contig_rows[i] <= b->split_rows) {
                ctal.push_back((int32_t)i);
                hact[i] = 0;
                nactive--;
                if (b->contig_rows[i] > cta_rows_max) cta_rows_max = b->contig_rows[i];
            }
    }
    if (!ctal.empty()) {
        FE3D_CUDA(cudaMemcpyAsync(b->cta_list, ctal.data(), sizeof(int32_t) * ctal.size(), cudaMemcpyHostToDevice,
                                  st));
        FE3D_CUDA(cudaEventRecord(b->cta_start, st));
        FE3D_CUDA(cudaStreamWaitEvent(b->cta_stream, b->cta_start, 0));
        const fe3d_pattern *pat = s->pat;
        CtaArgs ca{b->cta_list, (int)ctal.size(), b->rlo, b->rhi, b->nlo, b->nhi, pat->rowptr, pat->colind,
                   s->vals, s->start, s->size, b->node_inst, s->Dinv, fu, uu, s->r, s->z, b->ff,
                   tol2, o->maxiter, b->cta_status, b->cta_iters, cta_rows_max};
        const size_t smem = 2 * sizeof(double) * (size_t)cta_rows_max;
        FE3D_CUDA(cudaFuncSetAttribute(bcta_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        int per_sm = 0;
        FE3D_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, bcta_kernel, CT, smem));
        if (per_sm < 1) per_sm = 1;
        const int cap = kSMs * per_sm;
        bcta_kernel<<<(int)ctal.size() < cap ? (int)ctal.size() : cap, CT, smem, b->cta_stream>>>(ca);
        FE3D_CHECK_LAUNCH();
        FE3D_CUDA(cudaEventRecord(b->cta_done, b->cta_stream));
    }
    if ((rc = upload(b->flag, hact))) return rc;
    if ((rc = precondition(1))) return rc;
    FE3D_CUDA(cudaMemsetAsync(b->pq, 0, sizeof(double) * K, st));
    if ((rc = upload(b->active, hact))) return rc;
    if ((rc = compact(b, st))) return rc;
    int compacted_at = nactive;  // active instances when the lists were built
    const int chunk = o->check_every < 2 ? 2 : (int)(o->check_every & ~1);
    auto launch_iteration = [&](int pr) {
        double *rz_cur = b->rz + pr * K, *rz_nxt = b->rz + (pr ^ 1) * K;
        launch_bspmv<VT, PT>(lanes, sg, st, n, b, vals, p, q, rz_nxt, b->rr);
        bupdate_kernel<PT><<<ng, BS, 0, st>>>(s->nnodes, s->start, s->size, b->node_inst, b->active, Dinv, b->pq,
                                              rz_cur, p, q, uu, s->r, z, rz_nxt, b->rr, sck, isck, b->nodelist,
                                              b->lcount + 1);
        bdirection_kernel<PT><<<vg, BS, 0, st>>>(n, b->inst, b->active, rz_nxt, rz_cur, z, p, b->pq, K, b->rowlist,
                                                 b->lcount);
    };
    int64_t it = 0, since = 0, replacements = 0;
    std::vector<double> last_rt(K, 0.);
    std::vector<int> stall(K, 0);
    std::vector<double> rr_start(hrt);       // nested: FP64 residual at the instance's last restart
    std::vector<int64_t> it_start(K, 0);     // nested: iteration of that restart
    while (nactive > 0 && it < o->maxiter) {
        const int len = (int)((o->maxiter - it) < chunk ? (o->maxiter - it) : chunk);
        if (len == chunk) {
            cudaGraphExec_t &ge = b->graph[prec][par];
            if (!ge || b->graph_chunk[prec][par] != chunk) {
                if (ge) cudaGraphExecDestroy(ge);
                ge = nullptr;
                cudaGraph_t g = nullptr;
                FE3D_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
                for (int i = 0, pr = par; i < chunk; i++, pr ^= 1) launch_iteration(pr);
                FE3D_CUDA(cudaStreamEndCapture(st, &g));
                const cudaError_t e = cudaGraphInstantiate(&ge, g, 0);
                cudaGraphDestroy(g);
                if (e != cudaSuccess) {
                    ge = nullptr;
                    return FE3D_ERR_CUDA;
                }
                b->graph_chunk[prec][par] = chunk;
            }
            FE3D_CUDA(cudaGraphLaunch(ge, st));
        } else {
            for (int i = 0, pr = par; i < len; i++, pr ^= 1) launch_iteration(pr);
            if (len & 1) par ^= 1;
        }
        FE3D_CHECK_LAUNCH();
        it += len;
        since += len;
        FE3D_CUDA(cudaMemcpyAsync(hrr.data(), b->rr, sizeof(double) * K, cudaMemcpyDeviceToHost, st));
        FE3D_CUDA(cudaStreamSynchronize(st));
        const bool replace = prec == 1 && !nested && o->replace_every > 0 && since >= o->replace_every;
        std::vector<int> check(K, 0);
        int ncheck = 0;
        for (int64_t i = 0; i < K; i++) {
            if (!hact[i]) continue;
            if (!(hrr[i] == hrr[i]) || isinf(hrr[i])) {
                hact[i] = 0;
                status[i] = 3;
                iters[i] = it;
                nactive--;
            } else if (replace || hrr[i] <= tol2 * hff[i] ||
                       (nested && (hrr[i] <= inner2 * rr_start[i] ||
                                   (o->replace_every > 0 && it - it_start[i] >= o->replace_every)))) {
                check[i] = 1;
                ncheck++;
            }
        }
        if (ncheck) {
            if ((rc = true_res(check))) return rc;
            for (int64_t i = 0; i < K; i++) {
                if (!check[i]) continue;
                if (hrt[i] <= tol2 * hff[i]) {
                    hact[i] = 0;
                    status[i] = 0;
                    iters[i] = it;
                    nactive--;
                    check[i] = 0;
                }
            }
            // mixed precision: an instance whose FP64 residual has not
            // dropped below 0.9x of the previous replacement's three times in
            // a row stagnates (kappa * eps32 too large for FP32 directions):
            // status 4, left for an FP64 solve
            if (replace || nested)
                for (int64_t i = 0; i < K; i++) {
                    if (!check[i]) continue;
                    stall[i] = (last_rt[i] > 0. && hrt[i] > 0.81 * last_rt[i]) ? stall[i] + 1 : 0;
                    last_rt[i] = hrt[i];
                    if (stall[i] >= 3) {
                        hact[i] = 0;
                        status[i] = 4;
                        iters[i] = it;
                        nactive--;
                        check[i] = 0;
                    }
                }
            // the rest continue from the FP64 residual: a replacement keeps
            // the direction, a false convergence restarts
            if ((rc = upload(b->flag, check))) return rc;
            if ((rc = precondition(replace ? 0 : 1))) return rc;
            if (nested) {
                for (int64_t i = 0; i < K; i++)
                    if (check[i]) {
                        rr_start[i] = hrt[i];
                        it_start[i] = it;
                        replacements++;
                    }
            }
            if (replace) {
                replacements++;
                since = 0;
            }
        }
        if ((rc = upload(b->active, hact))) return rc;
        // drop the rows of finished instances from the lists once a quarter
        // of the listed instances has finished
        if (nactive > 0 && 4 * nactive <= 3 * compacted_at) {
            if ((rc = compact(b, st))) return rc;
            compacted_at = nactive;
        }
    }
    for (int64_t i = 0; i < K; i++)
        if (hact[i]) iters[i] = it;
    int64_t it_all = it;
    if (!ctal.empty()) {
        FE3D_CUDA(cudaStreamWaitEvent(st, b->cta_done, 0));
        std::vector<int> cs(K);
        std::vector<int64_t> ci(K);
        FE3D_CUDA(cudaMemcpyAsync(cs.data(), b->cta_status, sizeof(int) * K, cudaMemcpyDeviceToHost, st));
        FE3D_CUDA(cudaMemcpyAsync(ci.data(), b->cta_iters, sizeof(int64_t) * K, cudaMemcpyDeviceToHost, st));
        FE3D_CUDA(cudaStreamSynchronize(st));
        for (int32_t i : ctal) {
            status[i] = cs[i];
            iters[i] = ci[i];
            if (ci[i] > it_all) it_all = ci[i];
        }
    }
    std::vector<int> all(K, 1);
    if ((rc = true_res(all))) return rc;
    total->status = 0;
    total->iterations = it_all;
    total->replacements = replacements;
    double worst = 0.;
    for (int64_t i = 0; i < K; i++) {
        const double rel = hff[i] > 0. ? sqrt(hrt[i] / hff[i]) : 0.;
        if (hact[i]) status[i] = rel <= o->tol ? 0 : 1;
        if (status[i] > total->status) total->status = status[i];
        if (rel > worst || !(rel == rel)) worst = rel;
        relres[i] = rel;
    }
    total->relres = worst;
    return FE3D_OK;
}

}  // namespace

extern "C" int fe3d_bsolver_solve(fe3d_bsolver *b, const double *f, double *u, const fe3d_solve_opts *o,
                                  int *inst_status, int64_t *inst_iters, double *inst_relres,
                                  fe3d_solve_stats *total, void *stream) {
    if (!b || !o || !total) return FE3D_ERR_ARG;
    fe3d_solver *s = b->base;
    if (s->n > 0 && (!f || !u)) return FE3D_ERR_ARG;
    if (!s->ready) return FE3D_ERR_STATE;
    if (!(o->tol > 0) || o->maxiter < 0 || (o->precision != 0 && o->precision != 1 && o->precision != 3))
        return FE3D_ERR_ARG;
    if ((o->precision == 1 || o->precision == 3) && !s->have32) return FE3D_ERR_STATE;
    const int64_t n = s->n, K = b->ninst;
    cudaStream_t caller = as_stream(stream), st = s->stream;
    FE3D_CUDA(cudaEventRecord(s->ev_in, caller));
    FE3D_CUDA(cudaStreamWaitEvent(st, s->ev_in, 0));
    const size_t bytes = sizeof(double) * (size_t)n;
    if (n) {
        FE3D_CUDA(cudaMemcpyAsync(s->fin, f, bytes, cudaMemcpyDeviceToDevice, st));
        FE3D_CUDA(cudaMemcpyAsync(s->uin, u, bytes, cudaMemcpyDeviceToDevice, st));
    }
    std::vector<int> status(K);
    std::vector<int64_t> iters(K);
    std::vector<double> relres(K);
    int rc;
    if (o->precision == 1 || o->precision == 3)
        rc = bsolve<float, float>(b, s->fin, s->uin, o, o->precision, s->vals32, s->Dinv32, s->z32, s->p32,
                                  s->q32, status.data(), iters.data(), relres.data(), total);
    else
        rc = bsolve<double, double>(b, s->fin, s->uin, o, 0, s->vals, s->Dinv, s->z, s->p, s->q, status.data(),
                                    iters.data(), relres.data(), total);
    if (rc) return rc;
    for (int64_t i = 0; i < K; i++) {
        if (inst_status) inst_status[i] = status[i];
        if (inst_iters) inst_iters[i] = iters[i];
        if (inst_relres) inst_relres[i] = relres[i];
    }
    if (n) FE3D_CUDA(cudaMemcpyAsync(u, s->uin, bytes, cudaMemcpyDeviceToDevice, st));
    FE3D_CUDA(cudaEventRecord(s->ev_out, st));
    FE3D_CUDA(cudaStreamWaitEvent(caller, s->ev_out, 0));
    return FE3D_OK;
}
