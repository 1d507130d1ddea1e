// COO -> CSR assembly with boundary-condition elimination.
//
// Replaces the caller-side `coo_matrix((v, (r, c))).tocsc()` followed by
// `K[bu, :][:, bu]` of the reference's tests
// (tests/test_quad4_static_point_load.py:80-99).
//
// Pattern (once per mesh): every COO slot whose row and column are free DOFs
// gets the key (row', col') in the reduced numbering; keys are radix-sorted
// together with the slot index, equal keys form a segment, and the segment
// heads give the CSR row pointer and column indices.  The pattern keeps the
// sorted slot permutation `perm` and the segment starts `seg`.
// Numeric assembly (every update): vals[s] = sum of Kv[perm[t]] over the
// segment t in [seg[s], seg[s+1]), summed in ascending slot order, so the
// result is deterministic.
#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>

#include "common.cuh"
#include "fe3d_internal.h"

namespace fe3d {
namespace {

__global__ void free_flags_kernel(int64_t N, const uint8_t *fixed, int32_t *flag) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < N) flag[i] = fixed ? (fixed[i] ? 0 : 1) : 1;
}

__global__ void reduced_index_kernel(int64_t N, const int32_t *flag, const int32_t *scan,
                                     int32_t *row_of_dof, int64_t *dof_of_row) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= N) return;
    if (flag[i]) {
        row_of_dof[i] = scan[i];
        dof_of_row[scan[i]] = i;
    } else {
        row_of_dof[i] = -1;
    }
}

__global__ void coo_keys_kernel(int64_t nnz, const int64_t *Kr, const int64_t *Kc, int64_t N,
                                const int32_t *row_of_dof, int64_t nfree, uint64_t *keys,
                                int32_t *idx, int *err) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= nnz) return;
    const int64_t r = Kr[t], c = Kc[t];
    uint64_t key = ~0ull;
    if (r < 0 || c < 0 || r >= N || c >= N) {
        raise_error(err, kErrBounds);
    } else {
        const int32_t rr = row_of_dof[r], cc = row_of_dof[c];
        if (rr >= 0 && cc >= 0) key = (uint64_t)rr * (uint64_t)nfree + (uint64_t)cc;
    }
    keys[t] = key;
    idx[t] = (int32_t)t;
}

__global__ void head_flags_kernel(int64_t nnz, const uint64_t *keys, int32_t *head) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= nnz) return;
    const uint64_t k = keys[t];
    head[t] = (k != ~0ull && (t == 0 || keys[t - 1] != k)) ? 1 : 0;
}

__global__ void segments_kernel(int64_t nnz, const uint64_t *keys, const int32_t *head,
                                const int32_t *hscan, int64_t nfree, int32_t *seg,
                                int32_t *colind, int32_t *row_count) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= nnz) return;
    if (head[t]) {
        const int32_t s = hscan[t];
        const uint64_t k = keys[t];
        seg[s] = (int32_t)t;
        colind[s] = (int32_t)(k % (uint64_t)nfree);
        atomicAdd(row_count + (k / (uint64_t)nfree), 1);
    }
}

__global__ void seg_end_kernel(int64_t nnz_valid, int64_t nseg, int32_t *seg) {
    seg[nseg] = (int32_t)nnz_valid;
}

__global__ void count_valid_kernel(int64_t nnz, const uint64_t *keys, unsigned long long *cnt) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t < nnz && keys[t] != ~0ull) atomicAdd(cnt, 1ull);
}

// Per row: the first (smallest) column as the base and 16-bit offsets of the
// row's columns from it; too_wide is set when a row spans 65,536 columns or more.
__global__ void col16_kernel(int64_t n, const int64_t *rowptr, const int32_t *colind, int32_t *colbase,
                             uint16_t *col16, int *too_wide) {
    const int64_t row = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (row >= n) return;
    const int64_t k0 = rowptr[row], k1 = rowptr[row + 1];
    const int32_t base = k1 > k0 ? colind[k0] : 0;
    colbase[row] = base;
    if (k1 > k0 && (int64_t)colind[k1 - 1] - base > 65535) {
        atomicOr(too_wide, 1);
        return;
    }
    for (int64_t k = k0; k < k1; k++) col16[k] = (uint16_t)(colind[k] - base);
}

__global__ void rowptr_kernel(int64_t n, const int64_t *scan, int64_t *rowptr, int64_t total) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) rowptr[i] = scan[i];
    if (i == n) rowptr[n] = total;
}

__global__ void widen_kernel(int64_t n, const int32_t *a, int64_t *b) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) b[i] = a[i];
}

// Numeric assembly: one thread per CSR entry (segment).
__global__ void __launch_bounds__(256) assemble_kernel(int64_t nseg, const int32_t *__restrict__ seg,
                                                       const int32_t *__restrict__ perm,
                                                       const double *__restrict__ Kv,
                                                       double *__restrict__ vals) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < nseg; s += stride) {
        const int32_t b = __ldg(seg + s), e = __ldg(seg + s + 1);
        double acc = 0.;
        for (int32_t t = b; t < e; t++) acc += __ldg(Kv + __ldg(perm + t));
        vals[s] = acc;
    }
}

template <typename T>
int dalloc(T **p, size_t n) {
    if (n == 0) n = 1;
    return cudaMalloc((void **)p, n * sizeof(T)) == cudaSuccess ? 0 : FE3D_ERR_NOMEM;
}

inline unsigned nblk(int64_t n, int bs = 256) { return (unsigned)((n + bs - 1) / bs > 0 ? (n + bs - 1) / bs : 1); }

}  // namespace
}  // namespace fe3d

using namespace fe3d;

extern "C" int fe3d_pattern_build(const int64_t *Kr, const int64_t *Kc, int64_t nnz_in, int64_t N,
                                  const uint8_t *fixed, fe3d_pattern **out, int *err, void *stream) {
    if (!out || nnz_in < 0 || N <= 0 || (nnz_in > 0 && (!Kr || !Kc))) return FE3D_ERR_ARG;
    if (nnz_in >= (int64_t)INT32_MAX || N >= (int64_t)INT32_MAX) return FE3D_ERR_ARG;
    *out = nullptr;
    cudaStream_t st = as_stream(stream);
    fe3d_pattern *p = new fe3d_pattern();
    p->N = N;
    p->nnz_in = nnz_in;
    int rc = 0;
    int32_t *flag = nullptr, *scan = nullptr, *idx = nullptr, *head = nullptr, *hscan = nullptr;
    int32_t *row_count = nullptr;
    int64_t *rc64 = nullptr, *rscan = nullptr;
    uint64_t *keys = nullptr, *keys_sorted = nullptr;
    void *tmp = nullptr;
    size_t tmp_bytes = 0, need = 0;
    unsigned long long *dcount = nullptr;
    int *wide = nullptr;
    int hwide = 0;
    unsigned long long hcount = 0;
    int32_t nfree32 = 0, nseg32 = 0, last_head = 0, last_hscan = 0;
    int32_t last_flag = 0, last_scan = 0;
#define TRY(x)                  \
    do {                        \
        rc = (x);               \
        if (rc) goto fail;      \
    } while (0)
#define TRYC(x)                                     \
    do {                                            \
        if ((x) != cudaSuccess) {                   \
            rc = FE3D_ERR_CUDA;                     \
            goto fail;                              \
        }                                           \
    } while (0)
    // reduced numbering of the free DOFs
    TRY(dalloc(&flag, N));
    TRY(dalloc(&scan, N));
    TRY(dalloc(&p->row_of_dof, N));
    free_flags_kernel<<<nblk(N), 256, 0, st>>>(N, fixed, flag);
    TRYC(cub::DeviceScan::ExclusiveSum(nullptr, need, flag, scan, (int)N, st));
    tmp_bytes = need;
    TRYC(cudaMalloc(&tmp, tmp_bytes));
    TRYC(cub::DeviceScan::ExclusiveSum(tmp, tmp_bytes, flag, scan, (int)N, st));
    TRYC(cudaMemcpyAsync(&last_flag, flag + N - 1, 4, cudaMemcpyDeviceToHost, st));
    TRYC(cudaMemcpyAsync(&last_scan, scan + N - 1, 4, cudaMemcpyDeviceToHost, st));
    TRYC(cudaStreamSynchronize(st));
    nfree32 = last_flag + last_scan;
    p->nrows = nfree32;
    TRY(dalloc(&p->dof_of_row, p->nrows));
    reduced_index_kernel<<<nblk(N), 256, 0, st>>>(N, flag, scan, p->row_of_dof, p->dof_of_row);
    // keys of the kept slots, sorted with their slot index
    TRY(dalloc(&keys, nnz_in));
    TRY(dalloc(&keys_sorted, nnz_in));
    TRY(dalloc(&idx, nnz_in));
    TRY(dalloc(&p->perm, nnz_in));
    if (nnz_in > 0) {
        coo_keys_kernel<<<nblk(nnz_in), 256, 0, st>>>(nnz_in, Kr, Kc, N, p->row_of_dof,
                                                      p->nrows > 0 ? p->nrows : 1, keys, idx, err);
        {
            int end_bit = 1;
            while (end_bit < 64 && ((1ull << end_bit) - 1) < (uint64_t)p->nrows * (uint64_t)p->nrows) end_bit++;
            // the drop marker ~0 must sort last: use all 64 bits when needed
            end_bit = 64;
            TRYC(cub::DeviceRadixSort::SortPairs(nullptr, need, keys, keys_sorted, idx, p->perm,
                                                 (int)nnz_in, 0, end_bit, st));
            if (need > tmp_bytes) {
                cudaFree(tmp);
                tmp_bytes = need;
                TRYC(cudaMalloc(&tmp, tmp_bytes));
            }
            TRYC(cub::DeviceRadixSort::SortPairs(tmp, tmp_bytes, keys, keys_sorted, idx, p->perm,
                                                 (int)nnz_in, 0, end_bit, st));
        }
        // segments
        TRY(dalloc(&head, nnz_in));
        TRY(dalloc(&hscan, nnz_in));
        head_flags_kernel<<<nblk(nnz_in), 256, 0, st>>>(nnz_in, keys_sorted, head);
        TRYC(cub::DeviceScan::ExclusiveSum(nullptr, need, head, hscan, (int)nnz_in, st));
        if (need > tmp_bytes) {
            cudaFree(tmp);
            tmp_bytes = need;
            TRYC(cudaMalloc(&tmp, tmp_bytes));
        }
        TRYC(cub::DeviceScan::ExclusiveSum(tmp, tmp_bytes, head, hscan, (int)nnz_in, st));
        TRYC(cudaMemcpyAsync(&last_head, head + nnz_in - 1, 4, cudaMemcpyDeviceToHost, st));
        TRYC(cudaMemcpyAsync(&last_hscan, hscan + nnz_in - 1, 4, cudaMemcpyDeviceToHost, st));
        TRY(dalloc(&dcount, 1));
        TRYC(cudaMemsetAsync(dcount, 0, sizeof(*dcount), st));
        count_valid_kernel<<<nblk(nnz_in), 256, 0, st>>>(nnz_in, keys_sorted, dcount);
        TRYC(cudaMemcpyAsync(&hcount, dcount, sizeof(hcount), cudaMemcpyDeviceToHost, st));
        TRYC(cudaStreamSynchronize(st));
        nseg32 = last_head + last_hscan;
    }
    p->nnz = nseg32;
    p->nnz_valid = (int64_t)hcount;
    TRY(dalloc(&p->seg, p->nnz + 1));
    TRY(dalloc(&p->colind, p->nnz));
    TRY(dalloc(&row_count, p->nrows + 1));
    TRY(dalloc(&p->rowptr, p->nrows + 1));
    TRYC(cudaMemsetAsync(row_count, 0, sizeof(int32_t) * (p->nrows + 1), st));
    if (nnz_in > 0) {
        segments_kernel<<<nblk(nnz_in), 256, 0, st>>>(nnz_in, keys_sorted, head, hscan, p->nrows > 0 ? p->nrows : 1,
                                                      p->seg, p->colind, row_count);
    }
    seg_end_kernel<<<1, 1, 0, st>>>(p->nnz_valid, p->nnz, p->seg);
    // row pointer = exclusive scan of the per-row counts (64-bit)
    TRY(dalloc(&rc64, p->nrows + 1));
    TRY(dalloc(&rscan, p->nrows + 1));
    widen_kernel<<<nblk(p->nrows + 1), 256, 0, st>>>(p->nrows + 1, row_count, rc64);
    TRYC(cub::DeviceScan::ExclusiveSum(nullptr, need, rc64, rscan, (int)(p->nrows + 1), st));
    if (need > tmp_bytes) {
        cudaFree(tmp);
        tmp_bytes = need;
        TRYC(cudaMalloc(&tmp, tmp_bytes));
    }
    TRYC(cub::DeviceScan::ExclusiveSum(tmp, tmp_bytes, rc64, rscan, (int)(p->nrows + 1), st));
    rowptr_kernel<<<nblk(p->nrows + 1), 256, 0, st>>>(p->nrows, rscan, p->rowptr, p->nnz);
    if (p->nrows > 0 && p->nnz > 0) {
        // compressed columns for the SpMV (2 bytes per entry instead of 4)
        TRY(dalloc(&p->colbase, p->nrows));
        TRY(dalloc(&p->col16, p->nnz));
        TRY(dalloc(&wide, 1));
        TRYC(cudaMemsetAsync(wide, 0, sizeof(int), st));
        col16_kernel<<<nblk(p->nrows), 256, 0, st>>>(p->nrows, p->rowptr, p->colind, p->colbase, p->col16, wide);
        TRYC(cudaMemcpyAsync(&hwide, wide, sizeof(int), cudaMemcpyDeviceToHost, st));
    }
    TRYC(cudaStreamSynchronize(st));
    TRYC(cudaGetLastError());
    if (hwide) {
        cudaFree(p->colbase);
        cudaFree(p->col16);
        p->colbase = nullptr;
        p->col16 = nullptr;
    }
    cudaFree(wide);
    wide = nullptr;
    cudaFree(flag); cudaFree(scan); cudaFree(keys); cudaFree(keys_sorted); cudaFree(idx);
    cudaFree(head); cudaFree(hscan); cudaFree(row_count); cudaFree(rc64); cudaFree(rscan);
    cudaFree(tmp); cudaFree(dcount);
    *out = p;
    return FE3D_OK;
fail:
    cudaFree(flag); cudaFree(scan); cudaFree(keys); cudaFree(keys_sorted); cudaFree(idx);
    cudaFree(head); cudaFree(hscan); cudaFree(row_count); cudaFree(rc64); cudaFree(rscan);
    cudaFree(tmp); cudaFree(dcount); cudaFree(wide);
    fe3d_pattern_free(p);
    return rc;
#undef TRY
#undef TRYC
}

extern "C" int fe3d_pattern_free(fe3d_pattern *p) {
    if (!p) return FE3D_OK;
    cudaFree(p->row_of_dof);
    cudaFree(p->dof_of_row);
    cudaFree(p->perm);
    cudaFree(p->seg);
    cudaFree(p->colind);
    cudaFree(p->rowptr);
    cudaFree(p->colbase);
    cudaFree(p->col16);
    cudaFree(p->nbrptr);
    cudaFree(p->nbr);
    cudaFree(p->nboff);
    cudaFree(p->noderow);
    delete p;
    return FE3D_OK;
}

extern "C" int fe3d_pattern_info(const fe3d_pattern *p, int64_t *nrows, int64_t *nnz,
                                 int64_t *nnz_in) {
    if (!p) return FE3D_ERR_ARG;
    if (nrows) *nrows = p->nrows;
    if (nnz) *nnz = p->nnz;
    if (nnz_in) *nnz_in = p->nnz_in;
    return FE3D_OK;
}

extern "C" int fe3d_pattern_arrays(const fe3d_pattern *p, const int64_t **rowptr,
                                   const int32_t **colind, const int64_t **dof_of_row,
                                   const int32_t **row_of_dof) {
    if (!p) return FE3D_ERR_ARG;
    if (rowptr) *rowptr = p->rowptr;
    if (colind) *colind = p->colind;
    if (dof_of_row) *dof_of_row = p->dof_of_row;
    if (row_of_dof) *row_of_dof = p->row_of_dof;
    return FE3D_OK;
}

extern "C" int fe3d_pattern_copy(const fe3d_pattern *p, int64_t *rowptr, int32_t *colind,
                                 int64_t *dof_of_row, void *stream) {
    if (!p) return FE3D_ERR_ARG;
    cudaStream_t st = as_stream(stream);
    if (rowptr)
        FE3D_CUDA(cudaMemcpyAsync(rowptr, p->rowptr, sizeof(int64_t) * (p->nrows + 1),
                                  cudaMemcpyDeviceToDevice, st));
    if (colind && p->nnz)
        FE3D_CUDA(cudaMemcpyAsync(colind, p->colind, sizeof(int32_t) * p->nnz, cudaMemcpyDeviceToDevice, st));
    if (dof_of_row && p->nrows)
        FE3D_CUDA(cudaMemcpyAsync(dof_of_row, p->dof_of_row, sizeof(int64_t) * p->nrows,
                                  cudaMemcpyDeviceToDevice, st));
    return FE3D_OK;
}

extern "C" int fe3d_assemble(const fe3d_pattern *p, const double *Kv, double *vals, void *stream) {
    if (!p || (p->nnz > 0 && (!Kv || !vals))) return FE3D_ERR_ARG;
    if (p->nnz > 0 && !p->perm) return FE3D_ERR_STATE;  // pattern built from elements: no COO slots
    if (p->nnz == 0) return FE3D_OK;
    const int64_t blocks = (p->nnz + 255) / 256;
    const unsigned grid = (unsigned)(blocks < kSMs * 16 ? blocks : kSMs * 16);
    assemble_kernel<<<grid, 256, 0, as_stream(stream)>>>(p->nnz, p->seg, p->perm, Kv, vals);
    FE3D_CHECK_LAUNCH();
    return FE3D_OK;
}
