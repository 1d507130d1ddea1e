// Fused element -> CSR assembly: the reduced CSR pattern built from element
// connectivity, and the scatter map that sends element blocks straight to
// their CSR positions (no COO triplets).
//
// Stands in for `coo_matrix((v, (r, c))).tocsc()` + `K[bu, :][:, bu]` of the
// reference tests (tests/test_quad4_static_point_load.py:80-99) for matrices
// whose elements couple every DOF of their nodes (the KC0 triplets of
// pyfe3d/quad4.pyx:1204-1313, quad4r.pyx:1145-4618, tria3r.pyx:950-2960,
// beamc.pyx:489-1352 write the full (6 nn)^2 block of every element).
//
// Pattern.  The node pairs (a, b) of every element are sorted and made
// unique: node a's neighbours.  The free DOFs keep their order (reduced
// numbering as in fe3d_pattern_build), so the free rows of node a are
// consecutive and share one column list: the free DOFs of its neighbours in
// ascending order.  Each node therefore has a row start rs, a row length L
// and, per neighbour, the offset of that neighbour's free columns.
//
// Scatter map.  Entry (a, m; b, n) of an element block lands at
//   rs[a] + rank_a(m) L[a] + boff(a, b) + rank_b(n),
// rank = number of free DOFs of the node below the given one.  Elements are
// coloured so that no two elements of one colour share a node (greedy, in
// element order); a colour is one launch, so its elements read, add and
// write their blocks without atomics, and every CSR entry is summed in the
// same order on every run.  In assign mode the first contributor of a
// node-pair block (lowest group, then lowest colour) stores instead of
// adding, so no clearing pass is needed.
#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>
#include <cub/device/device_select.cuh>

#include <vector>

#include "common.cuh"
#include "fe3d_internal.h"

namespace fe3d {
namespace {

inline unsigned nblk(int64_t n, int bs = 256) {
    const int64_t b = (n + bs - 1) / bs;
    return (unsigned)(b > 0 ? b : 1);
}

template <typename T>
int dalloc(T **p, size_t n) {
    if (n == 0) n = 1;
    return cudaMalloc((void **)p, n * sizeof(T)) == cudaSuccess ? 0 : FE3D_ERR_NOMEM;
}

__global__ void ef_free_flags(int64_t N, const uint8_t *fixed, int32_t *flag) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < N) flag[i] = fixed ? (fixed[i] ? 0 : 1) : 1;
}

__global__ void ef_reduced_index(int64_t N, const int32_t *flag, const int32_t *scan, int32_t *row_of_dof,
                                 int64_t *dof_of_row) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= N) return;
    if (flag[i]) {
        row_of_dof[i] = scan[i];
        dof_of_row[scan[i]] = i;
    } else {
        row_of_dof[i] = -1;
    }
}

// node pair keys a * nnodes + b of every element of a group
__global__ void ef_pair_keys(int64_t E, int nn, const int64_t *cdof, int64_t nnodes, uint64_t *keys, int *err) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t per = (int64_t)nn * nn;
    if (t >= E * per) return;
    const int64_t e = t / per;
    const int ij = (int)(t - e * per), i = ij / nn, j = ij - i * nn;
    const int64_t ca = cdof[e * nn + i], cb = cdof[e * nn + j];
    uint64_t key = ~0ull;
    if (ca < 0 || cb < 0 || ca % 6 || cb % 6 || ca / 6 >= nnodes || cb / 6 >= nnodes)
        raise_error(err, kErrBounds);
    else
        key = (uint64_t)(ca / 6) * (uint64_t)nnodes + (uint64_t)(cb / 6);
    keys[t] = key;
}

// neighbour node and per-node counts of the unique pairs
__global__ void ef_pairs_split(int64_t npairs, const uint64_t *ukeys, int64_t nnodes, int32_t *nbr,
                               unsigned long long *count) {
    const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (k >= npairs) return;
    const uint64_t key = ukeys[k];
    nbr[k] = (int32_t)(key % (uint64_t)nnodes);
    atomicAdd(count + key / (uint64_t)nnodes, 1ull);
}

// per node: free mask, neighbour offsets and row length
__global__ void ef_node_rows(int64_t nnodes, const int32_t *row_of_dof, const int64_t *nbrptr,
                             const int32_t *nbr, int32_t *nboff, fe3d_noderow *nr, int *maxlen) {
    const int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (a >= nnodes) return;
    int fm = 0;
#pragma unroll
    for (int m = 0; m < 6; m++) fm |= (row_of_dof[6 * a + m] >= 0) << m;
    int off = 0;
    for (int64_t k = nbrptr[a]; k < nbrptr[a + 1]; k++) {
        nboff[k] = off;
        int fb = 0;
        const int64_t b = nbr[k];
#pragma unroll
        for (int n = 0; n < 6; n++) fb += row_of_dof[6 * b + n] >= 0;
        off += fb;
    }
    nr[a].rs = -1;
    nr[a].L = off;
    nr[a].fm = fm;
    atomicMax(maxlen, off);
}

__global__ void ef_row_len(int64_t nrows, const int64_t *dof_of_row, const fe3d_noderow *nr, int64_t *len) {
    const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (r < nrows) len[r] = nr[dof_of_row[r] / 6].L;
}

__global__ void ef_rowptr(int64_t n, const int64_t *scan, int64_t *rowptr, const int64_t *len) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) rowptr[i] = scan[i];
    if (i == n - 1) rowptr[n] = scan[i] + len[i];
}

// row start of each node and the column indices of its rows
__global__ void ef_columns(int64_t nnodes, const int32_t *row_of_dof, const int64_t *rowptr, const int64_t *nbrptr,
                           const int32_t *nbr, fe3d_noderow *nr, int32_t *colind) {
    const int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (a >= nnodes) return;
    const int fm = nr[a].fm;
    if (!fm) return;
    const int m0 = __ffs(fm) - 1;
    const int64_t r0 = row_of_dof[6 * a + m0];
    const int64_t rs = rowptr[r0];
    nr[a].rs = rs;
    const int L = nr[a].L;
    const int nfa = __popc(fm);
    int off = 0;
    for (int64_t k = nbrptr[a]; k < nbrptr[a + 1]; k++) {
        const int64_t b = nbr[k];
#pragma unroll
        for (int n = 0; n < 6; n++) {
            const int32_t c = row_of_dof[6 * b + n];
            if (c < 0) continue;
            for (int i = 0; i < nfa; i++) colind[rs + (int64_t)i * L + off] = c;
            off++;
        }
    }
}

__global__ void ef_col16(int64_t n, const int64_t *rowptr, const int32_t *colind, int32_t *colbase,
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

// ---------------------------------------------------------------- map
__global__ void ef_nodes_of(int64_t E, int nn, const int64_t *cdof, int64_t nnodes, int32_t *node, int *err) {
    const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= E) return;
    bool ok = true;
    int32_t v[8];
    for (int i = 0; i < nn; i++) {
        const int64_t c = cdof[e * nn + i];
        if (c < 0 || c % 6 || c / 6 >= nnodes) {
            ok = false;
            v[i] = 0;
        } else {
            v[i] = (int32_t)(c / 6);
        }
        for (int j = 0; j < i; j++) ok &= v[j] != v[i];
    }
    if (!ok) raise_error(err, kErrBounds);
    for (int i = 0; i < nn; i++) node[e * nn + i] = v[i];
}

__device__ __forceinline__ int64_t find_pair(const int64_t *nbrptr, const int32_t *nbr, int32_t a, int32_t b) {
    int64_t lo = nbrptr[a], hi = nbrptr[a + 1];
    while (lo < hi) {
        const int64_t mid = (lo + hi) >> 1;
        if (nbr[mid] < b) lo = mid + 1;
        else hi = mid;
    }
    return (lo < nbrptr[a + 1] && nbr[lo] == b) ? lo : -1;
}

// block offsets, and the lowest (group, colour) key of every node pair
__global__ void ef_map_offsets(int64_t E, int nn, const int32_t *node, const uint8_t *color, int gkey,
                               const int64_t *nbrptr, const int32_t *nbr, const int32_t *nboff, int32_t *boff,
                               int *firstkey, int *err) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t per = (int64_t)nn * nn;
    if (t >= E * per) return;
    const int64_t e = t / per;
    const int ij = (int)(t - e * per), i = ij / nn, j = ij - i * nn;
    const int64_t k = find_pair(nbrptr, nbr, node[e * nn + i], node[e * nn + j]);
    if (k < 0) {
        raise_error(err, kErrBounds);
        boff[t] = 0;
        return;
    }
    boff[t] = nboff[k];
    atomicMin(firstkey + k, (gkey << 8) | color[e]);
}

__global__ void ef_map_first(int64_t E, int nn, const int32_t *node, const uint8_t *color, int gkey,
                             const int64_t *nbrptr, const int32_t *nbr, const int *firstkey, uint32_t *first) {
    const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= E) return;
    uint32_t bits = 0;
    const int key = (gkey << 8) | color[e];
    for (int i = 0; i < nn; i++)
        for (int j = 0; j < nn; j++) {
            const int64_t k = find_pair(nbrptr, nbr, node[e * nn + i], node[e * nn + j]);
            if (k >= 0 && firstkey[k] == key) bits |= 1u << (i * nn + j);
        }
    first[e] = bits;
}

__global__ void ef_fill_int(int64_t n, int *a, int v) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) a[i] = v;
}

// ------------------------------------------------------------- scatter
// One warp per element of the colour: lanes over the (6 nn)^2 slots.
template <int NN>
__global__ void __launch_bounds__(256) ef_scatter(int64_t cnt, const int32_t *order, const int32_t *node,
                                                  const int32_t *boff, const uint32_t *first,
                                                  const fe3d_noderow *nr, const int64_t *init_k,
                                                  const double *Kv, int64_t nk, double *vals, int64_t nnz,
                                                  int assign, int *err) {
    constexpr int ND = 6 * NN, NS = ND * ND;
    const int lane = threadIdx.x & 31;
    const int64_t w = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t t = w; t < cnt; t += nw) {
        const int64_t e = order[t];
        const int64_t k0 = init_k[e];
        if (k0 < 0 || k0 + NS > nk) {
            if (lane == 0) raise_error(err, kErrBounds);
            continue;
        }
        long long rs[NN];
        int L[NN], fm[NN];
#pragma unroll
        for (int i = 0; i < NN; i++) {
            const fe3d_noderow q = nr[node[e * NN + i]];
            rs[i] = q.rs;
            L[i] = q.L;
            fm[i] = q.fm;
        }
        const uint32_t fb = assign ? first[e] : 0u;
        for (int s = lane; s < NS; s += 32) {
            const int row = s / ND, col = s - row * ND;
            const int a = row / 6, m = row - 6 * a, b = col / 6, n = col - 6 * b;
            if (!((fm[a] >> m) & 1) || !((fm[b] >> n) & 1)) continue;
            const int64_t pos = rs[a] + (int64_t)__popc(fm[a] & ((1 << m) - 1)) * L[a] +
                                boff[e * NN * NN + a * NN + b] + __popc(fm[b] & ((1 << n) - 1));
            if (pos < 0 || pos >= nnz) {
                raise_error(err, kErrBounds);
                continue;
            }
            const double v = Kv[k0 + s];
            if ((fb >> (a * NN + b)) & 1) vals[pos] = v;
            else vals[pos] += v;
        }
    }
}

void free_group(fe3d_fmap_group &g) {
    cudaFree(g.node);
    cudaFree(g.boff);
    cudaFree(g.first);
    cudaFree(g.order);
    g.node = nullptr;
    g.boff = g.order = nullptr;
    g.first = nullptr;
}

}  // namespace
}  // namespace fe3d

using namespace fe3d;

extern "C" int fe3d_pattern_build_elements(const fe3d_elem_group *groups, int ngroups, int64_t N,
                                           const uint8_t *fixed, fe3d_pattern **out, int *err, void *stream) {
    if (!out || !groups || ngroups < 1 || ngroups > kFmapMaxGroups || N <= 0 || N % 6) return FE3D_ERR_ARG;
    if (N >= (int64_t)INT32_MAX) return FE3D_ERR_ARG;
    int64_t npk = 0;
    for (int g = 0; g < ngroups; g++) {
        if (groups[g].E < 0 || groups[g].nn < 1 || groups[g].nn > 4) return FE3D_ERR_ARG;
        if (groups[g].E > 0 && !groups[g].cdof) return FE3D_ERR_ARG;
        npk += groups[g].E * groups[g].nn * groups[g].nn;
    }
    if (npk >= (int64_t)INT32_MAX) return FE3D_ERR_ARG;
    *out = nullptr;
    cudaStream_t st = as_stream(stream);
    fe3d_pattern *p = new fe3d_pattern();
    const int64_t nnodes = N / 6;
    p->N = N;
    p->nnodes = nnodes;
    int rc = 0;
    int32_t *flag = nullptr, *scan = nullptr;
    uint64_t *keys = nullptr, *skeys = nullptr, *ukeys = nullptr;
    unsigned long long *count = nullptr;
    int64_t *len = nullptr, *lscan = nullptr, *dnum = nullptr;
    int *dmax = nullptr, *wide = nullptr;
    void *tmp = nullptr;
    size_t tmp_bytes = 0, need = 0;
    int32_t last_flag = 0, last_scan = 0;
    int64_t npairs = 0, hnnz = 0;
    int hwide = 0;
    int64_t off = 0;
#define TRY(x)             \
    do {                   \
        rc = (x);          \
        if (rc) goto fail; \
    } while (0)
#define TRYC(x)                   \
    do {                          \
        if ((x) != cudaSuccess) { \
            rc = FE3D_ERR_CUDA;   \
            goto fail;            \
        }                         \
    } while (0)
#define GROW()                                      \
    do {                                            \
        if (need > tmp_bytes) {                     \
            cudaFree(tmp);                          \
            tmp = nullptr;                          \
            tmp_bytes = need;                       \
            TRYC(cudaMalloc(&tmp, tmp_bytes));      \
        }                                           \
    } while (0)
    // reduced numbering of the free DOFs (ascending, as fe3d_pattern_build)
    TRY(dalloc(&flag, N));
    TRY(dalloc(&scan, N));
    TRY(dalloc(&p->row_of_dof, N));
    ef_free_flags<<<nblk(N), 256, 0, st>>>(N, fixed, flag);
    TRYC(cub::DeviceScan::ExclusiveSum(nullptr, need, flag, scan, (int)N, st));
    GROW();
    TRYC(cub::DeviceScan::ExclusiveSum(tmp, tmp_bytes, flag, scan, (int)N, st));
    TRYC(cudaMemcpyAsync(&last_flag, flag + N - 1, 4, cudaMemcpyDeviceToHost, st));
    TRYC(cudaMemcpyAsync(&last_scan, scan + N - 1, 4, cudaMemcpyDeviceToHost, st));
    TRYC(cudaStreamSynchronize(st));
    p->nrows = last_flag + last_scan;
    TRY(dalloc(&p->dof_of_row, p->nrows));
    ef_reduced_index<<<nblk(N), 256, 0, st>>>(N, flag, scan, p->row_of_dof, p->dof_of_row);
    // unique node pairs of all groups
    TRY(dalloc(&keys, npk));
    TRY(dalloc(&skeys, npk));
    TRY(dalloc(&ukeys, npk));
    for (int g = 0; g < ngroups; g++) {
        const int64_t n = groups[g].E * groups[g].nn * groups[g].nn;
        if (n > 0) ef_pair_keys<<<nblk(n), 256, 0, st>>>(groups[g].E, groups[g].nn, groups[g].cdof, nnodes,
                                                          keys + off, err);
        off += n;
    }
    TRYC(cudaGetLastError());
    TRY(dalloc(&dnum, 1));
    TRYC(cudaMemsetAsync(dnum, 0, sizeof(int64_t), st));
    if (npk > 0) {
        TRYC(cub::DeviceRadixSort::SortKeys(nullptr, need, keys, skeys, (int)npk, 0, 64, st));
        GROW();
        TRYC(cub::DeviceRadixSort::SortKeys(tmp, tmp_bytes, keys, skeys, (int)npk, 0, 64, st));
        TRYC(cub::DeviceSelect::Unique(nullptr, need, skeys, ukeys, dnum, (int)npk, st));
        GROW();
        TRYC(cub::DeviceSelect::Unique(tmp, tmp_bytes, skeys, ukeys, dnum, (int)npk, st));
    }
    TRYC(cudaMemcpyAsync(&npairs, dnum, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
    TRYC(cudaStreamSynchronize(st));
    // bad keys (~0) sort last: drop them (their elements raised the error word)
    if (npairs > 0) {
        uint64_t lastkey = 0;
        TRYC(cudaMemcpy(&lastkey, ukeys + npairs - 1, sizeof(uint64_t), cudaMemcpyDeviceToHost));
        if (lastkey == ~0ull) npairs--;
    }
    TRY(dalloc(&p->nbr, npairs));
    TRY(dalloc(&p->nboff, npairs));
    TRY(dalloc(&count, nnodes + 1));
    TRY(dalloc(&p->nbrptr, nnodes + 1));
    TRYC(cudaMemsetAsync(count, 0, sizeof(unsigned long long) * (nnodes + 1), st));
    if (npairs > 0) ef_pairs_split<<<nblk(npairs), 256, 0, st>>>(npairs, ukeys, nnodes, p->nbr, count);
    TRYC(cub::DeviceScan::ExclusiveSum(nullptr, need, (const int64_t *)count, p->nbrptr, (int)(nnodes + 1), st));
    GROW();
    TRYC(cub::DeviceScan::ExclusiveSum(tmp, tmp_bytes, (const int64_t *)count, p->nbrptr, (int)(nnodes + 1), st));
    // node rows, row pointer, column indices
    TRY(dalloc(&p->noderow, nnodes));
    TRY(dalloc(&dmax, 1));
    TRYC(cudaMemsetAsync(dmax, 0, sizeof(int), st));
    ef_node_rows<<<nblk(nnodes), 256, 0, st>>>(nnodes, p->row_of_dof, p->nbrptr, p->nbr, p->nboff, p->noderow, dmax);
    TRYC(cudaMemcpyAsync(&p->max_row_len, dmax, sizeof(int), cudaMemcpyDeviceToHost, st));
    TRY(dalloc(&p->rowptr, p->nrows + 1));
    if (p->nrows > 0) {
        TRY(dalloc(&len, p->nrows));
        TRY(dalloc(&lscan, p->nrows));
        ef_row_len<<<nblk(p->nrows), 256, 0, st>>>(p->nrows, p->dof_of_row, p->noderow, len);
        TRYC(cub::DeviceScan::ExclusiveSum(nullptr, need, len, lscan, (int)p->nrows, st));
        GROW();
        TRYC(cub::DeviceScan::ExclusiveSum(tmp, tmp_bytes, len, lscan, (int)p->nrows, st));
        ef_rowptr<<<nblk(p->nrows), 256, 0, st>>>(p->nrows, lscan, p->rowptr, len);
        TRYC(cudaMemcpyAsync(&hnnz, p->rowptr + p->nrows, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
    } else {
        TRYC(cudaMemsetAsync(p->rowptr, 0, sizeof(int64_t), st));
    }
    TRYC(cudaStreamSynchronize(st));
    p->nnz = hnnz;
    TRY(dalloc(&p->colind, p->nnz));
    ef_columns<<<nblk(nnodes), 256, 0, st>>>(nnodes, p->row_of_dof, p->rowptr, p->nbrptr, p->nbr, p->noderow,
                                              p->colind);
    if (p->nrows > 0 && p->nnz > 0) {
        TRY(dalloc(&p->colbase, p->nrows));
        TRY(dalloc(&p->col16, p->nnz));
        TRY(dalloc(&wide, 1));
        TRYC(cudaMemsetAsync(wide, 0, sizeof(int), st));
        ef_col16<<<nblk(p->nrows), 256, 0, st>>>(p->nrows, p->rowptr, p->colind, p->colbase, p->col16, wide);
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
    cudaFree(flag); cudaFree(scan); cudaFree(keys); cudaFree(skeys); cudaFree(ukeys); cudaFree(count);
    cudaFree(len); cudaFree(lscan); cudaFree(dnum); cudaFree(dmax); cudaFree(wide); cudaFree(tmp);
    *out = p;
    return FE3D_OK;
fail:
    cudaFree(flag); cudaFree(scan); cudaFree(keys); cudaFree(skeys); cudaFree(ukeys); cudaFree(count);
    cudaFree(len); cudaFree(lscan); cudaFree(dnum); cudaFree(dmax); cudaFree(wide); cudaFree(tmp);
    fe3d_pattern_free(p);
    return rc;
#undef TRY
#undef TRYC
#undef GROW
}

extern "C" int fe3d_fmap_build(const fe3d_pattern *p, const fe3d_elem_group *groups, int ngroups, fe3d_fmap **out,
                               int *err, void *stream) {
    if (!p || !out || !groups || ngroups < 1 || ngroups > kFmapMaxGroups) return FE3D_ERR_ARG;
    if (!p->nbrptr || !p->noderow) return FE3D_ERR_STATE;  // not built from elements
    for (int g = 0; g < ngroups; g++)
        if (groups[g].E < 0 || groups[g].nn < 1 || groups[g].nn > 4 || (groups[g].E > 0 && !groups[g].cdof))
            return FE3D_ERR_ARG;
    *out = nullptr;
    cudaStream_t st = as_stream(stream);
    fe3d_fmap *m = new fe3d_fmap();
    m->pat = p;
    m->ngroups = ngroups;
    int rc = 0;
    int *firstkey = nullptr;
    uint8_t *dcolor[kFmapMaxGroups] = {};
    int64_t npairs = 0;
    std::vector<int32_t> hnode;
    std::vector<uint8_t> hcolor;
    std::vector<uint64_t> used;
    std::vector<int32_t> horder;
#define TRY(x)             \
    do {                   \
        rc = (x);          \
        if (rc) goto fail; \
    } while (0)
#define TRYC(x)                   \
    do {                          \
        if ((x) != cudaSuccess) { \
            rc = FE3D_ERR_CUDA;   \
            goto fail;            \
        }                         \
    } while (0)
    TRYC(cudaMemcpyAsync(&npairs, p->nbrptr + p->nnodes, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
    TRYC(cudaStreamSynchronize(st));
    TRY(dalloc(&firstkey, npairs));
    if (npairs > 0) ef_fill_int<<<nblk(npairs), 256, 0, st>>>(npairs, firstkey, 0x7fffffff);
    used.assign((size_t)p->nnodes, 0ull);
    for (int g = 0; g < ngroups; g++) {
        fe3d_fmap_group &G = m->g[g];
        G.E = groups[g].E;
        G.nn = groups[g].nn;
        const int nn = G.nn;
        TRY(dalloc(&G.node, G.E * nn));
        TRY(dalloc(&G.boff, G.E * nn * nn));
        TRY(dalloc(&G.first, G.E));
        TRY(dalloc(&G.order, G.E));
        TRY(dalloc(&dcolor[g], G.E));
        if (G.E == 0) continue;
        ef_nodes_of<<<nblk(G.E), 256, 0, st>>>(G.E, nn, groups[g].cdof, p->nnodes, G.node, err);
        TRYC(cudaGetLastError());
        // greedy colouring on the host: the lowest colour that no element
        // sharing a node has taken (per-node bit masks of the colours taken)
        hnode.resize((size_t)(G.E * nn));
        TRYC(cudaMemcpyAsync(hnode.data(), G.node, sizeof(int32_t) * G.E * nn, cudaMemcpyDeviceToHost, st));
        TRYC(cudaStreamSynchronize(st));
        for (auto &u : used) u = 0ull;
        hcolor.resize((size_t)G.E);
        int64_t counts[64] = {};
        int ncol = 0;
        for (int64_t e = 0; e < G.E; e++) {
            uint64_t taken = 0;
            for (int i = 0; i < nn; i++) taken |= used[hnode[e * nn + i]];
            if (taken == ~0ull) {
                rc = FE3D_ERR_ARG;  // more than 64 colours
                goto fail;
            }
            const int c = __builtin_ctzll(~taken);
            hcolor[e] = (uint8_t)c;
            for (int i = 0; i < nn; i++) used[hnode[e * nn + i]] |= 1ull << c;
            counts[c]++;
            if (c + 1 > ncol) ncol = c + 1;
        }
        G.ncolors = ncol;
        G.cstart[0] = 0;
        for (int c = 0; c < ncol; c++) G.cstart[c + 1] = G.cstart[c] + counts[c];
        horder.resize((size_t)G.E);
        {
            int64_t pos[65];
            for (int c = 0; c <= ncol; c++) pos[c] = G.cstart[c];
            for (int64_t e = 0; e < G.E; e++) horder[pos[hcolor[e]]++] = (int32_t)e;
        }
        TRYC(cudaMemcpyAsync(dcolor[g], hcolor.data(), G.E, cudaMemcpyHostToDevice, st));
        TRYC(cudaMemcpyAsync(G.order, horder.data(), sizeof(int32_t) * G.E, cudaMemcpyHostToDevice, st));
        ef_map_offsets<<<nblk(G.E * nn * nn), 256, 0, st>>>(G.E, nn, G.node, dcolor[g], g, p->nbrptr, p->nbr,
                                                             p->nboff, G.boff, firstkey, err);
        TRYC(cudaGetLastError());
        TRYC(cudaStreamSynchronize(st));  // the host buffers are reused by the next group
    }
    // assign bits: the node pair's lowest (group, colour) key is the element's own
    for (int g = 0; g < ngroups; g++) {
        fe3d_fmap_group &G = m->g[g];
        if (G.E == 0) continue;
        ef_map_first<<<nblk(G.E), 256, 0, st>>>(G.E, G.nn, G.node, dcolor[g], g, p->nbrptr, p->nbr, firstkey,
                                                 G.first);
        TRYC(cudaGetLastError());
    }
    TRYC(cudaStreamSynchronize(st));
    cudaFree(firstkey);
    for (int g = 0; g < kFmapMaxGroups; g++) cudaFree(dcolor[g]);
    *out = m;
    return FE3D_OK;
fail:
    cudaFree(firstkey);
    for (int g = 0; g < kFmapMaxGroups; g++) cudaFree(dcolor[g]);
    fe3d_fmap_free(m);
    return rc;
#undef TRY
#undef TRYC
}

extern "C" int fe3d_fmap_free(fe3d_fmap *m) {
    if (!m) return FE3D_OK;
    for (int g = 0; g < m->ngroups; g++) free_group(m->g[g]);
    delete m;
    return FE3D_OK;
}

extern "C" int fe3d_fmap_info(const fe3d_fmap *m, int g, int *ncolors, int64_t *counts) {
    if (!m || g < 0 || g >= m->ngroups) return FE3D_ERR_ARG;
    const fe3d_fmap_group &G = m->g[g];
    if (ncolors) *ncolors = G.ncolors;
    if (counts)
        for (int c = 0; c < G.ncolors; c++) counts[c] = G.cstart[c + 1] - G.cstart[c];
    return FE3D_OK;
}

extern "C" int fe3d_csr_scatter(const fe3d_fmap *m, int g, const int64_t *init_k, const double *Kv, int64_t nk,
                                double *vals, int mode, int *err, void *stream) {
    if (!m || g < 0 || g >= m->ngroups || (mode != FE3D_CSR_ADD && mode != FE3D_CSR_ASSIGN)) return FE3D_ERR_ARG;
    const fe3d_fmap_group &G = m->g[g];
    if (G.E == 0) return FE3D_OK;
    if (!init_k || !Kv || !vals || nk < 0) return FE3D_ERR_ARG;
    cudaStream_t st = as_stream(stream);
    const fe3d_noderow *nr = m->pat->noderow;
    for (int c = 0; c < G.ncolors; c++) {
        const int64_t cnt = G.cstart[c + 1] - G.cstart[c];
        if (cnt == 0) continue;
        const int64_t blocks = (cnt * 32 + 255) / 256;
        const unsigned grid = (unsigned)(blocks < kSMs * 8 ? blocks : kSMs * 8);
        const int32_t *ord = G.order + G.cstart[c];
        const int as = mode == FE3D_CSR_ASSIGN;
        switch (G.nn) {
            case 1: ef_scatter<1><<<grid, 256, 0, st>>>(cnt, ord, G.node, G.boff, G.first, nr, init_k, Kv, nk, vals, m->pat->nnz, as, err); break;
            case 2: ef_scatter<2><<<grid, 256, 0, st>>>(cnt, ord, G.node, G.boff, G.first, nr, init_k, Kv, nk, vals, m->pat->nnz, as, err); break;
            case 3: ef_scatter<3><<<grid, 256, 0, st>>>(cnt, ord, G.node, G.boff, G.first, nr, init_k, Kv, nk, vals, m->pat->nnz, as, err); break;
            default: ef_scatter<4><<<grid, 256, 0, st>>>(cnt, ord, G.node, G.boff, G.first, nr, init_k, Kv, nk, vals, m->pat->nnz, as, err); break;
        }
        FE3D_CHECK_LAUNCH();
    }
    return FE3D_OK;
}
