// Opaque objects behind the C ABI (device arrays owned by the library).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

// Free-row layout of one node in a pattern built from element connectivity:
// its free rows are consecutive, start at CSR position rs (-1 when the node
// has no free DOF) and all have L entries; fm holds the free-DOF bits.
struct __align__(16) fe3d_noderow {
    long long rs;
    int L;
    int fm;
};

struct fe3d_pattern {
    int64_t N = 0;          // DOFs of the full system
    int64_t nrows = 0;      // free DOFs (rows of the reduced system)
    int64_t nnz = 0;        // CSR entries of the reduced system
    int64_t nnz_in = 0;     // COO slots the pattern was built from
    int64_t nnz_valid = 0;  // COO slots with a free row and a free column
    int32_t *row_of_dof = nullptr;  // [N] reduced row of a DOF, -1 when fixed
    int64_t *dof_of_row = nullptr;  // [nrows] full DOF of a reduced row
    int32_t *perm = nullptr;        // [nnz_in] COO slots sorted by (row, col)
    int32_t *seg = nullptr;         // [nnz + 1] segment starts in perm
    int32_t *colind = nullptr;      // [nnz]
    int64_t *rowptr = nullptr;      // [nrows + 1]
    // compressed columns for the solver's SpMV when every row spans fewer than
    // 65,536 columns: colind[k] = colbase[row] + col16[k] (else both NULL)
    int32_t *colbase = nullptr;     // [nrows]
    uint16_t *col16 = nullptr;      // [nnz]
    // node-block structure (patterns built from element connectivity only;
    // perm and seg are then NULL): the neighbours of node a are
    // nbr[nbrptr[a] .. nbrptr[a+1]) in ascending order, and the free columns
    // of neighbour nbr[k] start at offset nboff[k] within node a's rows
    int64_t nnodes = 0;
    int64_t *nbrptr = nullptr;      // [nnodes + 1]
    int32_t *nbr = nullptr;         // [npairs]
    int32_t *nboff = nullptr;       // [npairs]
    fe3d_noderow *noderow = nullptr;  // [nnodes]
    int max_row_len = 0;            // largest L over the nodes
};

// Element -> CSR scatter map of one element group (fused assembly).
struct fe3d_fmap_group {
    int64_t E = 0;
    int nn = 0;                     // nodes per element
    int32_t *node = nullptr;        // [E, nn] node indices
    int32_t *boff = nullptr;        // [E, nn, nn] offset of node j's columns in node i's rows
    uint32_t *first = nullptr;      // [E] bit i nn + j: this element assigns block (i, j)
    int32_t *order = nullptr;       // [E] elements sorted by colour
    int ncolors = 0;
    int64_t cstart[65] = {};        // colour c is order[cstart[c] .. cstart[c+1])
};

constexpr int kFmapMaxGroups = 8;

struct fe3d_fmap {
    const fe3d_pattern *pat = nullptr;
    int ngroups = 0;
    fe3d_fmap_group g[kFmapMaxGroups];
};

// Block-Jacobi PCG state (pcg.cu); the batched solver (bpcg.cu) reuses its
// node blocks, block inverses, work vectors and private stream.
struct fe3d_solver {
    const fe3d_pattern *pat = nullptr;
    int64_t n = 0, nnodes = 0;
    int bs = 6;  // DOFs per node
    int32_t *start = nullptr;
    int8_t *size = nullptr;
    double *Dinv = nullptr;
    float *Dinv32 = nullptr;
    const double *vals = nullptr;  // FP64 values (caller-owned, set by setup)
    int ready = 0;                 // setup has run (vals may be NULL when nnz == 0)
    float *vals32 = nullptr;
    double *r = nullptr;
    double *z = nullptr, *p = nullptr, *q = nullptr;
    float *z32 = nullptr, *p32 = nullptr, *q32 = nullptr;
    double *ppq = nullptr, *prz = nullptr, *prr = nullptr, *prf = nullptr;
    double *scal = nullptr;  // [0..1] rz double buffer, [2] rr, [3] alpha, [4] ff, [5..7] spare
    int *nonpos = nullptr;
    int nparts = 0;
    int spmv_grid = 0, node_grid = 0, vec_grid = 0;
    int have32 = 0;
    // private stream: iteration chunks are captured once as CUDA graphs
    // (the legacy default stream cannot be captured) and replayed
    cudaStream_t stream = nullptr;
    cudaEvent_t ev_in = nullptr, ev_out = nullptr;
    double *uin = nullptr, *fin = nullptr;  // stable operands of the graphs
    double *xhi = nullptr, *xlo = nullptr;  // double-double solution base
    double *sc = nullptr;  // [2n]: row scales sqrt(K_ii), then their inverses; FP32 data hold
                           // S^-1 K S^-1 and S Dinv S
    cudaGraphExec_t graph[3][2] = {};     // [precision][parity]
    int graph_chunk[3][2] = {};
    int graph_flex[3][2] = {};
    int graph_lanes[3][2] = {};
    int lanes[3] = {0, 0, 0};             // SpMV lanes per row [precision], tuned at setup
    float2 *vals2 = nullptr, *p2 = nullptr;  // split-FP32 (hi, lo) values and direction
    int have2 = 0;
    unsigned int *counter = nullptr;      // last-block-done counter of the reductions
};
