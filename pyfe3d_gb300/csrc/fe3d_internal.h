// Opaque objects behind the C ABI (device arrays owned by the library).
#pragma once
#include <stdint.h>

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
};
