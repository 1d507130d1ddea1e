// Shared definitions of the pyfe3d_gb300 CUDA library.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "fe3d_gb300.h"

#define FE3D_CHECK_LAUNCH()                                   \
    do {                                                      \
        cudaError_t e__ = cudaGetLastError();                 \
        if (e__ != cudaSuccess) return FE3D_ERR_LAUNCH;       \
    } while (0)

#define FE3D_CUDA(call)                                       \
    do {                                                      \
        cudaError_t e__ = (call);                             \
        if (e__ != cudaSuccess) return FE3D_ERR_CUDA;         \
    } while (0)

namespace fe3d {

constexpr int kSMs = 152;                 // GB300
constexpr double kGauss = 0.5773502691896257645092;

// Device error word bits (OR-ed by kernels, read by the host).
constexpr int kErrBounds = 1;             // an index/offset outside the caller's buffers
constexpr int kErrNonFinite = 2;          // NaN/Inf met where the caller asked to check

__device__ __forceinline__ void raise_error(int *err, int bit) {
    if (err) atomicOr(err, bit);
}

inline cudaStream_t as_stream(void *s) { return reinterpret_cast<cudaStream_t>(s); }

// CTAs of `kernel` resident on one SM at this block size and dynamic shared
// memory (1 if the query fails).  Persistent grids of kSMs times this run in
// one wave; a larger cap leaves a partial second wave.
template <class F>
inline int resident_per_sm(F kernel, int threads, size_t smem) {
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kernel, threads, smem) != cudaSuccess || n < 1) {
        (void)cudaGetLastError();
        n = 1;
    }
    return n;
}

// Property record layouts (doubles per record).
enum ShellField {
    SP_A11, SP_A12, SP_A16, SP_A22, SP_A26, SP_A66,
    SP_B11, SP_B12, SP_B16, SP_B22, SP_B26, SP_B66,
    SP_D11, SP_D12, SP_D16, SP_D22, SP_D26, SP_D66,
    SP_E44, SP_E45, SP_E55, SP_SCF13, SP_SCF23, SP_H,
    SP_RHO, SP_RHOZ, SP_RHOZ2, SP_STRIDE = FE3D_SHELL_PROP_STRIDE
};
enum BeamField {
    BP_A, BP_E, BP_G, BP_IYY, BP_IZZ, BP_IYZ, BP_J, BP_AY, BP_AZ,
    BP_RHO, BP_RHOY, BP_RHOZ, BP_RHOY2, BP_RHOZ2, BP_RHOYZ,
    BP_STRIDE = FE3D_BEAM_PROP_STRIDE
};

// In-plane constitutive rotation X' = T X T^T with the rows
// a = (m11^2, m12^2, 2 m11 m12), b = (m21^2, m22^2, 2 m21 m22),
// c = (m11 m21, m12 m22, m11 m22 + m12 m21); X and X' hold 11 12 16 22 26 66.
__device__ __forceinline__ void rotate_plane(const double m11, const double m12,
                                             const double m21, const double m22,
                                             const double *X, double *Y) {
    const double T[3][3] = {{m11 * m11, m12 * m12, 2. * m11 * m12},
                            {m21 * m21, m22 * m22, 2. * m21 * m22},
                            {m11 * m21, m12 * m22, m11 * m22 + m12 * m21}};
    const double S[3][3] = {{X[0], X[1], X[2]}, {X[1], X[3], X[4]}, {X[2], X[4], X[5]}};
    double TS[3][3];
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++) TS[i][j] = T[i][0] * S[0][j] + T[i][1] * S[1][j] + T[i][2] * S[2][j];
    auto y = [&](int i, int j) { return TS[i][0] * T[j][0] + TS[i][1] * T[j][1] + TS[i][2] * T[j][2]; };
    Y[0] = y(0, 0);
    Y[1] = y(1, 0);
    Y[2] = y(2, 0);
    Y[3] = y(1, 1);
    Y[4] = y(2, 1);
    Y[5] = y(2, 2);
}

// Bilinear quadrilateral: Jacobian determinant, shape functions and their
// Cartesian derivatives at (xi, eta) from the nodal (x, y) of the element.
__device__ __forceinline__ void quad_derivs(const double *xy, double xi, double eta,
                                            double &detJ, double *N, double *Nx, double *Ny) {
    const double x1 = xy[0], y1 = xy[1], x2 = xy[2], y2 = xy[3];
    const double x3 = xy[4], y3 = xy[5], x4 = xy[6], y4 = xy[7];
    const double J11 = -0.5 * x1 + 0.5 * x2 + 0.5 * (eta + 1) * (0.5 * x1 - 0.5 * x2 + 0.5 * x3 - 0.5 * x4);
    const double J12 = -0.5 * y1 + 0.5 * y2 + 0.5 * (eta + 1) * (0.5 * y1 - 0.5 * y2 + 0.5 * y3 - 0.5 * y4);
    const double J21 = -0.5 * x1 + 0.5 * x4 - 0.25 * (-x1 + x2) * (xi + 1) + 0.25 * (x3 - x4) * (xi + 1);
    const double J22 = -0.5 * y1 + 0.5 * y4 - 0.25 * (xi + 1) * (-y1 + y2) + 0.25 * (xi + 1) * (y3 - y4);
    detJ = J11 * J22 - J12 * J21;
    const double inv = 1. / detJ;
    const double j11 = J22 * inv, j12 = -J12 * inv, j21 = -J21 * inv, j22 = J11 * inv;
    const double dxi[4] = {0.25 * (eta - 1), 0.25 * (1 - eta), 0.25 * (eta + 1), -0.25 * (eta + 1)};
    const double det[4] = {0.25 * (xi - 1), -0.25 * (xi + 1), 0.25 * (xi + 1), 0.25 * (1 - xi)};
    const double sx[4] = {-1., 1., 1., -1.}, sy[4] = {-1., -1., 1., 1.};
#pragma unroll
    for (int a = 0; a < 4; a++) {
        N[a] = 0.25 * (1 + sx[a] * xi) * (1 + sy[a] * eta);
        Nx[a] = j11 * dxi[a] + j12 * det[a];
        Ny[a] = j21 * dxi[a] + j22 * det[a];
    }
}

}  // namespace fe3d
