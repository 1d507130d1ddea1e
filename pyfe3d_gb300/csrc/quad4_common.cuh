// Device code shared by the Quad4 kernels (one copy per translation unit).
#pragma once
#include "common.cuh"

namespace fe3d {
namespace {

constexpr int TILE = 32;     // elements per CTA iteration
constexpr int NT = 128;      // threads per CTA (4 warps)
constexpr int NPT = 5;       // 4 Gauss points + centre
constexpr int GPW = 13;      // per point: w*detJ, N[4], Nx[4], Ny[4]
// padded row stride (doubles) of a staged 24x24 block: 28 keeps rows 16-byte
// aligned, and the 16-byte accesses of the 8 node-pair lanes of a quarter
// warp (nodes a, a + 1 by b = 0..3: offsets 6 KROW a + 6 b) fall on 8
// distinct groups of 4 banks (3 KROW = 4 mod 8)
constexpr int KROW = 28;
constexpr int KSTAGE = 24 * KROW;

enum : int { F_VALID = 1, F_THICK = 2, F_ROTATE = 4 };

struct __align__(16) ElemS {
    double xy[8];     // nodal (x, y) in the evaluation frame
    double R[9];      // element -> global rotation (row-major)
    double abd[36];   // 6x6 ABD in the evaluation frame
    double es[3];     // E44 E45 E55 (with shear correction) in the evaluation frame
    double area;
    long long init_k;
    long long c[4];
    int flags;
    int pad;
};

// Quad4 frame (quad4.pyx:491-624): R from the diagonals, optional material
// direction projection into m (left untouched when it does not project).
__device__ __forceinline__ void q4_rotation(const double *p1, const double *p2,
                                            const double *p3, const double *p4,
                                            const double *xmat, double *R, double *m) {
    double v13[3], v42[3], z[3], xa[3], y[3], t;
#pragma unroll
    for (int i = 0; i < 3; i++) {
        v13[i] = p3[i] - p1[i];
        v42[i] = p2[i] - p4[i];
    }
    z[0] = v42[1] * v13[2] - v42[2] * v13[1];
    z[1] = -v42[0] * v13[2] + v42[2] * v13[0];
    z[2] = v42[0] * v13[1] - v42[1] * v13[0];
    // normalisations by the reciprocal square root (FP64 square roots and
    // divisions are costly on this part, and this frame is on the critical
    // path of the element kernels; it agrees with the reference's frame to
    // rounding)
    const double zz = z[0] * z[0] + z[1] * z[1] + z[2] * z[2];
    double it = rsqrt(zz);
    z[0] *= it; z[1] *= it; z[2] *= it;
#pragma unroll
    for (int i = 0; i < 3; i++) xa[i] = (v13[i] + v42[i]) * 0.5;
    it = rsqrt(xa[0] * xa[0] + xa[1] * xa[1] + xa[2] * xa[2]);
    xa[0] *= it; xa[1] *= it; xa[2] *= it;
    y[0] = z[1] * xa[2] - z[2] * xa[1];
    y[1] = z[2] * xa[0] - z[0] * xa[2];
    y[2] = z[0] * xa[1] - z[1] * xa[0];
    it = rsqrt(y[0] * y[0] + y[1] * y[1] + y[2] * y[2]);
    y[0] *= it; y[1] *= it; y[2] *= it;
#pragma unroll
    for (int i = 0; i < 3; i++) {
        R[3 * i + 0] = xa[i];
        R[3 * i + 1] = y[i];
        R[3 * i + 2] = z[i];
    }
    if (!xmat) return;
    const double tol = sqrt(zz) / 1e10;
    double xm[3] = {xmat[0], xmat[1], xmat[2]}, ym[3];
    const double xn = sqrt(xm[0] * xm[0] + xm[1] * xm[1] + xm[2] * xm[2]);
    xm[0] /= xn; xm[1] /= xn; xm[2] /= xn;
    if (xn > tol) {
        ym[0] = z[1] * xm[2] - z[2] * xm[1];
        ym[1] = z[2] * xm[0] - z[0] * xm[2];
        ym[2] = z[0] * xm[1] - z[1] * xm[0];
        t = sqrt(ym[0] * ym[0] + ym[1] * ym[1] + ym[2] * ym[2]);
        ym[0] /= t; ym[1] /= t; ym[2] /= t;
        if (t > tol) {
            xm[0] = ym[1] * z[2] - ym[2] * z[1];
            xm[1] = ym[2] * z[0] - ym[0] * z[2];
            xm[2] = ym[0] * z[1] - ym[1] * z[0];
            t = sqrt(xm[0] * xm[0] + xm[1] * xm[1] + xm[2] * xm[2]);
            xm[0] /= t; xm[1] /= t; xm[2] /= t;
            const double cth = xm[0] * xa[0] + xm[1] * xa[1] + xm[2] * xa[2];
            m[0] = cth;
            m[3] = cth;
            m[1] = (xm[0] * y[0] + xm[1] * y[1] + xm[2] * y[2] > 0) ? -sqrt(1 - cth * cth)
                                                                    : sqrt(1 - cth * cth);
            m[2] = -m[1];
        }
    }
}

// R^T p for one node (quad4.pyx:714-728).
__device__ __forceinline__ void to_local(const double *R, const double *p, double *q) {
    q[0] = R[0] * p[0] + R[3] * p[1] + R[6] * p[2];
    q[1] = R[1] * p[0] + R[4] * p[1] + R[7] * p[2];
    q[2] = R[2] * p[0] + R[5] * p[1] + R[8] * p[2];
}

__device__ __forceinline__ double shoelace(const double *xy) {
    return 0.5 * fabs((xy[0] * xy[3] + xy[2] * xy[5] + xy[4] * xy[7] + xy[6] * xy[1]) -
                      (xy[2] * xy[1] + xy[4] * xy[3] + xy[6] * xy[5] + xy[0] * xy[7]));
}

__device__ __forceinline__ bool is_flat(const double *R) {
    return R[2] == 0. && R[5] == 0. && R[6] == 0. && R[7] == 0. && R[8] > 0.;
}

// Isotropic section in the material frame: A, D rotation-invariant
// (A11 = A22, A16 = A26 = 0, A66 = (A11 - A12) / 2 up to rounding; same for
// D), B = 0 and shear E45 = 0, E44 = E55.
__device__ __forceinline__ bool iso_section(const double *P, double E44, double E45, double E55) {
    const double eps = 64. * 2.220446049250313e-16;
    bool iso = P[SP_A16] == 0. && P[SP_A26] == 0. && P[SP_D16] == 0. && P[SP_D26] == 0.;
#pragma unroll
    for (int i = 0; i < 6; i++) iso &= P[SP_B11 + i] == 0.;
    iso &= P[SP_A11] == P[SP_A22] && P[SP_D11] == P[SP_D22] && E45 == 0. && E44 == E55;
    iso &= fabs(P[SP_A66] - 0.5 * (P[SP_A11] - P[SP_A12])) <= eps * fabs(P[SP_A11]);
    iso &= fabs(P[SP_D66] - 0.5 * (P[SP_D11] - P[SP_D12])) <= eps * fabs(P[SP_D11]);
    return iso;
}

// Asynchronous 8-byte global -> shared copies (cp.async), used to prefetch
// the caller's current values of a staged block while it is being computed.
__device__ __forceinline__ void cp_async8(void *smem, const void *gmem) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async16(void *smem, const void *gmem) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// Constitutive data of one element in the evaluation frame: ABD rotated to
// the element axes when m12 != 0 (quad4.pyx:845-899), shear correction on E
// (quad4.pyx:903-905), then, for flat elements evaluated in the global frame,
// the in-plane rotation element -> global of ABD and of the shear matrix.
__device__ void q4_constitutive(const double *P, const double *m, const double *R,
                                bool global_frame, double *abd36, double *es) {
    double A[6], B[6], D[6];
    if (m[1] == 0.) {
#pragma unroll
        for (int i = 0; i < 6; i++) {
            A[i] = P[SP_A11 + i];
            B[i] = P[SP_B11 + i];
            D[i] = P[SP_D11 + i];
        }
    } else {
        rotate_plane(m[0], m[1], m[2], m[3], P + SP_A11, A);
        rotate_plane(m[0], m[1], m[2], m[3], P + SP_B11, B);
        rotate_plane(m[0], m[1], m[2], m[3], P + SP_D11, D);
    }
    double E44 = P[SP_E44] * P[SP_SCF23];
    double E45 = P[SP_E45] * 0.5 * (P[SP_SCF13] + P[SP_SCF23]);
    double E55 = P[SP_E55] * P[SP_SCF13];
    if (global_frame) {
        double t[6];
        rotate_plane(R[0], R[1], R[3], R[4], A, t);
#pragma unroll
        for (int i = 0; i < 6; i++) A[i] = t[i];
        rotate_plane(R[0], R[1], R[3], R[4], B, t);
#pragma unroll
        for (int i = 0; i < 6; i++) B[i] = t[i];
        rotate_plane(R[0], R[1], R[3], R[4], D, t);
#pragma unroll
        for (int i = 0; i < 6; i++) D[i] = t[i];
        // (gxz, gyz)_local = Q (gxz, gyz)_global, Q = [[r11, r21], [r12, r22]]
        const double q00 = R[0], q01 = R[3], q10 = R[1], q11 = R[4];
        const double e00 = E55, e01 = E45, e11 = E44;  // (xz, yz) ordering
        const double a00 = e00 * q00 + e01 * q10, a01 = e00 * q01 + e01 * q11;
        const double a10 = e01 * q00 + e11 * q10, a11 = e01 * q01 + e11 * q11;
        const double g00 = q00 * a00 + q10 * a10;
        const double g01 = q00 * a01 + q10 * a11;
        const double g11 = q01 * a01 + q11 * a11;
        E55 = g00;
        E45 = g01;
        E44 = g11;
    }
    // full symmetric 6x6 [[A, B], [B, D]]
    const int idx[3][3] = {{0, 1, 2}, {1, 3, 4}, {2, 4, 5}};
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++) {
            abd36[6 * i + j] = A[idx[i][j]];
            abd36[6 * i + j + 3] = B[idx[i][j]];
            abd36[6 * (i + 3) + j] = B[idx[i][j]];
            abd36[6 * (i + 3) + j + 3] = D[idx[i][j]];
        }
    es[0] = E44;
    es[1] = E45;
    es[2] = E55;
}

// --- KC0 pair block -------------------------------------------------------
// Membrane/bending strains (exx, eyy, gxy, kxx, kyy, kxy) produced by the
// x- and y-derivatives of each in-plane DOF (quad4.pyx:958-1000):
// u -> (exx, gxy), v -> (gxy, eyy), rx -> -(kxy, kyy), ry -> (kxx, kxy).
__device__ __forceinline__ void kc0_block(const double H[3][3], const double H0[3][3],
                                          const double Hs[3][3], const double *abd,
                                          const double *es, double K[6][6]) {
    const int dof[4] = {0, 1, 3, 4};
    const int sidx[4][2] = {{0, 2}, {2, 1}, {5, 4}, {3, 5}};
    const double sg[4] = {1., 1., -1., 1.};
#pragma unroll
    for (int i = 0; i < 6; i++)
#pragma unroll
        for (int j = 0; j < 6; j++) K[i][j] = 0.;
#pragma unroll
    for (int mi = 0; mi < 4; mi++)
#pragma unroll
        for (int ni = 0; ni < 4; ni++) {
            double s = 0.;
#pragma unroll
            for (int p = 0; p < 2; p++)
#pragma unroll
                for (int q = 0; q < 2; q++)
                    s += abd[6 * sidx[mi][p] + sidx[ni][q]] * H[1 + p][1 + q];
            K[dof[mi]][dof[ni]] = sg[mi] * sg[ni] * s;
        }
    // drilling penalty with unit weight (quad4.pyx:1053-1073):
    // d = u N_y/2 - v N_x/2 + rz N
    K[0][0] += 0.25 * H[2][2];
    K[0][1] -= 0.25 * H[2][1];
    K[1][0] -= 0.25 * H[1][2];
    K[1][1] += 0.25 * H[1][1];
    K[0][5] += 0.5 * H[2][0];
    K[1][5] -= 0.5 * H[1][0];
    K[5][0] += 0.5 * H[0][2];
    K[5][1] -= 0.5 * H[0][1];
    K[5][5] += H[0][0];
    // transverse shear, (gyz, gxz) = (w_y - rx N, w_x + ry N)
    // (quad4.pyx:1032-1051, 1127-1171); Hs is the gradient tensor of the
    // thin (centre) or thick (2x2) rule, H0 the centre rule.
    const double E44 = es[0], E45 = es[1], E55 = es[2];
    K[2][2] += E44 * Hs[2][2] + E45 * (Hs[2][1] + Hs[1][2]) + E55 * Hs[1][1];
    K[2][3] -= E44 * H0[2][0] + E45 * H0[1][0];
    K[2][4] += E45 * H0[2][0] + E55 * H0[1][0];
    K[3][2] -= E44 * H0[0][2] + E45 * H0[0][1];
    K[4][2] += E45 * H0[0][2] + E55 * H0[0][1];
    K[3][3] += E44 * H0[0][0];
    K[3][4] -= E45 * H0[0][0];
    K[4][3] -= E45 * H0[0][0];
    K[4][4] += E55 * H0[0][0];
}

// K <- T K T^T with T = blockdiag(R, R) (quad4.pyx:1297-1313).
__device__ __forceinline__ void rotate_block(const double *R, double K[6][6]) {
    double T[6][6];
#pragma unroll
    for (int bi = 0; bi < 2; bi++)
#pragma unroll
        for (int bj = 0; bj < 2; bj++) {
            double tmp[3][3];
#pragma unroll
            for (int i = 0; i < 3; i++)
#pragma unroll
                for (int j = 0; j < 3; j++)
                    tmp[i][j] = R[3 * i + 0] * K[3 * bi + 0][3 * bj + j] +
                                R[3 * i + 1] * K[3 * bi + 1][3 * bj + j] +
                                R[3 * i + 2] * K[3 * bi + 2][3 * bj + j];
#pragma unroll
            for (int i = 0; i < 3; i++)
#pragma unroll
                for (int j = 0; j < 3; j++)
                    T[3 * bi + i][3 * bj + j] = tmp[i][0] * R[3 * j + 0] + tmp[i][1] * R[3 * j + 1] +
                                                tmp[i][2] * R[3 * j + 2];
        }
#pragma unroll
    for (int i = 0; i < 6; i++)
#pragma unroll
        for (int j = 0; j < 6; j++) K[i][j] = T[i][j];
}

struct Q4Args {
    int64_t E;
    const int64_t *cdof;
    const int64_t *init_k;
    const double *x;
    int64_t nx;
    const double *xmat;
    int xmat_stride;
    const double *R, *m, *xe, *area;
    const double *props;
    int64_t nprops;
    const int32_t *pid;
    int64_t *Kr, *Kc;
    double *Kv;
    int64_t nk;
    int values_only;
    int *err;
    int vec16;  // KC0 write-out: output arrays 16-byte aligned
};

// Phase A for KC0: one thread per element of the tile.
__device__ void kc0_phase_a(const Q4Args &a, int64_t e, ElemS &s) {
    s.flags = 0;
    long long c[4];
    bool ok = true;
#pragma unroll
    for (int i = 0; i < 4; i++) {
        c[i] = a.cdof[4 * e + i];
        s.c[i] = c[i];
    }
    const long long k0 = a.init_k ? a.init_k[e] : 0;
    s.init_k = k0;
    if (a.init_k && (k0 < 0 || k0 + 576 > a.nk)) ok = false;
    const int64_t p = a.pid ? (int64_t)a.pid[e] : e;
    if (p < 0 || p >= a.nprops) ok = false;
    if (a.x) {
#pragma unroll
        for (int i = 0; i < 4; i++)
            if (c[i] < 0 || c[i] / 2 + 3 > a.nx) ok = false;
    } else {
#pragma unroll
        for (int i = 0; i < 4; i++)
            if (c[i] < 0) ok = false;
    }
    if (!ok) {
        raise_error(a.err, kErrBounds);
        return;
    }
    double R[9], m[4] = {1., 0., 0., 1.};
    bool global_frame = false;
    double ar;
    if (a.x) {
        const double *p1 = a.x + c[0] / 2, *p2 = a.x + c[1] / 2, *p3 = a.x + c[2] / 2,
                     *p4 = a.x + c[3] / 2;
        const double *xm = a.xmat ? a.xmat + (int64_t)a.xmat_stride * e : nullptr;
        q4_rotation(p1, p2, p3, p4, xm, R, m);
        global_frame = is_flat(R);
        if (global_frame) {
            s.xy[0] = 0.;
            s.xy[1] = 0.;
            s.xy[2] = p2[0] - p1[0];
            s.xy[3] = p2[1] - p1[1];
            s.xy[4] = p3[0] - p1[0];
            s.xy[5] = p3[1] - p1[1];
            s.xy[6] = p4[0] - p1[0];
            s.xy[7] = p4[1] - p1[1];
        } else {
            const double *pp[4] = {p1, p2, p3, p4};
#pragma unroll
            for (int i = 0; i < 4; i++) {
                double q[3];
                to_local(R, pp[i], q);
                s.xy[2 * i] = q[0];
                s.xy[2 * i + 1] = q[1];
            }
        }
        ar = shoelace(s.xy);
    } else {
#pragma unroll
        for (int i = 0; i < 9; i++) R[i] = a.R[9 * e + i];
#pragma unroll
        for (int i = 0; i < 4; i++) m[i] = a.m[4 * e + i];
#pragma unroll
        for (int i = 0; i < 4; i++) {
            s.xy[2 * i] = a.xe[12 * e + 3 * i];
            s.xy[2 * i + 1] = a.xe[12 * e + 3 * i + 1];
        }
        ar = a.area[e];
    }
#pragma unroll
    for (int i = 0; i < 9; i++) s.R[i] = R[i];
    s.area = ar;
    const double *P = a.props + (int64_t)SP_STRIDE * p;
    q4_constitutive(P, m, R, global_frame, s.abd, s.es);
    // h / sqrt(area) >= 1 as the reference evaluates it; the division only
    // decides when h < sqrt(area) (h >= sqrt(area) implies the rounded
    // quotient is >= 1)
    const double sq = sqrt(ar);
    const bool thick = P[SP_H] >= sq || P[SP_H] / sq >= 1.;
    s.flags = F_VALID | (thick ? F_THICK : 0) | (global_frame ? 0 : F_ROTATE);
}

// ue[6 NN e + 6 j ..] = R^T u at the NN nodes of element e (the probe_ue
// updates of quad4.pyx:627-679 and tria3r.pyx:426-477).
template <int NN>
__global__ void probe_ue_kernel(int64_t E, const int64_t *cdof, const double *u, int64_t nu,
                                const double *R, double *ue, int *err) {
    const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= E) return;
    double r[9];
#pragma unroll
    for (int i = 0; i < 9; i++) r[i] = R[9 * e + i];
#pragma unroll
    for (int j = 0; j < NN; j++) {
        const long long c = cdof[NN * e + j];
        if (c < 0 || c + 6 > nu) {
            raise_error(err, kErrBounds);
            return;
        }
        to_local(r, u + c, ue + 6 * NN * e + 6 * j);
        to_local(r, u + c + 3, ue + 6 * NN * e + 6 * j + 3);
    }
}

__device__ __forceinline__ void point_coords(int g, double &xi, double &eta) {
    // Gauss point order of quad4.pyx:927-935: (xi, eta) = (-,-), (-,+), (+,-), (+,+)
    if (g == 4) {
        xi = 0.;
        eta = 0.;
        return;
    }
    xi = (g & 2) ? kGauss : -kGauss;
    eta = (g & 1) ? kGauss : -kGauss;
}

}  // namespace
}  // namespace fe3d
