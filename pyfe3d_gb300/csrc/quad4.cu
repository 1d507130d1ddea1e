// Quad4 element kernels: frame, probe ue, KC0, KG, M, fint.
//
// Element matrices follow pyfe3d/quad4.pyx (cited per kernel).  The KC0
// kernel is organised for GB300, where FP64 issue (about 1.2 TFLOP/s) is the
// scarce resource next to HBM:
//   phase A  one thread per element: frame, constitutive data, thin/thick
//            flag (vectorised across elements, full warps);
//   phase A2 one thread per (element, integration point): Jacobian and
//            shape-function derivatives at the 4 Gauss points and the centre;
//   phase B  one thread per (element, node pair a,b): the 6x6 block
//            K_ab = sum_pq H^pq_ab C^pq from the 3x3 tensor
//            H^pq_ab = sum_gp w detJ D^p N_a D^q N_b (p,q in {N, d/dx, d/dy}),
//            staged in shared memory and streamed out coalesced with the
//            += read-modify-write of the caller's values.
// Flat elements whose normal is +Z (r13=r23=r31=r32=0) are evaluated
// directly in the global frame with the constitutive matrices rotated in
// plane; that removes the R Ke R^T transform (about 40% of the FP64 work).
// Other elements are evaluated in the element frame and rotated per block.
#include "common.cuh"

namespace fe3d {
namespace {

constexpr int TILE = 32;     // elements per CTA iteration
constexpr int NT = 128;      // threads per CTA (4 warps)
constexpr int NPT = 5;       // 4 Gauss points + centre
constexpr int GPW = 13;      // per point: w*detJ, N[4], Nx[4], Ny[4]
constexpr int KROW = 25;     // padded row stride of the staged 24x24 block
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
    t = sqrt(z[0] * z[0] + z[1] * z[1] + z[2] * z[2]);
    z[0] /= t; z[1] /= t; z[2] /= t;
    const double tol = t / 1e10;
#pragma unroll
    for (int i = 0; i < 3; i++) xa[i] = (v13[i] + v42[i]) / 2.;
    t = sqrt(xa[0] * xa[0] + xa[1] * xa[1] + xa[2] * xa[2]);
    xa[0] /= t; xa[1] /= t; xa[2] /= t;
    y[0] = z[1] * xa[2] - z[2] * xa[1];
    y[1] = z[2] * xa[0] - z[0] * xa[2];
    y[2] = z[0] * xa[1] - z[1] * xa[0];
    t = sqrt(y[0] * y[0] + y[1] * y[1] + y[2] * y[2]);
    y[0] /= t; y[1] /= t; y[2] /= t;
#pragma unroll
    for (int i = 0; i < 3; i++) {
        R[3 * i + 0] = xa[i];
        R[3 * i + 1] = y[i];
        R[3 * i + 2] = z[i];
    }
    if (!xmat) return;
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
    const bool thick = P[SP_H] / sqrt(ar) >= 1.;
    s.flags = F_VALID | (thick ? F_THICK : 0) | (global_frame ? 0 : F_ROTATE);
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

struct KC0Smem {
    ElemS se[TILE];
    double sgp[TILE][NPT][GPW];
    double stage[NT / 32][2][KSTAGE];
};

__global__ void __launch_bounds__(NT, 3) quad4_kc0_kernel(Q4Args a) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    KC0Smem &S = *reinterpret_cast<KC0Smem *>(smem_raw);
    ElemS *se = S.se;
    auto &sgp = S.sgp;
    auto &stage = S.stage;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int64_t ntiles = (a.E + TILE - 1) / TILE;
    for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int64_t e0 = tile * TILE;
        __syncthreads();
        if (tid < TILE) {
            const int64_t e = e0 + tid;
            if (e < a.E) kc0_phase_a(a, e, se[tid]);
            else se[tid].flags = 0;
        }
        __syncthreads();
        for (int it = tid; it < TILE * NPT; it += NT) {
            const int el = it / NPT, g = it % NPT;
            if (!(se[el].flags & F_VALID)) continue;
            double xi, eta, detJ, N[4], Nx[4], Ny[4];
            point_coords(g, xi, eta);
            quad_derivs(se[el].xy, xi, eta, detJ, N, Nx, Ny);
            double *o = sgp[el][g];
            o[0] = (g == 4) ? 4. * detJ : detJ;
#pragma unroll
            for (int i = 0; i < 4; i++) {
                o[1 + i] = N[i];
                o[5 + i] = Nx[i];
                o[9 + i] = Ny[i];
            }
        }
        __syncthreads();
        // phase B: each warp owns 2 elements per round, 16 node pairs each
        const int half = lane >> 4, pair = lane & 15, na = pair >> 2, nb = pair & 3;
        for (int round = 0; round < TILE / 8; round++) {
            const int el = round * 8 + warp * 2 + half;
            const ElemS &s = se[el];
            const bool valid = s.flags & F_VALID;
            if (valid) {
                double H[3][3], H0[3][3], Hs[3][3];
#pragma unroll
                for (int p = 0; p < 3; p++)
#pragma unroll
                    for (int q = 0; q < 3; q++) H[p][q] = 0.;
#pragma unroll
                for (int g = 0; g < 4; g++) {
                    const double *o = sgp[el][g];
                    const double w = o[0];
                    const double va[3] = {w * o[1 + na], w * o[5 + na], w * o[9 + na]};
                    const double vb[3] = {o[1 + nb], o[5 + nb], o[9 + nb]};
#pragma unroll
                    for (int p = 0; p < 3; p++)
#pragma unroll
                        for (int q = 0; q < 3; q++) H[p][q] += va[p] * vb[q];
                }
                {
                    const double *o = sgp[el][4];
                    const double w = o[0];
                    const double va[3] = {w * o[1 + na], w * o[5 + na], w * o[9 + na]};
                    const double vb[3] = {o[1 + nb], o[5 + nb], o[9 + nb]};
#pragma unroll
                    for (int p = 0; p < 3; p++)
#pragma unroll
                        for (int q = 0; q < 3; q++) H0[p][q] = va[p] * vb[q];
                }
                const bool thick = s.flags & F_THICK;
#pragma unroll
                for (int p = 0; p < 3; p++)
#pragma unroll
                    for (int q = 0; q < 3; q++) Hs[p][q] = thick ? H[p][q] : H0[p][q];
                double K[6][6];
                kc0_block(H, H0, Hs, s.abd, s.es, K);
                if (s.flags & F_ROTATE) rotate_block(s.R, K);
                double *st = stage[warp][half];
#pragma unroll
                for (int m = 0; m < 6; m++)
#pragma unroll
                    for (int n = 0; n < 6; n++) st[(6 * na + m) * KROW + 6 * nb + n] = K[m][n];
            }
            __syncwarp();
            // coalesced write-out of the warp's two elements
#pragma unroll
            for (int h = 0; h < 2; h++) {
                const ElemS &t = se[round * 8 + warp * 2 + h];
                if (!(t.flags & F_VALID)) continue;
                const long long k0 = t.init_k;
                const double *st = stage[warp][h];
                double *kv = a.Kv + k0;
#pragma unroll 6
                for (int i = lane; i < 576; i += 32) {
                    const int row = i / 24, col = i - row * 24;
                    kv[i] += st[row * KROW + col];
                }
                if (!a.values_only) {
                    long long *kr = (long long *)a.Kr + k0, *kc = (long long *)a.Kc + k0;
#pragma unroll 6
                    for (int i = lane; i < 576; i += 32) {
                        const int row = i / 24, col = i - row * 24;
                        kr[i] = t.c[row / 6] + row % 6;
                        kc[i] = t.c[col / 6] + col % 6;
                    }
                }
            }
            __syncwarp();
        }
    }
}

// --- frame / probe kernels --------------------------------------------------
__global__ void quad4_frame_kernel(int64_t E, const int64_t *cdof, const double *x, int64_t nx,
                                   const double *xmat, int xmat_stride, double *Ro, double *mo,
                                   double *xeo, double *areao, int *err) {
    const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= E) return;
    long long c[4];
#pragma unroll
    for (int i = 0; i < 4; i++) {
        c[i] = cdof[4 * e + i];
        if (c[i] < 0 || c[i] / 2 + 3 > nx) {
            raise_error(err, kErrBounds);
            return;
        }
    }
    const double *pp[4] = {x + c[0] / 2, x + c[1] / 2, x + c[2] / 2, x + c[3] / 2};
    double R[9], m[4] = {1., 0., 0., 1.};
    if (mo) {
#pragma unroll
        for (int i = 0; i < 4; i++) m[i] = mo[4 * e + i];
    }
    q4_rotation(pp[0], pp[1], pp[2], pp[3], xmat ? xmat + (int64_t)xmat_stride * e : nullptr, R, m);
    if (Ro)
#pragma unroll
        for (int i = 0; i < 9; i++) Ro[9 * e + i] = R[i];
    if (mo)
#pragma unroll
        for (int i = 0; i < 4; i++) mo[4 * e + i] = m[i];
    double xe[12];
#pragma unroll
    for (int i = 0; i < 4; i++) to_local(R, pp[i], xe + 3 * i);
    if (xeo)
#pragma unroll
        for (int i = 0; i < 12; i++) xeo[12 * e + i] = xe[i];
    if (areao) {
        const double xy[8] = {xe[0], xe[1], xe[3], xe[4], xe[6], xe[7], xe[9], xe[10]};
        areao[e] = shoelace(xy);
    }
}

// Quad4.update_probe_xe with the frame held by the element (quad4.pyx:682-752).
__global__ void quad4_probe_xe_kernel(int64_t E, const int64_t *cdof, const double *x, int64_t nx,
                                      const double *R, double *xeo, double *areao, int *err) {
    const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= E) return;
    double r[9], xe[12];
#pragma unroll
    for (int i = 0; i < 9; i++) r[i] = R[9 * e + i];
#pragma unroll
    for (int i = 0; i < 4; i++) {
        const long long c = cdof[4 * e + i];
        if (c < 0 || c / 2 + 3 > nx) {
            raise_error(err, kErrBounds);
            return;
        }
        to_local(r, x + c / 2, xe + 3 * i);
    }
    if (xeo)
#pragma unroll
        for (int i = 0; i < 12; i++) xeo[12 * e + i] = xe[i];
    if (areao) {
        const double xy[8] = {xe[0], xe[1], xe[3], xe[4], xe[6], xe[7], xe[9], xe[10]};
        areao[e] = shoelace(xy);
    }
}

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

// --- KG (quad4.pyx:1365-2257) ----------------------------------------------
// Phase A: frame, ue and the in-plane stress resultants at the 4 Gauss
// points; phase B: one thread per node pair writes the 3x3 translational
// block r_m3 r_n3 G_ab of the row-major 12x12 layout.
constexpr int KG_ROW = 13;
struct __align__(16) KGElemS {
    double R[9];
    double g[4][11];   // per Gauss point: Nx[4], Ny[4], detJ*Nxx, detJ*Nyy, detJ*Nxy
    long long init_k;
    long long c[4];
    int flags;
    int pad;
};

__global__ void __launch_bounds__(NT) quad4_kg_kernel(Q4Args a, const double *u, int64_t nu,
                                                      const double *ue_in) {
    __shared__ KGElemS se[TILE];
    __shared__ double stage[NT / 32][2][12 * KG_ROW];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int64_t ntiles = (a.E + TILE - 1) / TILE;
    for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int64_t e0 = tile * TILE;
        __syncthreads();
        if (tid < TILE) {
            KGElemS &s = se[tid];
            s.flags = 0;
            const int64_t e = e0 + tid;
            if (e < a.E) {
                long long c[4];
                bool ok = true;
                for (int i = 0; i < 4; i++) {
                    c[i] = a.cdof[4 * e + i];
                    s.c[i] = c[i];
                    if (c[i] < 0) ok = false;
                    if (a.x && c[i] / 2 + 3 > a.nx) ok = false;
                    if (a.x && c[i] + 6 > nu) ok = false;
                }
                const long long k0 = a.init_k[e];
                s.init_k = k0;
                if (k0 < 0 || k0 + 144 > a.nk) ok = false;
                const int64_t p = a.pid ? (int64_t)a.pid[e] : e;
                if (p < 0 || p >= a.nprops) ok = false;
                if (!ok) {
                    raise_error(a.err, kErrBounds);
                } else {
                    double R[9], m[4] = {1., 0., 0., 1.}, xy[8], ue[24];
                    if (a.x) {
                        const double *pp[4] = {a.x + c[0] / 2, a.x + c[1] / 2, a.x + c[2] / 2,
                                               a.x + c[3] / 2};
                        q4_rotation(pp[0], pp[1], pp[2], pp[3],
                                    a.xmat ? a.xmat + (int64_t)a.xmat_stride * e : nullptr, R, m);
                        for (int i = 0; i < 4; i++) {
                            double q[3];
                            to_local(R, pp[i], q);
                            xy[2 * i] = q[0];
                            xy[2 * i + 1] = q[1];
                            to_local(R, u + c[i], ue + 6 * i);
                            to_local(R, u + c[i] + 3, ue + 6 * i + 3);
                        }
                    } else {
                        for (int i = 0; i < 9; i++) R[i] = a.R[9 * e + i];
                        for (int i = 0; i < 4; i++) m[i] = a.m[4 * e + i];
                        for (int i = 0; i < 4; i++) {
                            xy[2 * i] = a.xe[12 * e + 3 * i];
                            xy[2 * i + 1] = a.xe[12 * e + 3 * i + 1];
                        }
                        for (int i = 0; i < 24; i++) ue[i] = ue_in[24 * e + i];
                    }
                    for (int i = 0; i < 9; i++) s.R[i] = R[i];
                    const double *P = a.props + (int64_t)SP_STRIDE * p;
                    double A[6], B[6];
                    if (m[1] == 0.) {
                        for (int i = 0; i < 6; i++) {
                            A[i] = P[SP_A11 + i];
                            B[i] = P[SP_B11 + i];
                        }
                    } else {
                        rotate_plane(m[0], m[1], m[2], m[3], P + SP_A11, A);
                        rotate_plane(m[0], m[1], m[2], m[3], P + SP_B11, B);
                    }
                    for (int g = 0; g < 4; g++) {
                        double xi, eta, detJ, N[4], Nx[4], Ny[4];
                        point_coords(g, xi, eta);
                        quad_derivs(xy, xi, eta, detJ, N, Nx, Ny);
                        double exx = 0, eyy = 0, gxy = 0, kxx = 0, kyy = 0, kxy = 0;
                        for (int i = 0; i < 4; i++) {
                            const double *ui = ue + 6 * i;
                            exx += Nx[i] * ui[0];
                            eyy += Ny[i] * ui[1];
                            gxy += Ny[i] * ui[0] + Nx[i] * ui[1];
                            kxx += Nx[i] * ui[4];
                            kyy -= Ny[i] * ui[3];
                            kxy += Ny[i] * ui[4] - Nx[i] * ui[3];
                            s.g[g][i] = Nx[i];
                            s.g[g][4 + i] = Ny[i];
                        }
                        s.g[g][8] = detJ * (A[0] * exx + A[1] * eyy + A[2] * gxy + B[0] * kxx + B[1] * kyy + B[2] * kxy);
                        s.g[g][9] = detJ * (A[1] * exx + A[3] * eyy + A[4] * gxy + B[1] * kxx + B[3] * kyy + B[4] * kxy);
                        s.g[g][10] = detJ * (A[2] * exx + A[4] * eyy + A[5] * gxy + B[2] * kxx + B[4] * kyy + B[5] * kxy);
                    }
                    s.flags = F_VALID;
                }
            }
        }
        __syncthreads();
        const int half = lane >> 4, pair = lane & 15, na = pair >> 2, nb = pair & 3;
        for (int round = 0; round < TILE / 8; round++) {
            const int el = round * 8 + warp * 2 + half;
            const KGElemS &s = se[el];
            if (s.flags & F_VALID) {
                double G = 0.;
#pragma unroll
                for (int g = 0; g < 4; g++) {
                    const double *o = s.g[g];
                    const double ax = o[na], ay = o[4 + na], bx = o[nb], by = o[4 + nb];
                    G += bx * (ax * o[8] + ay * o[10]) + by * (ax * o[10] + ay * o[9]);
                }
                const double r3[3] = {s.R[2], s.R[5], s.R[8]};
                double *st = stage[warp][half];
#pragma unroll
                for (int mm = 0; mm < 3; mm++)
#pragma unroll
                    for (int nn = 0; nn < 3; nn++) st[(3 * na + mm) * KG_ROW + 3 * nb + nn] = r3[mm] * r3[nn] * G;
            }
            __syncwarp();
#pragma unroll
            for (int h = 0; h < 2; h++) {
                const KGElemS &t = se[round * 8 + warp * 2 + h];
                if (!(t.flags & F_VALID)) continue;
                const long long k0 = t.init_k;
                const double *st = stage[warp][h];
                for (int i = lane; i < 144; i += 32) {
                    const int row = i / 12, col = i - row * 12;
                    a.Kv[k0 + i] += st[row * KG_ROW + col];
                    a.Kr[k0 + i] = t.c[row / 3] + row % 3;
                    a.Kc[k0 + i] = t.c[col / 3] + col % 3;
                }
            }
            __syncwarp();
        }
    }
}

// --- M (quad4.pyx:3083-9489) -------------------------------------------------
// M_ab = h_ab G with h_ab = int N_a N_b (2x2 Gauss, area/16, or 2x2 Lobatto)
// and G = R L R^T, L = [intrho on u,v,w; (u,ry) = intrhoz, (v,rx) = -intrhoz;
// intrhoz2 on rx,ry] (local).  Slot layout: mtype 0/1 skip (m,n) with
// |m-n| = 3 (20 slots per row); mtype 2 keeps only translation-translation
// and rotation-rotation blocks (12 slots per row).
struct __align__(16) MElemS {
    double G[36];
    double h[16];
    long long init_k;
    long long c[4];
    int flags;
    int pad;
};

__global__ void __launch_bounds__(NT) quad4_m_kernel(Q4Args a, int mtype) {
    __shared__ MElemS se[TILE];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int64_t ntiles = (a.E + TILE - 1) / TILE;
    const int ncol = (mtype == 2) ? 12 : 20;
    const int size = 24 * ncol;
    for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int64_t e0 = tile * TILE;
        __syncthreads();
        if (tid < TILE) {
            MElemS &s = se[tid];
            s.flags = 0;
            const int64_t e = e0 + tid;
            if (e < a.E) {
                long long c[4];
                bool ok = true;
                for (int i = 0; i < 4; i++) {
                    c[i] = a.cdof[4 * e + i];
                    s.c[i] = c[i];
                    if (c[i] < 0 || (a.x && c[i] / 2 + 3 > a.nx)) ok = false;
                }
                const long long k0 = a.init_k[e];
                s.init_k = k0;
                if (k0 < 0 || k0 + size > a.nk) ok = false;
                const int64_t p = a.pid ? (int64_t)a.pid[e] : e;
                if (p < 0 || p >= a.nprops) ok = false;
                if (!ok) {
                    raise_error(a.err, kErrBounds);
                } else {
                    double R[9], xy[8], ar;
                    if (a.x) {
                        double m[4] = {1., 0., 0., 1.};
                        const double *pp[4] = {a.x + c[0] / 2, a.x + c[1] / 2, a.x + c[2] / 2,
                                               a.x + c[3] / 2};
                        q4_rotation(pp[0], pp[1], pp[2], pp[3], nullptr, R, m);
                        for (int i = 0; i < 4; i++) {
                            double q[3];
                            to_local(R, pp[i], q);
                            xy[2 * i] = q[0];
                            xy[2 * i + 1] = q[1];
                        }
                        ar = shoelace(xy);
                    } else {
                        for (int i = 0; i < 9; i++) R[i] = a.R[9 * e + i];
                        for (int i = 0; i < 4; i++) {
                            xy[2 * i] = a.xe[12 * e + 3 * i];
                            xy[2 * i + 1] = a.xe[12 * e + 3 * i + 1];
                        }
                        ar = a.area[e];
                    }
                    for (int i = 0; i < 16; i++) s.h[i] = 0.;
                    if (mtype == 1) {
                        for (int i = 0; i < 16; i++) s.h[i] = 0.0625 * ar;
                    } else {
                        for (int g = 0; g < 4; g++) {
                            double xi = (g & 2) ? 1. : -1., eta = (g & 1) ? 1. : -1.;
                            if (mtype == 0) {
                                xi *= kGauss;
                                eta *= kGauss;
                            }
                            double detJ, N[4], Nx[4], Ny[4];
                            quad_derivs(xy, xi, eta, detJ, N, Nx, Ny);
                            for (int i = 0; i < 4; i++)
                                for (int j = 0; j < 4; j++) s.h[4 * i + j] += N[i] * N[j] * detJ;
                        }
                    }
                    const double *P = a.props + (int64_t)SP_STRIDE * p;
                    const double rho = P[SP_RHO], rz = P[SP_RHOZ], rz2 = P[SP_RHOZ2];
                    for (int mm = 0; mm < 3; mm++)
                        for (int nn = 0; nn < 3; nn++) {
                            const double *ri = R + 3 * mm, *rj = R + 3 * nn;
                            s.G[6 * mm + nn] = rho * (ri[0] * rj[0] + ri[1] * rj[1] + ri[2] * rj[2]);
                            const double tr = rz * (ri[0] * rj[1] - ri[1] * rj[0]);
                            s.G[6 * mm + nn + 3] = tr;
                            s.G[6 * (nn + 3) + mm] = tr;
                            s.G[6 * (mm + 3) + nn + 3] = rz2 * (ri[0] * rj[0] + ri[1] * rj[1]);
                        }
                    s.flags = F_VALID;
                }
            }
        }
        __syncthreads();
        // one warp per element: lanes stream the element's slots in order
        for (int el = warp; el < TILE; el += NT / 32) {
            const MElemS &s = se[el];
            if (!(s.flags & F_VALID)) continue;
            const long long k0 = s.init_k;
            for (int i = lane; i < size; i += 32) {
                const int row = i / ncol, j = i - row * ncol;
                const int na = row / 6, mm = row % 6;
                int nb, nn;
                if (mtype == 2) {
                    nb = j / 3;
                    nn = (mm < 3 ? 0 : 3) + j % 3;
                } else {
                    nb = j / 5;
                    const int jj = j % 5, skip = (mm + 3) % 6;
                    nn = jj + (jj >= skip ? 1 : 0);
                }
                a.Kv[k0 + i] += s.h[4 * na + nb] * s.G[6 * mm + nn];
                a.Kr[k0 + i] = s.c[na] + mm;
                a.Kc[k0 + i] = s.c[nb] + nn;
            }
        }
    }
}

// --- fint (quad4.pyx:1174-1201, 1316-1362) ------------------------------------
// Thread per (element, node pair): f_a += Ke_ab ue_b (local), rotated to
// global; the four pair contributions of a node are summed in registers by
// the 4 lanes sharing node a, then added atomically (elements share nodes).
__global__ void __launch_bounds__(NT, 3) quad4_fint_kernel(Q4Args a, const double *ue_in,
                                                           double *fint, int64_t nf) {
    __shared__ ElemS se[TILE];
    __shared__ double sgp[TILE][NPT][GPW];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int64_t ntiles = (a.E + TILE - 1) / TILE;
    for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int64_t e0 = tile * TILE;
        __syncthreads();
        if (tid < TILE) {
            const int64_t e = e0 + tid;
            if (e < a.E) {
                kc0_phase_a(a, e, se[tid]);
                for (int i = 0; i < 4; i++)
                    if (se[tid].c[i] + 6 > nf) {
                        raise_error(a.err, kErrBounds);
                        se[tid].flags = 0;
                    }
            } else {
                se[tid].flags = 0;
            }
        }
        __syncthreads();
        for (int it = tid; it < TILE * NPT; it += NT) {
            const int el = it / NPT, g = it % NPT;
            if (!(se[el].flags & F_VALID)) continue;
            double xi, eta, detJ, N[4], Nx[4], Ny[4];
            point_coords(g, xi, eta);
            quad_derivs(se[el].xy, xi, eta, detJ, N, Nx, Ny);
            double *o = sgp[el][g];
            o[0] = (g == 4) ? 4. * detJ : detJ;
            for (int i = 0; i < 4; i++) {
                o[1 + i] = N[i];
                o[5 + i] = Nx[i];
                o[9 + i] = Ny[i];
            }
        }
        __syncthreads();
        const int half = lane >> 4, pair = lane & 15, na = pair >> 2, nb = pair & 3;
        for (int round = 0; round < TILE / 8; round++) {
            const int el = round * 8 + warp * 2 + half;
            const int64_t e = e0 + el;
            const ElemS &s = se[el];
            double f[6] = {0., 0., 0., 0., 0., 0.};
            if (s.flags & F_VALID) {
                double H[3][3] = {}, H0[3][3], Hs[3][3];
                for (int g = 0; g < 4; g++) {
                    const double *o = sgp[el][g];
                    const double w = o[0];
                    const double va[3] = {w * o[1 + na], w * o[5 + na], w * o[9 + na]};
                    const double vb[3] = {o[1 + nb], o[5 + nb], o[9 + nb]};
                    for (int p = 0; p < 3; p++)
                        for (int q = 0; q < 3; q++) H[p][q] += va[p] * vb[q];
                }
                const double *o = sgp[el][4];
                const double va[3] = {o[0] * o[1 + na], o[0] * o[5 + na], o[0] * o[9 + na]};
                const double vb[3] = {o[1 + nb], o[5 + nb], o[9 + nb]};
                for (int p = 0; p < 3; p++)
                    for (int q = 0; q < 3; q++) H0[p][q] = va[p] * vb[q];
                const bool thick = s.flags & F_THICK;
                for (int p = 0; p < 3; p++)
                    for (int q = 0; q < 3; q++) Hs[p][q] = thick ? H[p][q] : H0[p][q];
                double K[6][6];
                kc0_block(H, H0, Hs, s.abd, s.es, K);
                // fint uses local Ke and local ue (probe mode): rotate f only.
                const double *ueb = ue_in + 24 * e + 6 * nb;
                double fl[6];
                for (int mm = 0; mm < 6; mm++) {
                    double t = 0.;
                    for (int nn = 0; nn < 6; nn++) t += K[mm][nn] * ueb[nn];
                    fl[mm] = t;
                }
                for (int g = 0; g < 2; g++)
                    for (int i = 0; i < 3; i++)
                        f[3 * g + i] = s.R[3 * i] * fl[3 * g] + s.R[3 * i + 1] * fl[3 * g + 1] +
                                       s.R[3 * i + 2] * fl[3 * g + 2];
            }
            // sum the 4 pairs (a, 0..3) held by lanes 4a..4a+3 of the half warp
            for (int i = 0; i < 6; i++) {
                f[i] += __shfl_xor_sync(0xffffffffu, f[i], 1);
                f[i] += __shfl_xor_sync(0xffffffffu, f[i], 2);
            }
            if ((s.flags & F_VALID) && nb == 0)
                for (int i = 0; i < 6; i++) atomicAdd(fint + s.c[na] + i, f[i]);
        }
    }
}

inline int grid_for(int64_t E, int per_sm) {
    const int64_t tiles = (E + TILE - 1) / TILE;
    const int64_t cap = (int64_t)kSMs * per_sm;
    return (int)(tiles < cap ? (tiles > 0 ? tiles : 1) : cap);
}

}  // namespace
}  // namespace fe3d

using namespace fe3d;

extern "C" int fe3d_quad4_frame(int64_t E, const int64_t *cdof, const double *x, int64_t nx,
                                const double *xmat, int xmat_stride, double *R, double *m,
                                double *xe, double *area, int *err, void *stream) {
    if (E < 0 || (E > 0 && (!cdof || !x))) return FE3D_ERR_ARG;
    if (xmat && xmat_stride != 0 && xmat_stride != 3) return FE3D_ERR_ARG;
    if (E == 0) return FE3D_OK;
    const int bs = 128;
    quad4_frame_kernel<<<(unsigned)((E + bs - 1) / bs), bs, 0, as_stream(stream)>>>(
        E, cdof, x, nx, xmat, xmat_stride, R, m, xe, area, err);
    FE3D_CHECK_LAUNCH();
    return FE3D_OK;
}

extern "C" int fe3d_quad4_probe_xe(int64_t E, const int64_t *cdof, const double *x, int64_t nx,
                                   const double *R, double *xe, double *area, int *err,
                                   void *stream) {
    if (E < 0 || (E > 0 && (!cdof || !x || !R))) return FE3D_ERR_ARG;
    if (E == 0) return FE3D_OK;
    const int bs = 128;
    quad4_probe_xe_kernel<<<(unsigned)((E + bs - 1) / bs), bs, 0, as_stream(stream)>>>(E, cdof, x, nx,
                                                                                        R, xe, area, err);
    FE3D_CHECK_LAUNCH();
    return FE3D_OK;
}

extern "C" int fe3d_quad4_probe_ue(int64_t E, const int64_t *cdof, const double *u, int64_t nu,
                                   const double *R, double *ue, int *err, void *stream) {
    if (E < 0 || (E > 0 && (!cdof || !u || !R || !ue))) return FE3D_ERR_ARG;
    if (E == 0) return FE3D_OK;
    const int bs = 128;
    probe_ue_kernel<4><<<(unsigned)((E + bs - 1) / bs), bs, 0, as_stream(stream)>>>(E, cdof, u, nu, R,
                                                                                   ue, err);
    FE3D_CHECK_LAUNCH();
    return FE3D_OK;
}

extern "C" int fe3d_quad4_kc0(int64_t E, const int64_t *cdof, const int64_t *init_k,
                              const double *x, int64_t nx, const double *xmat, int xmat_stride,
                              const double *R, const double *m, const double *xe,
                              const double *area, const double *props, int64_t nprops,
                              const int32_t *pid, int64_t *Kr, int64_t *Kc, double *Kv, int64_t nk,
                              int values_only, int *err, void *stream) {
    if (E < 0) return FE3D_ERR_ARG;
    if (E == 0) return FE3D_OK;
    if (!cdof || !init_k || !props || !Kv || nprops <= 0) return FE3D_ERR_ARG;
    if (!values_only && (!Kr || !Kc)) return FE3D_ERR_ARG;
    if (!x && (!R || !m || !xe || !area)) return FE3D_ERR_ARG;
    if (xmat && xmat_stride != 0 && xmat_stride != 3) return FE3D_ERR_ARG;
    Q4Args a{E, cdof, init_k, x, nx, xmat, xmat_stride, R, m, xe, area, props, nprops, pid,
             Kr, Kc, Kv, nk, values_only, err};
    static bool attr_set = false;
    if (!attr_set) {
        FE3D_CUDA(cudaFuncSetAttribute(quad4_kc0_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)sizeof(KC0Smem)));
        attr_set = true;
    }
    quad4_kc0_kernel<<<grid_for(E, 3), NT, sizeof(KC0Smem), as_stream(stream)>>>(a);
    FE3D_CHECK_LAUNCH();
    return FE3D_OK;
}

extern "C" int fe3d_quad4_kg(int64_t E, const int64_t *cdof, const int64_t *init_k,
                             const double *x, int64_t nx, const double *xmat, int xmat_stride,
                             const double *u, int64_t nu, const double *R, const double *m,
                             const double *xe, const double *ue, const double *props,
                             int64_t nprops, const int32_t *pid, int64_t *Kr, int64_t *Kc,
                             double *Kv, int64_t nk, int *err, void *stream) {
    if (E < 0) return FE3D_ERR_ARG;
    if (E == 0) return FE3D_OK;
    if (!cdof || !init_k || !props || !Kv || !Kr || !Kc || nprops <= 0) return FE3D_ERR_ARG;
    if (x && !u) return FE3D_ERR_ARG;
    if (!x && (!R || !m || !xe || !ue)) return FE3D_ERR_ARG;
    if (xmat && xmat_stride != 0 && xmat_stride != 3) return FE3D_ERR_ARG;
    Q4Args a{E, cdof, init_k, x, nx, xmat, xmat_stride, R, m, xe, nullptr, props, nprops, pid,
             Kr, Kc, Kv, nk, 0, err};
    quad4_kg_kernel<<<grid_for(E, 4), NT, 0, as_stream(stream)>>>(a, u, nu, ue);
    FE3D_CHECK_LAUNCH();
    return FE3D_OK;
}

extern "C" int fe3d_quad4_m(int64_t E, const int64_t *cdof, const int64_t *init_k,
                            const double *x, int64_t nx, const double *R, const double *xe,
                            const double *area, const double *props, int64_t nprops,
                            const int32_t *pid, int64_t *Kr, int64_t *Kc, double *Kv, int64_t nk,
                            int mtype, int *err, void *stream) {
    if (E < 0 || mtype < 0 || mtype > 2) return FE3D_ERR_ARG;
    if (E == 0) return FE3D_OK;
    if (!cdof || !init_k || !props || !Kv || !Kr || !Kc || nprops <= 0) return FE3D_ERR_ARG;
    if (!x && (!R || !xe || !area)) return FE3D_ERR_ARG;
    Q4Args a{E, cdof, init_k, x, nx, nullptr, 0, R, nullptr, xe, area, props, nprops, pid,
             Kr, Kc, Kv, nk, 0, err};
    quad4_m_kernel<<<grid_for(E, 4), NT, 0, as_stream(stream)>>>(a, mtype);
    FE3D_CHECK_LAUNCH();
    return FE3D_OK;
}

extern "C" int fe3d_quad4_fint(int64_t E, const int64_t *cdof, const double *R, const double *m,
                               const double *xe, const double *area, const double *ue,
                               const double *props, int64_t nprops, const int32_t *pid,
                               double *fint, int64_t nf, int *err, void *stream) {
    if (E < 0) return FE3D_ERR_ARG;
    if (E == 0) return FE3D_OK;
    if (!cdof || !R || !m || !xe || !area || !ue || !props || !fint || nprops <= 0)
        return FE3D_ERR_ARG;
    Q4Args a{E, cdof, nullptr, nullptr, 0, nullptr, 0, R, m, xe, area, props, nprops, pid,
             nullptr, nullptr, nullptr, INT64_MAX, 1, err};
    quad4_fint_kernel<<<grid_for(E, 3), NT, 0, as_stream(stream)>>>(a, ue, fint, nf);
    FE3D_CHECK_LAUNCH();
    return FE3D_OK;
}
