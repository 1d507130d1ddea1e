// Quad4 constitutive stiffness KC0: Quad4.update_KC0 (pyfe3d/quad4.pyx:1204-1313)
// with the local matrix of _update_probe_KC0ve (pyfe3d/quad4.pyx:755-1171).
//
// GB300 organisation.  FP64 issues at 1/64 of the FP32 rate on this part,
// so the kernel keeps FP64 for what needs it -- the element frame, the
// constitutive rotation and the += accumulation into the caller's values --
// and carries the per-node-pair contractions in float-float on the FP32 pipe:
//
//   phase A   one thread per element (FP64): frame R (and material cosines),
//             flatness test, constitutive matrices in the evaluation frame,
//             nodal coordinates relative to node 1, thin/thick flag.
//   phase A2  one thread per (element, point) at the 4 Gauss points and the
//             centre: Jacobian, determinant and Cartesian shape derivatives.
//   phase B   one thread per (element, node pair a <= b): the tensor
//             H^pq_ab = sum_points w detJ D^p N_a D^q N_b, p, q in
//             {N, d/dx, d/dy}, then the 6x6 block K_ab = sum_pq C^pq H^pq and,
//             by symmetry, K_ba = K_ab^T.  Each non-zero entry is converted
//             to double with integer operations and added (FP64) to the
//             caller's value; entries that are exactly zero (10 of 36 per
//             block for flat elements) are += 0 in the reference and are not
//             touched.
//   indices   row/column indices are streamed out coalesced per tile.
//
// Flat elements whose normal is +Z (r13 = r23 = r31 = r32 = 0) are evaluated
// in the global frame with in-plane rotated constitutive matrices, which
// equals R Ke R^T without the transform.  Other elements (and the probe
// mode that reads the element state) use an FP64 evaluation in the element
// frame followed by the block rotation, writing all 36 entries per block.
#include "ff.cuh"
#include "quad4_common.cuh"

namespace fe3d {
namespace {

constexpr int KT = 32;    // elements per CTA iteration
constexpr int KNT = 128;  // threads per CTA
constexpr int KPTS = 5;   // 4 Gauss points + centre
constexpr int KSLOT = 13; // per point: w detJ, N[4], Nx[4], Ny[4]

enum : int { KF_VALID = 1, KF_THICK = 2, KF_FP64 = 4 };

union Slot {
    double d;
    ff f;
};

struct __align__(16) KElem {
    double R[9];
    Slot abd[36];
    Slot es[3];
    Slot xy[8];
    long long init_k;
    long long c[4];
    int flags;
    int pad;
};

struct KSmem {
    KElem el[KT];
    Slot gp[KT][KPTS][KSLOT];
    ff shape[KPTS][3][4];
};

// shape-function values and natural derivatives at the 5 points, float-float:
// [point][0: N, 1: dN/dxi, 2: dN/deta][node]
__constant__ ff c_shape[KPTS][3][4];

// node pairs a <= b packed as 4-bit fields: pair pr = (a, b)
constexpr unsigned long long kPairA = 0x3221110000ull;
constexpr unsigned long long kPairB = 0x3323213210ull;

// zero pattern of a flat element's global 6x6 block (u v w rx ry rz)
__host__ __device__ constexpr bool kc0_nonzero(int m, int n) {
    return !((m == 2 && (n == 0 || n == 1 || n == 5)) || (n == 2 && (m == 0 || m == 1 || m == 5)) ||
             (m == 5 && (n == 3 || n == 4)) || (n == 5 && (m == 3 || m == 4)));
}

__device__ void kc0_phase_a2(const Q4Args &a, int64_t e, KElem &s) {
    s.flags = 0;
    long long c[4];
    bool ok = true;
#pragma unroll
    for (int i = 0; i < 4; i++) {
        c[i] = a.cdof[4 * e + i];
        s.c[i] = c[i];
        if (c[i] < 0 || (a.x && c[i] / 2 + 3 > a.nx)) ok = false;
    }
    const long long k0 = a.init_k[e];
    s.init_k = k0;
    if (k0 < 0 || k0 + 576 > a.nk) ok = false;
    const int64_t p = a.pid ? (int64_t)a.pid[e] : e;
    if (p < 0 || p >= a.nprops) ok = false;
    if (!ok) {
        raise_error(a.err, kErrBounds);
        return;
    }
    const double *P = a.props + (int64_t)SP_STRIDE * p;
    double R[9], m[4] = {1., 0., 0., 1.}, xy[8], abd[36], es[3], ar;
    bool fp64 = true;
    if (a.x) {
        const double *pp[4] = {a.x + c[0] / 2, a.x + c[1] / 2, a.x + c[2] / 2, a.x + c[3] / 2};
        q4_rotation(pp[0], pp[1], pp[2], pp[3], a.xmat ? a.xmat + (int64_t)a.xmat_stride * e : nullptr,
                    R, m);
        if (is_flat(R)) {
#pragma unroll
            for (int i = 0; i < 4; i++) {
                xy[2 * i] = pp[i][0] - pp[0][0];
                xy[2 * i + 1] = pp[i][1] - pp[0][1];
            }
            q4_constitutive(P, m, R, true, abd, es);
            bool safe = true;
#pragma unroll
            for (int i = 0; i < 36; i++) safe &= ff_safe(abd[i]);
#pragma unroll
            for (int i = 0; i < 3; i++) safe &= ff_safe(es[i]);
#pragma unroll
            for (int i = 0; i < 8; i++) safe &= ff_safe(xy[i]);
            fp64 = !safe;
        }
        if (fp64) {
#pragma unroll
            for (int i = 0; i < 4; i++) {
                double q[3];
                to_local(R, pp[i], q);
                xy[2 * i] = q[0];
                xy[2 * i + 1] = q[1];
            }
            q4_constitutive(P, m, R, false, abd, es);
        }
        ar = shoelace(xy);
    } else {
#pragma unroll
        for (int i = 0; i < 9; i++) R[i] = a.R[9 * e + i];
#pragma unroll
        for (int i = 0; i < 4; i++) m[i] = a.m[4 * e + i];
#pragma unroll
        for (int i = 0; i < 4; i++) {
            xy[2 * i] = a.xe[12 * e + 3 * i];
            xy[2 * i + 1] = a.xe[12 * e + 3 * i + 1];
        }
        q4_constitutive(P, m, R, false, abd, es);
        ar = a.area[e];
    }
#pragma unroll
    for (int i = 0; i < 9; i++) s.R[i] = R[i];
    if (fp64) {
#pragma unroll
        for (int i = 0; i < 36; i++) s.abd[i].d = abd[i];
#pragma unroll
        for (int i = 0; i < 3; i++) s.es[i].d = es[i];
#pragma unroll
        for (int i = 0; i < 8; i++) s.xy[i].d = xy[i];
    } else {
#pragma unroll
        for (int i = 0; i < 36; i++) s.abd[i].f = ff_from_double(abd[i]);
#pragma unroll
        for (int i = 0; i < 3; i++) s.es[i].f = ff_from_double(es[i]);
#pragma unroll
        for (int i = 0; i < 8; i++) s.xy[i].f = ff_from_double(xy[i]);
    }
    const bool thick = P[SP_H] / sqrt(ar) >= 1.;
    s.flags = KF_VALID | (thick ? KF_THICK : 0) | (fp64 ? KF_FP64 : 0);
}

// Jacobian and Cartesian derivatives at point g in float-float.
__device__ void point_ff(const KElem &s, const ff (*shape)[3][4], int g, Slot *o) {
    ff x[4], y[4];
#pragma unroll
    for (int i = 0; i < 4; i++) {
        x[i] = s.xy[2 * i].f;
        y[i] = s.xy[2 * i + 1].f;
    }
    ff J11 = ff_mul(x[0], shape[g][1][0]), J12 = ff_mul(y[0], shape[g][1][0]);
    ff J21 = ff_mul(x[0], shape[g][2][0]), J22 = ff_mul(y[0], shape[g][2][0]);
#pragma unroll
    for (int i = 1; i < 4; i++) {
        J11 = ff_fma(x[i], shape[g][1][i], J11);
        J12 = ff_fma(y[i], shape[g][1][i], J12);
        J21 = ff_fma(x[i], shape[g][2][i], J21);
        J22 = ff_fma(y[i], shape[g][2][i], J22);
    }
    const ff det = ff_fma(J11, J22, ff_neg(ff_mul(J12, J21)));
    const ff inv = ff_rcp(det);
    o[0].f = (g == 4) ? ff_scale(det, 4.f) : det;
#pragma unroll
    for (int i = 0; i < 4; i++) {
        const ff dxi = shape[g][1][i], deta = shape[g][2][i];
        o[1 + i].f = shape[g][0][i];
        o[5 + i].f = ff_mul(ff_fma(J22, dxi, ff_neg(ff_mul(J12, deta))), inv);
        o[9 + i].f = ff_mul(ff_fma(J11, deta, ff_neg(ff_mul(J21, dxi))), inv);
    }
}

__device__ __forceinline__ ff ffz() { return {0.f, 0.f}; }

// Float-float 6x6 block of a flat element in the global frame; the same
// strain-displacement relations as kc0_block (quad4.pyx:958-1171).
__device__ __forceinline__ void kc0_block_ff(const ff H[3][3], const ff H0[3][3], const ff Hs[3][3],
                                             const Slot *abd, const Slot *es, ff K[6][6]) {
    const int dof[4] = {0, 1, 3, 4};
    const int sidx[4][2] = {{0, 2}, {2, 1}, {5, 4}, {3, 5}};
    const bool neg[4] = {false, false, true, false};
#pragma unroll
    for (int i = 0; i < 6; i++)
#pragma unroll
        for (int j = 0; j < 6; j++) K[i][j] = ffz();
#pragma unroll
    for (int mi = 0; mi < 4; mi++)
#pragma unroll
        for (int ni = 0; ni < 4; ni++) {
            ff s = ff_mul(abd[6 * sidx[mi][0] + sidx[ni][0]].f, H[1][1]);
            s = ff_fma(abd[6 * sidx[mi][0] + sidx[ni][1]].f, H[1][2], s);
            s = ff_fma(abd[6 * sidx[mi][1] + sidx[ni][0]].f, H[2][1], s);
            s = ff_fma(abd[6 * sidx[mi][1] + sidx[ni][1]].f, H[2][2], s);
            K[dof[mi]][dof[ni]] = (neg[mi] != neg[ni]) ? ff_neg(s) : s;
        }
    // drilling with unit weight: d = u N_y/2 - v N_x/2 + rz N
    K[0][0] = ff_add(K[0][0], ff_scale(H[2][2], 0.25f));
    K[0][1] = ff_add(K[0][1], ff_scale(H[2][1], -0.25f));
    K[1][0] = ff_add(K[1][0], ff_scale(H[1][2], -0.25f));
    K[1][1] = ff_add(K[1][1], ff_scale(H[1][1], 0.25f));
    K[0][5] = ff_scale(H[2][0], 0.5f);
    K[1][5] = ff_scale(H[1][0], -0.5f);
    K[5][0] = ff_scale(H[0][2], 0.5f);
    K[5][1] = ff_scale(H[0][1], -0.5f);
    K[5][5] = H[0][0];
    // transverse shear, (gyz, gxz) = (w_y - rx N, w_x + ry N)
    const ff E44 = es[0].f, E45 = es[1].f, E55 = es[2].f;
    K[2][2] = ff_fma(E44, Hs[2][2], ff_fma(E45, ff_add(Hs[2][1], Hs[1][2]), ff_mul(E55, Hs[1][1])));
    K[2][3] = ff_neg(ff_fma(E44, H0[2][0], ff_mul(E45, H0[1][0])));
    K[2][4] = ff_fma(E45, H0[2][0], ff_mul(E55, H0[1][0]));
    K[3][2] = ff_neg(ff_fma(E44, H0[0][2], ff_mul(E45, H0[0][1])));
    K[4][2] = ff_fma(E45, H0[0][2], ff_mul(E55, H0[0][1]));
    K[3][3] = ff_fma(E44, H0[0][0], K[3][3]);
    K[3][4] = ff_fma(ff_neg(E45), H0[0][0], K[3][4]);
    K[4][3] = ff_fma(ff_neg(E45), H0[0][0], K[4][3]);
    K[4][4] = ff_fma(E55, H0[0][0], K[4][4]);
}

__global__ void __launch_bounds__(KNT, 4) quad4_kc0_ff_kernel(Q4Args a) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    KSmem &S = *reinterpret_cast<KSmem *>(smem_raw);
    const int tid = threadIdx.x;
    for (int i = tid; i < KPTS * 12; i += KNT) (&S.shape[0][0][0])[i] = (&c_shape[0][0][0])[i];
    const int64_t ntiles = (a.E + KT - 1) / KT;
    for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int64_t e0 = tile * KT;
        __syncthreads();
        if (tid < KT) {
            const int64_t e = e0 + tid;
            if (e < a.E) kc0_phase_a2(a, e, S.el[tid]);
            else S.el[tid].flags = 0;
        }
        __syncthreads();
        // phase A2: points
        for (int it = tid; it < KT * KPTS; it += KNT) {
            const int el = it / KPTS, g = it - el * KPTS;
            const KElem &s = S.el[el];
            if (!(s.flags & KF_VALID)) continue;
            Slot *o = S.gp[el][g];
            if (s.flags & KF_FP64) {
                double xi, eta, detJ, N[4], Nx[4], Ny[4], xy[8];
#pragma unroll
                for (int i = 0; i < 8; i++) xy[i] = s.xy[i].d;
                point_coords(g, xi, eta);
                quad_derivs(xy, xi, eta, detJ, N, Nx, Ny);
                o[0].d = (g == 4) ? 4. * detJ : detJ;
#pragma unroll
                for (int i = 0; i < 4; i++) {
                    o[1 + i].d = N[i];
                    o[5 + i].d = Nx[i];
                    o[9 + i].d = Ny[i];
                }
            } else {
                point_ff(s, S.shape, g, o);
            }
        }
        __syncthreads();
        // phase B: node pairs a <= b
        for (int it = tid; it < KT * 10; it += KNT) {
            const int el = it / 10, pr = it - el * 10;
            const KElem &s = S.el[el];
            if (!(s.flags & KF_VALID)) continue;
            const int na = (int)((kPairA >> (4 * pr)) & 0xf), nb = (int)((kPairB >> (4 * pr)) & 0xf);
            double *kv = a.Kv + s.init_k;
            const int base_ab = 24 * 6 * na + 6 * nb, base_ba = 24 * 6 * nb + 6 * na;
            const bool thick = s.flags & KF_THICK;
            if (!(s.flags & KF_FP64)) {
                ff H[3][3], H0[3][3], Hs[3][3];
#pragma unroll
                for (int p = 0; p < 3; p++)
#pragma unroll
                    for (int q = 0; q < 3; q++) H[p][q] = ffz();
#pragma unroll
                for (int g = 0; g < 4; g++) {
                    const Slot *o = S.gp[el][g];
                    const ff w = o[0].f;
                    const ff va[3] = {ff_mul(w, o[1 + na].f), ff_mul(w, o[5 + na].f), ff_mul(w, o[9 + na].f)};
                    const ff vb[3] = {o[1 + nb].f, o[5 + nb].f, o[9 + nb].f};
#pragma unroll
                    for (int p = 0; p < 3; p++)
#pragma unroll
                        for (int q = 0; q < 3; q++) H[p][q] = ff_fma(va[p], vb[q], H[p][q]);
                }
                {
                    const Slot *o = S.gp[el][4];
                    const ff w = o[0].f;
                    const ff va[3] = {ff_mul(w, o[1 + na].f), ff_mul(w, o[5 + na].f), ff_mul(w, o[9 + na].f)};
                    const ff vb[3] = {o[1 + nb].f, o[5 + nb].f, o[9 + nb].f};
#pragma unroll
                    for (int p = 0; p < 3; p++)
#pragma unroll
                        for (int q = 0; q < 3; q++) H0[p][q] = ff_mul(va[p], vb[q]);
                }
#pragma unroll
                for (int p = 0; p < 3; p++)
#pragma unroll
                    for (int q = 0; q < 3; q++) Hs[p][q] = thick ? H[p][q] : H0[p][q];
                ff K[6][6];
                kc0_block_ff(H, H0, Hs, s.abd, s.es, K);
#pragma unroll
                for (int m = 0; m < 6; m++)
#pragma unroll
                    for (int n = 0; n < 6; n++) {
                        if (!kc0_nonzero(m, n)) continue;
                        const double v = ff_to_double(K[m][n]);
                        kv[base_ab + 24 * m + n] += v;
                        if (na != nb) kv[base_ba + 24 * n + m] += v;
                    }
            } else {
                double H[3][3], H0[3][3], Hs[3][3];
#pragma unroll
                for (int p = 0; p < 3; p++)
#pragma unroll
                    for (int q = 0; q < 3; q++) H[p][q] = 0.;
#pragma unroll
                for (int g = 0; g < 4; g++) {
                    const Slot *o = S.gp[el][g];
                    const double w = o[0].d;
                    const double va[3] = {w * o[1 + na].d, w * o[5 + na].d, w * o[9 + na].d};
                    const double vb[3] = {o[1 + nb].d, o[5 + nb].d, o[9 + nb].d};
#pragma unroll
                    for (int p = 0; p < 3; p++)
#pragma unroll
                        for (int q = 0; q < 3; q++) H[p][q] += va[p] * vb[q];
                }
                {
                    const Slot *o = S.gp[el][4];
                    const double w = o[0].d;
                    const double va[3] = {w * o[1 + na].d, w * o[5 + na].d, w * o[9 + na].d};
                    const double vb[3] = {o[1 + nb].d, o[5 + nb].d, o[9 + nb].d};
#pragma unroll
                    for (int p = 0; p < 3; p++)
#pragma unroll
                        for (int q = 0; q < 3; q++) H0[p][q] = va[p] * vb[q];
                }
#pragma unroll
                for (int p = 0; p < 3; p++)
#pragma unroll
                    for (int q = 0; q < 3; q++) Hs[p][q] = thick ? H[p][q] : H0[p][q];
                double abd[36], es[3];
#pragma unroll
                for (int i = 0; i < 36; i++) abd[i] = s.abd[i].d;
#pragma unroll
                for (int i = 0; i < 3; i++) es[i] = s.es[i].d;
                double K[6][6];
                kc0_block(H, H0, Hs, abd, es, K);
                rotate_block(s.R, K);
                for (int m = 0; m < 6; m++)
                    for (int n = 0; n < 6; n++) {
                        kv[base_ab + 24 * m + n] += K[m][n];
                        if (na != nb) kv[base_ba + 24 * n + m] += K[m][n];
                    }
            }
        }
        // indices, coalesced over the tile
        if (!a.values_only) {
            for (int i = tid; i < KT * 576; i += KNT) {
                const int el = i / 576, k = i - el * 576;
                const KElem &s = S.el[el];
                if (!(s.flags & KF_VALID)) continue;
                const int row = k / 24, col = k - row * 24;
                const int64_t dst = s.init_k + k;
                a.Kr[dst] = s.c[row / 6] + row % 6;
                a.Kc[dst] = s.c[col / 6] + col % 6;
            }
        }
    }
}

int g_shape_ready[64] = {0};

int upload_shape_table() {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return FE3D_ERR_CUDA;
    if (dev < 64 && g_shape_ready[dev]) return FE3D_OK;
    ff h[KPTS][3][4];
    const double sx[4] = {-1., 1., 1., -1.}, sy[4] = {-1., -1., 1., 1.};
    for (int g = 0; g < KPTS; g++) {
        double xi, eta;
        if (g == 4) {
            xi = 0.;
            eta = 0.;
        } else {
            xi = (g & 2) ? kGauss : -kGauss;
            eta = (g & 1) ? kGauss : -kGauss;
        }
        for (int i = 0; i < 4; i++) {
            const double v[3] = {0.25 * (1 + sx[i] * xi) * (1 + sy[i] * eta), 0.25 * sx[i] * (1 + sy[i] * eta),
                                 0.25 * sy[i] * (1 + sx[i] * xi)};
            for (int t = 0; t < 3; t++) {
                const float hi = (float)v[t];
                h[g][t][i] = {hi, (float)(v[t] - (double)hi)};
            }
        }
    }
    if (cudaMemcpyToSymbol(c_shape, h, sizeof(h)) != cudaSuccess) return FE3D_ERR_CUDA;
    if (cudaFuncSetAttribute(quad4_kc0_ff_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)sizeof(KSmem)) != cudaSuccess)
        return FE3D_ERR_CUDA;
    if (dev < 64) g_shape_ready[dev] = 1;
    return FE3D_OK;
}

}  // namespace
}  // namespace fe3d

using namespace fe3d;

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
    const int rc = upload_shape_table();
    if (rc) return rc;
    Q4Args a{E, cdof, init_k, x, nx, xmat, xmat_stride, R, m, xe, area, props, nprops, pid,
             Kr, Kc, Kv, nk, values_only, err};
    const int64_t tiles = (E + KT - 1) / KT;
    const int64_t cap = (int64_t)kSMs * 4;
    const int grid = (int)(tiles < cap ? tiles : cap);
    quad4_kc0_ff_kernel<<<grid, KNT, sizeof(KSmem), as_stream(stream)>>>(a);
    FE3D_CHECK_LAUNCH();
    return FE3D_OK;
}
