// Quad4 element kernels: frame, probe xe/ue, KG, M, fint (KC0 lives in
// quad4_kc0.cu).  Element matrices follow pyfe3d/quad4.pyx (cited per
// kernel).  Each kernel stages per-element data with one thread per element
// (full warps for the FP64 frame work) and then spreads the per-node-pair
// work over the threads of the block.
#include "ff.cuh"
#include "quad4_common.cuh"

namespace fe3d {
namespace {

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

// --- KG (quad4.pyx:1365-2257) ----------------------------------------------
// Phase A: one warp forms the frame, ue and the material-frame A and B of
// the tile's 32 elements; phase A2: warp g evaluates Gauss point g (the
// in-plane stress resultants and the vectors detJ Nmat grad N_a) of all 32;
// phase B: one lane per node pair forms the 3x3 translational block
// r_m3 r_n3 G_ab of the row-major 12x12 layout, and the warp adds it onto
// the caller's values, which cp.async has copied to shared memory while the
// blocks were formed.  Elements flat in the global x-y plane have
// r13 = r23 = 0: only their 16 (w, w) values change.
constexpr int KG_ROW = 13;
constexpr int KG_FLATZ = 8;  // element flag: flat with normal along global z
constexpr int KG_FF = 16;    // element flag: Jacobian and derivatives in float-float
constexpr int KG_NOB = 32;   // element flag: B = 0, the resultants need no curvatures
struct __align__(16) KGElemS {
    double rr[9];      // r_m3 r_n3 (translational block pattern)
    double g[4][16];   // per Gauss point: Nx[4], Ny[4], then per node a the
                       // vector detJ Nmat grad N_a (x and y components)
    long long init_k;
    long long c[4];
    int flags;
    int pad;
};

// Phase-A output read by the per-point pass: local in-plane coordinates, and
// ue with A and B in the material frame (or the given resultants in ab[0..2]);
// 45 doubles (odd) so that lanes reading one field hit distinct banks.
struct KGScratch {
    union {
        double xy[8];  // local in-plane coordinates
        ff xyf[8];     // KG_FF: coordinates relative to node 1, float-float
    };
    double ue[24];
    double ab[12];
    double pad;
};

// The first two components of R^T p (the element-frame x and y of p): the KG
// strains read only u, v, rx, ry of each node in the element frame.  On an
// element flat in z the third row of R^T p adds R[6] p2 = R[7] p2 = 0.
__device__ __forceinline__ void to_local_xy(const double *R, const double *p, double *q, bool flatz) {
    if (flatz) {
        q[0] = R[0] * p[0] + R[3] * p[1];
        q[1] = R[1] * p[0] + R[4] * p[1];
    } else {
        q[0] = R[0] * p[0] + R[3] * p[1] + R[6] * p[2];
        q[1] = R[1] * p[0] + R[4] * p[1] + R[7] * p[2];
    }
}

// Jacobian, shape-function derivatives and detJ at Gauss point g from
// float-float coordinates relative to node 1 and the float-float table of
// dN/dxi, dN/deta (sh[g][0..1][node]); results rounded to double with integer
// operations (the FP32 pipe carries the work instead of the FP64 pipe).
__device__ __forceinline__ void kg_point_ff(const ff *xyf, const ff (*sh)[2][4], int g, double &detJ, double *Nx,
                                            double *Ny) {
    ff J11 = ff_mul(xyf[0], sh[g][0][0]), J12 = ff_mul(xyf[1], sh[g][0][0]);
    ff J21 = ff_mul(xyf[0], sh[g][1][0]), J22 = ff_mul(xyf[1], sh[g][1][0]);
#pragma unroll
    for (int i = 1; i < 4; i++) {
        J11 = ff_fma(xyf[2 * i], sh[g][0][i], J11);
        J12 = ff_fma(xyf[2 * i + 1], sh[g][0][i], J12);
        J21 = ff_fma(xyf[2 * i], sh[g][1][i], J21);
        J22 = ff_fma(xyf[2 * i + 1], sh[g][1][i], J22);
    }
    const ff det = ff_fma(J11, J22, ff_neg(ff_mul(J12, J21)));
    const ff inv = ff_rcp(det);
    detJ = ff_to_double(det);
#pragma unroll
    for (int i = 0; i < 4; i++) {
        const ff dxi = sh[g][0][i], deta = sh[g][1][i];
        Nx[i] = ff_to_double(ff_mul(ff_fma(J22, dxi, ff_neg(ff_mul(J12, deta))), inv));
        Ny[i] = ff_to_double(ff_mul(ff_fma(J11, deta, ff_neg(ff_mul(J21, dxi))), inv));
    }
}

// The caller's 144 values of the two elements (el0, el0 + 1) of a warp's
// round, copied into shared memory ahead of the block computation so that
// the += does not wait on one global load per slot.
__device__ __forceinline__ void kg_prefetch(const Q4Args &a, const KGElemS *se, double (*old)[144], int el0,
                                            int lane) {
#pragma unroll
    for (int h = 0; h < 2; h++) {
        const KGElemS &t = se[el0 + h];
        if (!(t.flags & F_VALID)) continue;
        if (t.flags & KG_FLATZ) {
            if (lane < 16) {
                const int i = (3 * (lane >> 2) + 2) * 12 + 3 * (lane & 3) + 2;
                cp_async8(&old[h][i], a.Kv + t.init_k + i);
            }
            continue;
        }
        for (int i = lane; i < 144; i += 32) cp_async8(&old[h][i], a.Kv + t.init_k + i);
    }
    cp_async_commit();
}

// Per Gauss point: from the derivatives o[0..7] and the resultants times
// detJ, the vectors detJ Nmat grad N_a into o[8 + 2a], o[9 + 2a], so that
// G_ab = sum_g grad N_b . (detJ Nmat grad N_a).
__device__ __forceinline__ void kg_point_vectors(double *o, double nxx, double nyy, double nxy) {
#pragma unroll
    for (int a = 0; a < 4; a++) {
        const double ax = o[a], ay = o[4 + a];
        o[8 + 2 * a] = ax * nxx + ay * nxy;
        o[9 + 2 * a] = ax * nxy + ay * nyy;
    }
}

// Phase A of KG in the global frame, for flat isotropic membrane sections
// (A rotation-invariant, B = 0) on elements flat in z with the nodes
// counter-clockwise in the global x-y plane.  With equal z along both
// diagonals the frame's normal is +z exactly (the flatness test of the KC0
// kernel), and G_ab = sum_g grad N_b . (detJ Nmat grad N_a) is invariant
// under the in-plane rotation to the element axes, so the coordinates, u and
// v are used in the global frame, without the frame, the rotation of ue or
// the material direction.  Returns false (nothing written) otherwise.
__device__ __forceinline__ bool kg_setup_global(const Q4Args &a, const long long *c, int64_t p, const double *u,
                                                KGElemS &s, KGScratch &q) {
    const double *p0 = a.x + c[0] / 2, *p1 = a.x + c[1] / 2, *p2 = a.x + c[2] / 2, *p3 = a.x + c[3] / 2;
    if (p2[2] != p0[2] || p1[2] != p3[2]) return false;
    const double cz = (p1[0] - p3[0]) * (p2[1] - p0[1]) - (p1[1] - p3[1]) * (p2[0] - p0[0]);
    const double *P = a.props + (int64_t)SP_STRIDE * p;
    const double eps = 64. * 2.220446049250313e-16;
    bool g = cz > 0. && P[SP_A16] == 0. && P[SP_A26] == 0. && P[SP_A11] == P[SP_A22] &&
             fabs(P[SP_A66] - 0.5 * (P[SP_A11] - P[SP_A12])) <= eps * fabs(P[SP_A11]);
    for (int i = 0; i < 6; i++) g &= P[SP_B11 + i] == 0.;
    if (!g) return false;
    const double *pp[4] = {p0, p1, p2, p3};
    bool ffok = true;
    double d[8];
    for (int i = 0; i < 4; i++) {
        q.xy[2 * i] = pp[i][0];
        q.xy[2 * i + 1] = pp[i][1];
        d[2 * i] = pp[i][0] - p0[0];
        d[2 * i + 1] = pp[i][1] - p0[1];
        ffok &= ff_safe(d[2 * i]) && ff_safe(d[2 * i + 1]);
        q.ue[6 * i] = u[c[i]];
        q.ue[6 * i + 1] = u[c[i] + 1];
    }
    if (ffok)
        for (int i = 0; i < 8; i++) q.xyf[i] = ff_from_double(d[i]);
    for (int i = 0; i < 6; i++) q.ab[i] = P[SP_A11 + i];
    for (int i = 0; i < 9; i++) s.rr[i] = i == 8 ? 1. : 0.;
    s.flags = F_VALID | KG_FLATZ | KG_NOB | (ffok ? KG_FF : 0);
    return true;
}

// The 144 rows and columns of element t at k0: 16-byte stores of slot pairs
// (2 q, 2 q + 1) (same row; columns of one node or of two neighbouring
// nodes) when the arrays and k0 allow, else 8-byte stores.
__device__ __forceinline__ void kg_write_indices(const Q4Args &a, const KGElemS &t, long long k0, int lane) {
    if (a.vec16 && !(k0 & 1)) {
        for (int q = lane; q < 72; q += 32) {
            const int i = 2 * q, row = i / 12, col = i - row * 12;
            const long long r = t.c[row / 3] + row % 3;
            *reinterpret_cast<longlong2 *>(a.Kr + k0 + i) = make_longlong2(r, r);
            *reinterpret_cast<longlong2 *>(a.Kc + k0 + i) =
                make_longlong2(t.c[col / 3] + col % 3, t.c[(col + 1) / 3] + (col + 1) % 3);
        }
        return;
    }
    for (int i = lane; i < 144; i += 32) {
        const int row = i / 12, col = i - row * 12;
        a.Kr[k0 + i] = t.c[row / 3] + row % 3;
        a.Kc[k0 + i] = t.c[col / 3] + col % 3;
    }
}

// With nstress (update_KG_given_stress, quad4.pyx:2259-3081): the stress
// resultants are the given constants (Nxx, Nyy, Nxy) of the element
// (nstress + ns_stride e) at every Gauss point instead of those of ue.
__global__ void __launch_bounds__(NT, 4) quad4_kg_kernel(Q4Args a, const double *u, int64_t nu,
                                                      const double *ue_in, const double *nstress,
                                                      int ns_stride) {
    __shared__ KGElemS se[TILE];
    // the per-point scratch is dead once the points are done: the caller's
    // values of each warp's round reuse its memory (static total under 48 KB)
    __shared__ union {
        KGScratch sq[TILE];
        double oldv[NT / 32][2][144];
    } su;
    KGScratch *sq = su.sq;
    double(*oldv)[2][144] = su.oldv;
    __shared__ double stage[NT / 32][2][12 * KG_ROW];
    // dN/dxi and dN/deta of the 4 nodes at the 4 Gauss points, float-float
    __shared__ ff shf[4][2][4];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (tid < 32) {
        const int g = tid >> 3, d = (tid >> 2) & 1, i = tid & 3;
        double xi, eta;
        point_coords(g, xi, eta);
        const double sx = (i == 1 || i == 2) ? 1. : -1., sy = (i >= 2) ? 1. : -1.;
        shf[g][d][i] = ff_from_double(d == 0 ? 0.25 * sx * (1 + sy * eta) : 0.25 * sy * (1 + sx * xi));
    }
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
                    if (a.x && !nstress && c[i] + 6 > nu) ok = false;
                }
                const long long k0 = a.init_k[e];
                s.init_k = k0;
                if (k0 < 0 || k0 + 144 > a.nk) ok = false;
                const int64_t p = a.pid ? (int64_t)a.pid[e] : e;
                if (!nstress && (p < 0 || p >= a.nprops)) ok = false;
                if (!ok) {
                    raise_error(a.err, kErrBounds);
                } else {
                    // xy and ue go straight to the shared scratch of the per-point pass
                    KGScratch &q = sq[tid];
                    double R[9], m[4] = {1., 0., 0., 1.}, *xy = q.xy, *ue = q.ue;
                    bool ffok = false;
                    if (a.x && !nstress && kg_setup_global(a, c, p, u, s, q)) {
                        // set up in the global frame
                    } else {
                        if (a.x) {
                            const double *pp[4] = {a.x + c[0] / 2, a.x + c[1] / 2, a.x + c[2] / 2,
                                                   a.x + c[3] / 2};
                            q4_rotation(pp[0], pp[1], pp[2], pp[3],
                                        a.xmat ? a.xmat + (int64_t)a.xmat_stride * e : nullptr, R, m);
                            const bool fz = R[2] == 0. && R[5] == 0.;
                            for (int i = 0; i < 4; i++) {
                                to_local_xy(R, pp[i], xy + 2 * i, fz);
                                if (!nstress) {
                                    to_local_xy(R, u + c[i], ue + 6 * i, fz);
                                    to_local_xy(R, u + c[i] + 3, ue + 6 * i + 3, fz);
                                }
                            }
                            if (fz) {
                                // float-float geometry from coordinates relative to node 1
                                ffok = true;
                                double d[8];
                                for (int i = 0; i < 4; i++) {
                                    d[2 * i] = xy[2 * i] - xy[0];
                                    d[2 * i + 1] = xy[2 * i + 1] - xy[1];
                                    ffok &= ff_safe(d[2 * i]) && ff_safe(d[2 * i + 1]);
                                }
                                if (ffok)
                                    for (int i = 0; i < 8; i++) q.xyf[i] = ff_from_double(d[i]);
                            }
                        } else {
                            for (int i = 0; i < 9; i++) R[i] = a.R[9 * e + i];
                            if (!nstress)
                                for (int i = 0; i < 4; i++) m[i] = a.m[4 * e + i];
                            for (int i = 0; i < 4; i++) {
                                xy[2 * i] = a.xe[12 * e + 3 * i];
                                xy[2 * i + 1] = a.xe[12 * e + 3 * i + 1];
                            }
                            if (!nstress)
                                for (int i = 0; i < 24; i++) ue[i] = ue_in[24 * e + i];
                        }
                        for (int mm = 0; mm < 3; mm++)
                            for (int nn = 0; nn < 3; nn++) s.rr[3 * mm + nn] = R[3 * mm + 2] * R[3 * nn + 2];
                        bool nob = false;
                        if (nstress) {
                            const double *ns = nstress + (int64_t)ns_stride * e;
                            q.ab[0] = ns[0];
                            q.ab[1] = ns[1];
                            q.ab[2] = ns[2];
                        } else {
                            const double *P = a.props + (int64_t)SP_STRIDE * p;
                            if (m[1] == 0.) {
                                for (int i = 0; i < 6; i++) {
                                    q.ab[i] = P[SP_A11 + i];
                                    q.ab[6 + i] = P[SP_B11 + i];
                                }
                            } else {
                                rotate_plane(m[0], m[1], m[2], m[3], P + SP_A11, q.ab);
                                rotate_plane(m[0], m[1], m[2], m[3], P + SP_B11, q.ab + 6);
                            }
                            nob = true;
                            for (int i = 0; i < 6; i++) nob &= q.ab[6 + i] == 0.;
                        }
                        // flat in the global x-y plane: r13 = r23 = 0, so r_m3 r_n3 is
                        // zero but for (w, w) and 128 of the 144 entries are zeros
                        s.flags = F_VALID | ((R[2] == 0. && R[5] == 0.) ? KG_FLATZ : 0) | (ffok ? KG_FF : 0) |
                                  (nob ? KG_NOB : 0);
                    }
                }
            }
        }
        __syncthreads();
        // phase A2: warp g evaluates Gauss point g of the tile's 32 elements
        // (full warps; the four points run on the four sub-partitions)
        for (int w = tid; w < TILE * 4; w += NT) {
            const int el = w & (TILE - 1), g = w / TILE;
            KGElemS &s = se[el];
            if (!(s.flags & F_VALID)) continue;
            const KGScratch &q = sq[el];
            double detJ, Nx[4], Ny[4];
            if (s.flags & KG_FF) {
                kg_point_ff(q.xyf, shf, g, detJ, Nx, Ny);
            } else {
                double xi, eta, N[4];
                point_coords(g, xi, eta);
                quad_derivs(q.xy, xi, eta, detJ, N, Nx, Ny);
            }
            if (nstress) {
                for (int i = 0; i < 4; i++) {
                    s.g[g][i] = Nx[i];
                    s.g[g][4 + i] = Ny[i];
                }
                kg_point_vectors(s.g[g], detJ * q.ab[0], detJ * q.ab[1], detJ * q.ab[2]);
            } else {
                const double *A = q.ab, *B = q.ab + 6;
                double exx = 0, eyy = 0, gxy = 0;
                for (int i = 0; i < 4; i++) {
                    const double *ui = q.ue + 6 * i;
                    exx += Nx[i] * ui[0];
                    eyy += Ny[i] * ui[1];
                    gxy += Ny[i] * ui[0] + Nx[i] * ui[1];
                    s.g[g][i] = Nx[i];
                    s.g[g][4 + i] = Ny[i];
                }
                double nxx = A[0] * exx + A[1] * eyy + A[2] * gxy;
                double nyy = A[1] * exx + A[3] * eyy + A[4] * gxy;
                double nxy = A[2] * exx + A[4] * eyy + A[5] * gxy;
                if (!(s.flags & KG_NOB)) {
                    double kxx = 0, kyy = 0, kxy = 0;
                    for (int i = 0; i < 4; i++) {
                        const double *ui = q.ue + 6 * i;
                        kxx += Nx[i] * ui[4];
                        kyy -= Ny[i] * ui[3];
                        kxy += Ny[i] * ui[4] - Nx[i] * ui[3];
                    }
                    nxx = nxx + B[0] * kxx + B[1] * kyy + B[2] * kxy;
                    nyy = nyy + B[1] * kxx + B[3] * kyy + B[4] * kxy;
                    nxy = nxy + B[2] * kxx + B[4] * kyy + B[5] * kxy;
                }
                kg_point_vectors(s.g[g], detJ * nxx, detJ * nyy, detJ * nxy);
            }
        }
        __syncthreads();
        const int half = lane >> 4, pair = lane & 15, na = pair >> 2, nb = pair & 3;
        for (int round = 0; round < TILE / 8; round++) {
            kg_prefetch(a, se, oldv[warp], round * 8 + warp * 2, lane);
            const int el = round * 8 + warp * 2 + half;
            const KGElemS &s = se[el];
            if (s.flags & F_VALID) {
                double G = 0.;
#pragma unroll
                for (int g = 0; g < 4; g++) {
                    const double *o = s.g[g];
                    G += o[nb] * o[8 + 2 * na] + o[4 + nb] * o[9 + 2 * na];
                }
                double *st = stage[warp][half];
                if (s.flags & KG_FLATZ) {
                    st[(3 * na + 2) * KG_ROW + 3 * nb + 2] = s.rr[8] * G;
                } else {
#pragma unroll
                    for (int mm = 0; mm < 3; mm++)
#pragma unroll
                        for (int nn = 0; nn < 3; nn++)
                            st[(3 * na + mm) * KG_ROW + 3 * nb + nn] = s.rr[3 * mm + nn] * G;
                }
            }
            cp_async_wait_all();
            __syncwarp();
#pragma unroll
            for (int h = 0; h < 2; h++) {
                const KGElemS &t = se[round * 8 + warp * 2 + h];
                if (!(t.flags & F_VALID)) continue;
                const long long k0 = t.init_k;
                const double *st = stage[warp][h];
                if (t.flags & KG_FLATZ) {
                    // the 16 (w, w) values on lanes 0..15 (one FP64 addition per
                    // warp); the other values stay as they are (+= 0), and all
                    // 144 indices are written
                    if (lane < 16) {
                        const int i = (3 * (lane >> 2) + 2) * 12 + 3 * (lane & 3) + 2;
                        a.Kv[k0 + i] = oldv[warp][h][i] + st[(i / 12) * KG_ROW + i % 12];
                    }
                    if (a.Kr) kg_write_indices(a, t, k0, lane);
                    continue;
                }
                for (int i = lane; i < 144; i += 32) {
                    const int row = i / 12, col = i - row * 12;
                    a.Kv[k0 + i] = oldv[warp][h][i] + st[row * KG_ROW + col];
                    if (a.Kr) {
                        a.Kr[k0 + i] = t.c[row / 3] + row % 3;
                        a.Kc[k0 + i] = t.c[col / 3] + col % 3;
                    }
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
            // the caller's values first (all loads in flight), then the stores
            double old[15];
#pragma unroll
            for (int u = 0; u < 15; u++) {
                const int i = lane + 32 * u;
                old[u] = i < size ? a.Kv[k0 + i] : 0.;
            }
#pragma unroll
            for (int u = 0; u < 15; u++) {
                const int i = lane + 32 * u;
                if (i >= size) break;
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
                a.Kv[k0 + i] = old[u] + s.h[4 * na + nb] * s.G[6 * mm + nn];
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
// fint[c + .] += R (KC0e ue) (update_fint) and/or finte = KC0e ue in the
// element frame (update_probe_finte, quad4.pyx:1174-1201); either may be NULL.
//
// Elements whose element-frame coordinates relative to node 1 are in the
// float-float range (FI_FF) take the point pass (Jacobian, detJ, Cartesian
// derivatives) and the node-pair tensors H, H0 in float-float, as the KC0
// kernel does; the blocks, K ue and the rotation stay FP64.
constexpr int FI_FF = 64;  // element flag (above the F_* bits of ElemS)
union FSlot {
    double d;
    ff f;
};

__global__ void __launch_bounds__(NT, 3) quad4_fint_kernel(Q4Args a, const double *ue_in,
                                                           double *fint, int64_t nf, double *finte) {
    __shared__ ElemS se[TILE];
    __shared__ FSlot sgp[TILE][NPT][GPW];
    __shared__ ff sxyf[TILE][8];
    // N, dN/dxi, dN/deta of the 4 nodes at the 4 Gauss points and the centre
    __shared__ ff shf[NPT][3][4];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (tid < NPT * 12) {
        const int g = tid / 12, t = (tid / 4) % 3, i = tid & 3;
        double xi, eta;
        point_coords(g, xi, eta);
        const double sx = (i == 1 || i == 2) ? 1. : -1., sy = (i >= 2) ? 1. : -1.;
        shf[g][t][i] = ff_from_double(t == 0   ? 0.25 * (1 + sx * xi) * (1 + sy * eta)
                                      : t == 1 ? 0.25 * sx * (1 + sy * eta)
                                               : 0.25 * sy * (1 + sx * xi));
    }
    const int64_t ntiles = (a.E + TILE - 1) / TILE;
    for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int64_t e0 = tile * TILE;
        __syncthreads();
        if (tid < TILE) {
            const int64_t e = e0 + tid;
            if (e < a.E) {
                ElemS &s = se[tid];
                kc0_phase_a(a, e, s);
                for (int i = 0; i < 4; i++)
                    if (fint && s.c[i] + 6 > nf) {
                        raise_error(a.err, kErrBounds);
                        s.flags = 0;
                    }
                if (s.flags & F_VALID) {
                    bool ffok = true;
                    double d[8];
                    for (int i = 0; i < 4; i++) {
                        d[2 * i] = s.xy[2 * i] - s.xy[0];
                        d[2 * i + 1] = s.xy[2 * i + 1] - s.xy[1];
                        ffok &= ff_safe(d[2 * i]) && ff_safe(d[2 * i + 1]);
                    }
                    if (ffok) {
                        for (int i = 0; i < 8; i++) sxyf[tid][i] = ff_from_double(d[i]);
                        s.flags |= FI_FF;
                    }
                }
            } else {
                se[tid].flags = 0;
            }
        }
        __syncthreads();
        for (int it = tid; it < TILE * NPT; it += NT) {
            const int el = it / NPT, g = it % NPT;
            if (!(se[el].flags & F_VALID)) continue;
            FSlot *o = sgp[el][g];
            if (se[el].flags & FI_FF) {
                const ff *x = sxyf[el];
                ff J11 = ff_mul(x[0], shf[g][1][0]), J12 = ff_mul(x[1], shf[g][1][0]);
                ff J21 = ff_mul(x[0], shf[g][2][0]), J22 = ff_mul(x[1], shf[g][2][0]);
                for (int i = 1; i < 4; i++) {
                    J11 = ff_fma(x[2 * i], shf[g][1][i], J11);
                    J12 = ff_fma(x[2 * i + 1], shf[g][1][i], J12);
                    J21 = ff_fma(x[2 * i], shf[g][2][i], J21);
                    J22 = ff_fma(x[2 * i + 1], shf[g][2][i], J22);
                }
                const ff det = ff_fma(J11, J22, ff_neg(ff_mul(J12, J21)));
                const ff inv = ff_rcp(det);
                o[0].f = (g == 4) ? ff_scale(det, 4.f) : det;
                for (int i = 0; i < 4; i++) {
                    const ff dxi = shf[g][1][i], deta = shf[g][2][i];
                    o[5 + i].f = ff_mul(ff_fma(J22, dxi, ff_neg(ff_mul(J12, deta))), inv);
                    o[9 + i].f = ff_mul(ff_fma(J11, deta, ff_neg(ff_mul(J21, dxi))), inv);
                }
                continue;
            }
            double xi, eta, detJ, N[4], Nx[4], Ny[4];
            point_coords(g, xi, eta);
            quad_derivs(se[el].xy, xi, eta, detJ, N, Nx, Ny);
            o[0].d = (g == 4) ? 4. * detJ : detJ;
            for (int i = 0; i < 4; i++) {
                o[1 + i].d = N[i];
                o[5 + i].d = Nx[i];
                o[9 + i].d = Ny[i];
            }
        }
        __syncthreads();
        const int half = lane >> 4, pair = lane & 15, na = pair >> 2, nb = pair & 3;
        for (int round = 0; round < TILE / 8; round++) {
            const int el = round * 8 + warp * 2 + half;
            const int64_t e = e0 + el;
            const ElemS &s = se[el];
            double f[6] = {0., 0., 0., 0., 0., 0.}, fl[6] = {0., 0., 0., 0., 0., 0.};
            if (s.flags & F_VALID) {
                double H[3][3] = {}, H0[3][3], Hs[3][3];
                if (s.flags & FI_FF) {
                    ff h[3][3];
                    for (int p = 0; p < 3; p++)
                        for (int q = 0; q < 3; q++) h[p][q] = {0.f, 0.f};
                    for (int g = 0; g < 4; g++) {
                        const FSlot *o = sgp[el][g];
                        const ff w = o[0].f;
                        const ff va[3] = {ff_mul(w, shf[g][0][na]), ff_mul(w, o[5 + na].f), ff_mul(w, o[9 + na].f)};
                        const ff vb[3] = {shf[g][0][nb], o[5 + nb].f, o[9 + nb].f};
                        for (int p = 0; p < 3; p++)
                            for (int q = 0; q < 3; q++) h[p][q] = ff_fma(va[p], vb[q], h[p][q]);
                    }
                    const FSlot *o = sgp[el][4];
                    const ff w = o[0].f;
                    const ff va[3] = {ff_mul(w, shf[4][0][na]), ff_mul(w, o[5 + na].f), ff_mul(w, o[9 + na].f)};
                    const ff vb[3] = {shf[4][0][nb], o[5 + nb].f, o[9 + nb].f};
                    for (int p = 0; p < 3; p++)
                        for (int q = 0; q < 3; q++) {
                            H[p][q] = ff_to_double(h[p][q]);
                            H0[p][q] = ff_to_double(ff_mul(va[p], vb[q]));
                        }
                } else {
                    for (int g = 0; g < 4; g++) {
                        const FSlot *o = sgp[el][g];
                        const double w = o[0].d;
                        const double va[3] = {w * o[1 + na].d, w * o[5 + na].d, w * o[9 + na].d};
                        const double vb[3] = {o[1 + nb].d, o[5 + nb].d, o[9 + nb].d};
                        for (int p = 0; p < 3; p++)
                            for (int q = 0; q < 3; q++) H[p][q] += va[p] * vb[q];
                    }
                    const FSlot *o = sgp[el][4];
                    const double va[3] = {o[0].d * o[1 + na].d, o[0].d * o[5 + na].d, o[0].d * o[9 + na].d};
                    const double vb[3] = {o[1 + nb].d, o[5 + nb].d, o[9 + nb].d};
                    for (int p = 0; p < 3; p++)
                        for (int q = 0; q < 3; q++) H0[p][q] = va[p] * vb[q];
                }
                const bool thick = s.flags & F_THICK;
                for (int p = 0; p < 3; p++)
                    for (int q = 0; q < 3; q++) Hs[p][q] = thick ? H[p][q] : H0[p][q];
                double K[6][6];
                kc0_block(H, H0, Hs, s.abd, s.es, K);
                // fint uses local Ke and local ue (probe mode): rotate f only.
                const double *ueb = ue_in + 24 * e + 6 * nb;
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
                fl[i] += __shfl_xor_sync(0xffffffffu, fl[i], 1);
                fl[i] += __shfl_xor_sync(0xffffffffu, fl[i], 2);
            }
            if ((s.flags & F_VALID) && nb == 0) {
                if (fint)
                    for (int i = 0; i < 6; i++) atomicAdd(fint + s.c[na] + i, f[i]);
                if (finte)
                    for (int i = 0; i < 6; i++) finte[24 * e + 6 * na + i] = fl[i];
            }
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

extern "C" int fe3d_quad4_kg(int64_t E, const int64_t *cdof, const int64_t *init_k,
                             const double *x, int64_t nx, const double *xmat, int xmat_stride,
                             const double *u, int64_t nu, const double *R, const double *m,
                             const double *xe, const double *ue, const double *props,
                             int64_t nprops, const int32_t *pid, int64_t *Kr, int64_t *Kc,
                             double *Kv, int64_t nk, int *err, void *stream) {
    if (E < 0) return FE3D_ERR_ARG;
    if (E == 0) return FE3D_OK;
    if (!cdof || !init_k || !props || !Kv || (!Kr) != (!Kc) || nprops <= 0) return FE3D_ERR_ARG;
    if (x && !u) return FE3D_ERR_ARG;
    if (!x && (!R || !m || !xe || !ue)) return FE3D_ERR_ARG;
    if (xmat && xmat_stride != 0 && xmat_stride != 3) return FE3D_ERR_ARG;
    Q4Args a{E, cdof, init_k, x, nx, xmat, xmat_stride, R, m, xe, nullptr, props, nprops, pid,
             Kr, Kc, Kv, nk, 0, err};
    a.vec16 = Kr && ((uintptr_t)Kr & 15u) == 0 && ((uintptr_t)Kc & 15u) == 0;
    quad4_kg_kernel<<<grid_for(E, 4), NT, 0, as_stream(stream)>>>(a, u, nu, ue, nullptr, 0);
    FE3D_CHECK_LAUNCH();
    return FE3D_OK;
}

extern "C" int fe3d_quad4_kg_given_stress(int64_t E, const int64_t *cdof, const int64_t *init_k,
                                          const double *x, int64_t nx, const double *xmat, int xmat_stride,
                                          const double *R, const double *xe, const double *nstress,
                                          int nstress_stride, int64_t *Kr, int64_t *Kc, double *Kv, int64_t nk,
                                          int *err, void *stream) {
    if (E < 0) return FE3D_ERR_ARG;
    if (E == 0) return FE3D_OK;
    if (!cdof || !init_k || !nstress || !Kv || (!Kr) != (!Kc)) return FE3D_ERR_ARG;
    if (nstress_stride != 0 && nstress_stride != 3) return FE3D_ERR_ARG;
    if (!x && (!R || !xe)) return FE3D_ERR_ARG;
    if (xmat && xmat_stride != 0 && xmat_stride != 3) return FE3D_ERR_ARG;
    // the probe-mode m is not read: the given resultants need no material rotation
    Q4Args a{E, cdof, init_k, x, nx, xmat, xmat_stride, R, nullptr, xe, nullptr, nullptr, 0, nullptr,
             Kr, Kc, Kv, nk, 0, err};
    a.vec16 = Kr && ((uintptr_t)Kr & 15u) == 0 && ((uintptr_t)Kc & 15u) == 0;
    quad4_kg_kernel<<<grid_for(E, 4), NT, 0, as_stream(stream)>>>(a, nullptr, 0, nullptr, nstress,
                                                                  nstress_stride);
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
    // 4 CTAs per SM (16 warps): measured faster than the 5 that fit (2.50 vs 2.62 ms)
    quad4_m_kernel<<<grid_for(E, 4), NT, 0, as_stream(stream)>>>(a, mtype);
    FE3D_CHECK_LAUNCH();
    return FE3D_OK;
}

extern "C" int fe3d_quad4_fint(int64_t E, const int64_t *cdof, const double *R, const double *m,
                               const double *xe, const double *area, const double *ue,
                               const double *props, int64_t nprops, const int32_t *pid,
                               double *fint, int64_t nf, int *err, void *stream) {
    return fe3d_quad4_finte(E, cdof, R, m, xe, area, ue, props, nprops, pid, fint, nf, nullptr, err, stream);
}

extern "C" int fe3d_quad4_finte(int64_t E, const int64_t *cdof, const double *R, const double *m,
                                const double *xe, const double *area, const double *ue,
                                const double *props, int64_t nprops, const int32_t *pid,
                                double *fint, int64_t nf, double *finte, int *err, void *stream) {
    if (E < 0) return FE3D_ERR_ARG;
    if (E == 0) return FE3D_OK;
    if (!cdof || !R || !m || !xe || !area || !ue || !props || (!fint && !finte) || nprops <= 0)
        return FE3D_ERR_ARG;
    Q4Args a{E, cdof, nullptr, nullptr, 0, nullptr, 0, R, m, xe, area, props, nprops, pid,
             nullptr, nullptr, nullptr, INT64_MAX, 1, err};
    quad4_fint_kernel<<<grid_for(E, 3), NT, 0, as_stream(stream)>>>(a, ue, fint, nf, finte);
    FE3D_CHECK_LAUNCH();
    return FE3D_OK;
}
