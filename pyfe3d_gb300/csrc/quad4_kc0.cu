// Quad4 constitutive stiffness KC0: Quad4.update_KC0 (pyfe3d/quad4.pyx:1204-1313)
// with the local matrix of _update_probe_KC0ve (pyfe3d/quad4.pyx:755-1171).
//
// GB300 organisation.  An FP64 instruction occupies the FP64 pipe for the
// whole warp whatever the number of active lanes, and FP64 issues at 1/64 of
// the FP32 rate, so the kernel counts FP64 warp-instructions per element:
//
//   phase A   one thread per element (FP64): frame R (and material cosines),
//             flatness test, constitutive matrices in the evaluation frame,
//             nodal coordinates relative to node 1, thin/thick flag.
//   phase A2  one thread per (element, point) at the 4 Gauss points and the
//             centre: Jacobian and Cartesian shape derivatives, computed in
//             float-float (FP32 pipe) for flat elements.
//   phase B   16 lanes per element, one per node pair (a, b): the tensor
//             H^pq_ab = sum_points w detJ D^p N_a D^q N_b (p, q in
//             {N, d/dx, d/dy}) accumulated in float-float and converted to
//             double with integer operations, then the 6x6 block
//             K_ab = sum_pq C^pq H^pq in FP64 added onto the staged values
//             in row groups (no lane holds a whole block: for isotropic
//             sections -- rotation-invariant A, D, E and B = 0 -- the 18
//             non-zeros in two groups, otherwise three rows at a time);
//   write-out each warp streams its two staged elements (576 values each)
//             with the coalesced += read-modify-write and the indices.
//
// CTAs of 8 warps (FE3D_KC0_WARPS), two per SM (FE3D_KC0_MINB, 128
// registers): 16 warps per SM; phase A runs on warp 0 while the other warps
// write out their last round of the previous tile.
//
// Flat elements whose normal is +Z (r13 = r23 = r31 = r32 = 0) are evaluated
// in the global frame with in-plane rotated constitutive matrices (no
// rotation at all for isotropic sections), which equals R Ke R^T without the
// transform.  Other elements, and the probe mode that reads the element
// state, are evaluated in FP64 in the element frame and rotated per block.
#include "fe3d_internal.h"
#include "ff.cuh"
#include "quad4_common.cuh"

namespace fe3d {
namespace {

#ifndef FE3D_KC0_TILE
#define FE3D_KC0_TILE 32
#endif
#ifndef FE3D_KC0_WARPS
#define FE3D_KC0_WARPS 8
#endif
constexpr int KT = FE3D_KC0_TILE;  // elements per CTA iteration (phase A: one lane each)
constexpr int KNT = 32 * FE3D_KC0_WARPS;  // threads per CTA
constexpr int KRND = 2 * FE3D_KC0_WARPS;  // elements per phase-B round (two per warp)
static_assert(KT % KRND == 0 && KT <= 32, "a tile is whole rounds of elements, phase A one warp");
constexpr int KPTS = 5;   // 4 Gauss points + centre
constexpr int KSLOT = 9;  // per point: w detJ, Nx[4], Ny[4] (N is the same for every element)

enum : int { KF_VALID = 1, KF_THICK = 2, KF_FP64 = 4, KF_ISO = 8 };

union Slot {
    double d;
    ff f;
};

struct __align__(16) KElem {
    double R[9];
    double abd[36];
    double es[3];
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
    double stage[KNT / 32][2][24 * KROW];
};

// shape-function values and natural derivatives at the 5 points, float-float:
// [point][0: N, 1: dN/dxi, 2: dN/deta][node]
__constant__ ff c_shape[KPTS][3][4];

// Element set-up shared by the triplet and the CSR kernels: frame,
// flatness, constitutive data and nodal coordinates of element e with DOF
// offsets c[4]; ok carries the caller's own checks.
__device__ void kc0_elem_setup(const Q4Args &a, int64_t e, const long long *c, bool ok, KElem &s) {
#pragma unroll
    for (int i = 0; i < 4; i++)
        if (c[i] < 0 || (a.x && c[i] / 2 + 3 > a.nx)) ok = false;
    const int64_t p = a.pid ? (int64_t)a.pid[e] : e;
    if (p < 0 || p >= a.nprops) ok = false;
    if (!ok) {
        raise_error(a.err, kErrBounds);
        return;
    }
    const double *P = a.props + (int64_t)SP_STRIDE * p;
    double R[9], m[4] = {1., 0., 0., 1.}, xy[8], ar;
    bool fp64 = true, iso = false;
    if (a.x) {
        const double *pp[4] = {a.x + c[0] / 2, a.x + c[1] / 2, a.x + c[2] / 2, a.x + c[3] / 2};
        q4_rotation(pp[0], pp[1], pp[2], pp[3], a.xmat ? a.xmat + (int64_t)a.xmat_stride * e : nullptr,
                    R, m);
        if (is_flat(R)) {
            bool safe = true;
#pragma unroll
            for (int i = 0; i < 4; i++) {
                xy[2 * i] = pp[i][0] - pp[0][0];
                xy[2 * i + 1] = pp[i][1] - pp[0][1];
                safe &= ff_safe(xy[2 * i]) && ff_safe(xy[2 * i + 1]);
            }
            fp64 = !safe;
        }
        if (!fp64) {
            const double E44 = P[SP_E44] * P[SP_SCF23];
            const double E45 = P[SP_E45] * 0.5 * (P[SP_SCF13] + P[SP_SCF23]);
            const double E55 = P[SP_E55] * P[SP_SCF13];
            iso = iso_section(P, E44, E45, E55);
            if (iso) {
                // rotation-invariant section: the material values are the
                // global-frame values (A11 A12 A66, D11 D12 D66, E44)
                s.abd[0] = P[SP_A11];
                s.abd[1] = P[SP_A12];
                s.abd[2] = P[SP_A66];
                s.abd[3] = P[SP_D11];
                s.abd[4] = P[SP_D12];
                s.abd[5] = P[SP_D66];
                s.es[0] = E44;
                s.es[1] = 0.;
                s.es[2] = E55;
            } else {
                q4_constitutive(P, m, R, true, s.abd, s.es);
            }
        } else {
#pragma unroll
            for (int i = 0; i < 4; i++) {
                double q[3];
                to_local(R, pp[i], q);
                xy[2 * i] = q[0];
                xy[2 * i + 1] = q[1];
            }
            q4_constitutive(P, m, R, false, s.abd, s.es);
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
        q4_constitutive(P, m, R, false, s.abd, s.es);
        ar = a.area[e];
    }
#pragma unroll
    for (int i = 0; i < 9; i++) s.R[i] = R[i];
    if (fp64) {
#pragma unroll
        for (int i = 0; i < 8; i++) s.xy[i].d = xy[i];
    } else {
#pragma unroll
        for (int i = 0; i < 8; i++) s.xy[i].f = ff_from_double(xy[i]);
    }
    // h / sqrt(area) >= 1 as the reference evaluates it; the division only
    // decides when h < sqrt(area) (h >= sqrt(area) implies the rounded
    // quotient is >= 1)
    const double sq = sqrt(ar);
    const bool thick = P[SP_H] >= sq || P[SP_H] / sq >= 1.;
    s.flags = KF_VALID | (thick ? KF_THICK : 0) | (fp64 ? KF_FP64 : 0) | (iso ? KF_ISO : 0);
}

__device__ void kc0_phase_a2(const Q4Args &a, int64_t e, KElem &s) {
    s.flags = 0;
    long long c[4];
#pragma unroll
    for (int i = 0; i < 4; i++) {
        c[i] = a.cdof[4 * e + i];
        s.c[i] = c[i];
    }
    const long long k0 = a.init_k[e];
    s.init_k = k0;
    kc0_elem_setup(a, e, c, k0 >= 0 && k0 + 576 <= a.nk, s);
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
        o[1 + i].f = ff_mul(ff_fma(J22, dxi, ff_neg(ff_mul(J12, deta))), inv);
        o[5 + i].f = ff_mul(ff_fma(J11, deta, ff_neg(ff_mul(J21, dxi))), inv);
    }
}

__device__ __forceinline__ ff ffz() { return {0.f, 0.f}; }


// Streams one staged element (24 x KROW doubles: current values + K) to the
// caller's arrays at k0: values and, unless values_only, the indices of the
// element's DOF offsets c[4].
__device__ __forceinline__ void write_staged(const Q4Args &a, const double *sv, long long k0, const long long *c,
                                             int lane) {
    double *kv = a.Kv + k0;
    if (a.vec16 && !(k0 & 1)) {
        // 16-byte stores: slots (2 lane + 64 j, + 1) share the row and the
        // column node
        long long *kr = (long long *)a.Kr + k0, *kc = (long long *)a.Kc + k0;
        int row = lane / 12, col = 2 * lane - 24 * row;
#pragma unroll 3
        for (int j = 0; j < 9; j++) {
            const int i = 2 * lane + 64 * j;
            *reinterpret_cast<double2 *>(kv + i) = *reinterpret_cast<const double2 *>(sv + row * KROW + col);
            if (!a.values_only) {
                const int ra = row / 6, cb = col / 6;
                const long long r = c[ra] + (row - 6 * ra), c0 = c[cb] + (col - 6 * cb);
                *reinterpret_cast<longlong2 *>(kr + i) = make_longlong2(r, r);
                *reinterpret_cast<longlong2 *>(kc + i) = make_longlong2(c0, c0 + 1);
            }
            col += 16;
            row += 2;
            if (col >= 24) {
                col -= 24;
                row += 1;
            }
        }
        return;
    }
#pragma unroll 6
    for (int i = lane; i < 576; i += 32) {
        const int row = i / 24, col = i - row * 24;
        kv[i] = sv[row * KROW + col];
    }
    if (!a.values_only) {
        long long *kr = (long long *)a.Kr + k0, *kc = (long long *)a.Kc + k0;
#pragma unroll 6
        for (int i = lane; i < 576; i += 32) {
            const int row = i / 24, col = i - row * 24;
            kr[i] = c[row / 6] + row % 6;
            kc[i] = c[col / 6] + col % 6;
        }
    }
}

// The element data of a staged element whose write-out is deferred, kept in
// the stage's padding columns (24, 25), which the values never use.
__device__ __forceinline__ long long *stage_meta(double *sv, int i) {
    return reinterpret_cast<long long *>(sv + (i >> 1) * KROW + 24 + (i & 1));
}

// Writes out a warp's two deferred elements.
__device__ __forceinline__ void flush_deferred(const Q4Args &a, double (*stage)[24 * KROW], int lane) {
#pragma unroll
    for (int hh = 0; hh < 2; hh++) {
        double *sv = stage[hh];
        if (!(*stage_meta(sv, 0) & KF_VALID)) continue;
        long long c[4];
#pragma unroll
        for (int i = 0; i < 4; i++) c[i] = *stage_meta(sv, 2 + i);
        write_staged(a, sv, *stage_meta(sv, 1), c, lane);
    }
    __syncwarp();
}

// N_i at point g in FP64, the expression of quad_derivs (elements evaluated
// in FP64 only).
__device__ __forceinline__ double shape_n(int g, int i) {
    double xi, eta;
    point_coords(g, xi, eta);
    const double sx = (i == 1 || i == 2) ? 1. : -1., sy = (i >= 2) ? 1. : -1.;
    return 0.25 * (1 + sx * xi) * (1 + sy * eta);
}

// The 4-point tensor H^pq_ab = sum_g w detJ D^p N_a D^q N_b (p, q in
// {N, d/dx, d/dy}) of node pair (na, nb) of element slot el: accumulated in
// float-float and rounded to double, or in FP64 for elements evaluated in
// FP64 (FF = false).
template <bool FF>
__device__ __forceinline__ void pair_h(const KSmem &S, int el, int na, int nb, double H[3][3]) {
    if (FF) {
        ff h[3][3];
#pragma unroll
        for (int p = 0; p < 3; p++)
#pragma unroll
            for (int q = 0; q < 3; q++) h[p][q] = ffz();
#pragma unroll
        for (int g = 0; g < 4; g++) {
            const Slot *o = S.gp[el][g];
            const ff w = o[0].f;
            const ff va[3] = {ff_mul(w, S.shape[g][0][na]), ff_mul(w, o[1 + na].f), ff_mul(w, o[5 + na].f)};
            const ff vb[3] = {S.shape[g][0][nb], o[1 + nb].f, o[5 + nb].f};
#pragma unroll
            for (int p = 0; p < 3; p++)
#pragma unroll
                for (int q = 0; q < 3; q++) h[p][q] = ff_fma(va[p], vb[q], h[p][q]);
        }
#pragma unroll
        for (int p = 0; p < 3; p++)
#pragma unroll
            for (int q = 0; q < 3; q++) H[p][q] = ff_to_double(h[p][q]);
    } else {
#pragma unroll
        for (int p = 0; p < 3; p++)
#pragma unroll
            for (int q = 0; q < 3; q++) H[p][q] = 0.;
#pragma unroll
        for (int g = 0; g < 4; g++) {
            const Slot *o = S.gp[el][g];
            const double w = o[0].d;
            const double va[3] = {w * shape_n(g, na), w * o[1 + na].d, w * o[5 + na].d};
            const double vb[3] = {shape_n(g, nb), o[1 + nb].d, o[5 + nb].d};
#pragma unroll
            for (int p = 0; p < 3; p++)
#pragma unroll
                for (int q = 0; q < 3; q++) H[p][q] += va[p] * vb[q];
        }
    }
}

// The centre-point (one-point rule) tensor H0^pq_ab, entry by entry.
template <bool FF>
struct CentreH;
template <>
struct CentreH<true> {
    ff a[3], b[3];
    __device__ __forceinline__ CentreH(const KSmem &S, int el, int na, int nb) {
        const Slot *o = S.gp[el][4];
        const ff w = o[0].f;
        a[0] = ff_mul(w, S.shape[4][0][na]);
        a[1] = ff_mul(w, o[1 + na].f);
        a[2] = ff_mul(w, o[5 + na].f);
        b[0] = S.shape[4][0][nb];
        b[1] = o[1 + nb].f;
        b[2] = o[5 + nb].f;
    }
    __device__ __forceinline__ double operator()(int p, int q) const { return ff_to_double(ff_mul(a[p], b[q])); }
};
template <>
struct CentreH<false> {
    double a[3], b[3];
    __device__ __forceinline__ CentreH(const KSmem &S, int el, int na, int nb) {
        const Slot *o = S.gp[el][4];
        const double w = o[0].d;
        a[0] = w * shape_n(4, na);
        a[1] = w * o[1 + na].d;
        a[2] = w * o[5 + na].d;
        b[0] = shape_n(4, nb);
        b[1] = o[1 + nb].d;
        b[2] = o[5 + nb].d;
    }
    __device__ __forceinline__ double operator()(int p, int q) const { return a[p] * b[q]; }
};

__device__ __forceinline__ void add2(double *st, int na, int nb, int m, int n, double x, double y) {
    double2 *q = reinterpret_cast<double2 *>(st + (6 * na + m) * KROW + 6 * nb + n);
    double2 o = *q;
    o.x += x;
    o.y += y;
    *q = o;
}

// Adds the 6x6 block K_ab of a flat isotropic element in the global frame
// (B = 0, E45 = 0; abd holds A11 A12 A66 D11 D12 D66, es E44 0 E55) onto the
// staged values: the non-zero terms of kc0_block for A11 = A22,
// A16 = A26 = 0 (same for D), with the unit drilling weight folded into the
// A66 terms.  The block couples (u, v, rz) and (w, rx, ry) only: the slot
// pairs that hold exact zeros (cols 2-3 of rows u, v, rz; cols 0-1 of rows
// w, rx, ry) are left as they are, and each group is added as soon as it is
// formed.
__device__ __forceinline__ void pair_add_iso(const KElem &s, const double H[3][3], const CentreH<true> &h0,
                                             double *st, int na, int nb) {
    const double *abd = s.abd;
    const double A11 = abd[0], A12 = abd[1], A66 = abd[2];
    const double am = A66 + 0.25, an = A66 - 0.25;
    // membrane and drilling: rows and columns u, v, rz
    add2(st, na, nb, 0, 0, A11 * H[1][1] + am * H[2][2], A12 * H[1][2] + an * H[2][1]);
    add2(st, na, nb, 0, 4, 0., 0.5 * H[2][0]);
    add2(st, na, nb, 1, 0, an * H[1][2] + A12 * H[2][1], am * H[1][1] + A11 * H[2][2]);
    add2(st, na, nb, 1, 4, 0., -0.5 * H[1][0]);
    add2(st, na, nb, 5, 0, 0.5 * H[0][2], -0.5 * H[0][1]);
    add2(st, na, nb, 5, 4, 0., H[0][0]);
    // bending and transverse shear: rows and columns w, rx, ry
    const double D11 = abd[3], D12 = abd[4], D66 = abd[5];
    const double E44 = s.es[0], E55 = s.es[2];
    const bool thick = s.flags & KF_THICK;
    const double c00 = h0(0, 0);
    const double hs22 = thick ? H[2][2] : h0(2, 2), hs11 = thick ? H[1][1] : h0(1, 1);
    add2(st, na, nb, 2, 2, E44 * hs22 + E55 * hs11, -E44 * h0(2, 0));
    add2(st, na, nb, 2, 4, E55 * h0(1, 0), 0.);
    add2(st, na, nb, 3, 2, -E44 * h0(0, 2), D66 * H[1][1] + D11 * H[2][2] + E44 * c00);
    add2(st, na, nb, 3, 4, -(D66 * H[1][2] + D12 * H[2][1]), 0.);
    add2(st, na, nb, 4, 2, E55 * h0(0, 1), -(D12 * H[1][2] + D66 * H[2][1]));
    add2(st, na, nb, 4, 4, D11 * H[1][1] + D66 * H[2][2] + E55 * c00, 0.);
}

// Adds the general 6x6 block K_ab (kc0_block; rotated to the global frame
// for elements evaluated in the element frame) onto the staged values,
// three rows at a time (a row block of T K T^T needs only the same row
// block of K).
template <bool FF>
__device__ __forceinline__ void pair_add_general(const KElem &s, const double H[3][3], const CentreH<FF> &h0,
                                                 double *st, int na, int nb) {
    const bool thick = s.flags & KF_THICK;
    double H0[3][3], Hs[3][3];
#pragma unroll
    for (int p = 0; p < 3; p++)
#pragma unroll
        for (int q = 0; q < 3; q++) {
            H0[p][q] = h0(p, q);
            Hs[p][q] = thick ? H[p][q] : H0[p][q];
        }
#pragma unroll
    for (int hb = 0; hb < 2; hb++) {
        double K[6][6];
        kc0_block(H, H0, Hs, s.abd, s.es, K);
        if (!FF) rotate_block(s.R, K);
#pragma unroll
        for (int m = 3 * hb; m < 3 * hb + 3; m++)
#pragma unroll
            for (int n = 0; n < 6; n += 2) add2(st, na, nb, m, n, K[m][n], K[m][n + 1]);
    }
}

// Phase B work of one lane: the node-pair tensor (before the caller's
// values are known to be staged) and the block added onto them (after).
__device__ __forceinline__ void pair_tensor(const KSmem &S, int el, int na, int nb, double H[3][3]) {
    const KElem &s = S.el[el];
    if (!(s.flags & KF_VALID)) return;
    if (s.flags & KF_FP64) pair_h<false>(S, el, na, nb, H);
    else pair_h<true>(S, el, na, nb, H);
}

__device__ __forceinline__ void pair_add(const KSmem &S, int el, int na, int nb, const double H[3][3], double *st) {
    const KElem &s = S.el[el];
    if (!(s.flags & KF_VALID)) return;
    if (s.flags & KF_FP64) {
        const CentreH<false> h0(S, el, na, nb);
        pair_add_general<false>(s, H, h0, st, na, nb);
    } else {
        const CentreH<true> h0(S, el, na, nb);
        if (s.flags & KF_ISO) pair_add_iso(s, H, h0, st, na, nb);
        else pair_add_general<true>(s, H, h0, st, na, nb);
    }
}

// Phase B of one round for a warp: the elements el0 (lanes 0-15) and el0 + 1
// (lanes 16-31), one lane per node pair: the caller's current values are
// prefetched into stage[0..1] with cp.async while the 6x6 blocks are
// computed, then the blocks are added onto them (ready for the write-out).
__device__ __forceinline__ void kc0_round(const Q4Args &a, KSmem &S, int el0, double (*stage)[24 * KROW],
                                          int lane) {
    const int half = lane >> 4, pair = lane & 15;
    const int na = pair >> 2, nb = pair & 3;
    const int el = el0 + half;
    double *st = stage[half];
    // prefetch the two elements' current values into the stage
#pragma unroll
    for (int hh = 0; hh < 2; hh++) {
        const KElem &t = S.el[el0 + hh];
        if (!(t.flags & KF_VALID)) continue;
        const double *kv = a.Kv + t.init_k;
        double *sv = stage[hh];
        if (a.vec16 && !(t.init_k & 1)) {
            // 16-byte pieces: slots 2 lane + 64 j, j = 0..8
            int row = lane / 12, col = 2 * lane - 24 * row;
#pragma unroll 3
            for (int j = 0; j < 9; j++) {
                cp_async16(sv + row * KROW + col, kv + 2 * lane + 64 * j);
                col += 16;
                row += 2;
                if (col >= 24) {
                    col -= 24;
                    row += 1;
                }
            }
        } else {
#pragma unroll 6
            for (int i = lane; i < 576; i += 32) {
                const int row = i / 24, col = i - row * 24;
                cp_async8(sv + row * KROW + col, kv + i);
            }
        }
    }
    cp_async_commit();
    double H[3][3];
    pair_tensor(S, el, na, nb, H);
    // all lanes' prefetches of both staged elements have landed
    cp_async_wait_all();
    __syncwarp();
    pair_add(S, el, na, nb, H, st);
    __syncwarp();
}

// Phase A2 for element slot el at point g: w detJ and the shape functions
// with their Cartesian derivatives (float-float for flat elements, FP64
// otherwise).
__device__ __forceinline__ void kc0_point(KSmem &S, int el, int g) {
    const KElem &s = S.el[el];
    if (!(s.flags & KF_VALID)) return;
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
            o[1 + i].d = Nx[i];
            o[5 + i].d = Ny[i];
        }
    } else {
        point_ff(s, S.shape, g, o);
    }
}

// The per-CTA copy of the float-float shape-function table.
__device__ __forceinline__ void kc0_tables(KSmem &S, int tid) {
    for (int i = tid; i < KPTS * 12; i += KNT) (&S.shape[0][0][0])[i] = (&c_shape[0][0][0])[i];
}

#ifndef FE3D_KC0_MINB
#define FE3D_KC0_MINB 2
#endif
__global__ void __launch_bounds__(KNT, FE3D_KC0_MINB) quad4_kc0_ff_kernel(Q4Args a) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    KSmem &S = *reinterpret_cast<KSmem *>(smem_raw);
    const int tid = threadIdx.x;
    kc0_tables(S, tid);
    const int64_t ntiles = (a.E + KT - 1) / KT;
    const int lane = tid & 31, warp = tid >> 5;
    // warps other than 0 defer the write-out of their last round of a tile
    // and do it while warp 0 runs phase A of the next tile
    bool pending = false;
    for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int64_t e0 = tile * KT;
        __syncthreads();
        if (tid < KT) {
            const int64_t e = e0 + tid;
            if (e < a.E) kc0_phase_a2(a, e, S.el[tid]);
            else S.el[tid].flags = 0;
        } else if (pending) {
            flush_deferred(a, S.stage[warp], lane);
            pending = false;
        }
        __syncthreads();
        // phase A2: integration points
        for (int it = tid; it < KT * KPTS; it += KNT) {
            const int el = it / KPTS, g = it - el * KPTS;
            kc0_point(S, el, g);
        }
        __syncthreads();
        // phase B: each warp owns 2 elements per round, one lane per node
        // pair; blocks are staged and then streamed out coalesced
        for (int round = 0; round < KT / KRND; round++) {
            kc0_round(a, S, round * KRND + warp * 2, S.stage[warp], lane);
            const bool defer = round == KT / KRND - 1 && warp != 0;
#pragma unroll
            for (int hh = 0; hh < 2; hh++) {
                const KElem &t = S.el[round * KRND + warp * 2 + hh];
                if (defer) {
                    double *sv = S.stage[warp][hh];
                    if (lane < 6) *stage_meta(sv, lane) = lane == 0 ? (long long)t.flags
                                                          : lane == 1 ? t.init_k : t.c[lane - 2];
                    continue;
                }
                if (!(t.flags & KF_VALID)) continue;
                write_staged(a, S.stage[warp][hh], t.init_k, t.c, lane);
            }
            pending = defer;
            __syncwarp();
        }
    }
    if (pending) flush_deferred(a, S.stage[warp], lane);
}


// ------------------------------------------------------ CSR write-out mode
// The same element computation with the blocks sent straight to the reduced
// CSR values through an element -> CSR scatter map (fused.cu): one launch
// per element colour (no two elements of a colour share a node), so the
// read-add-write of the CSR entries needs no atomics and sums every entry
// in a fixed order.  The node-pair blocks an element assigns (it is their
// first contributor) are stored without reading.

struct CsrArgs {
    const int32_t *order;  // the colour's elements
    int64_t cnt;
    const int32_t *node;   // [E, 4] node indices
    const int32_t *boff;   // [E, 16] offsets of node j's columns in node i's rows
    const uint32_t *first; // [E] assign bits
    const fe3d_noderow *nr;
    int64_t nnodes;
    double *vals;
    int64_t nnz;
    int assign;
    int atomic;  // one launch over all elements, blocks added with atomics (order unspecified)
};

// Per element of the tile: row length | free mask << 16 of its nodes, the
// block offsets and the assign bits (the nodes' row starts go to KElem.c).
struct __align__(8) CsrElem {
    int Lf[4];
    short boff[16];
    unsigned first;
    int pad;
};

struct KSmemCsr {
    KSmem s;
    CsrElem cm[KT];
};

// FE3D_KC0_MINB CTAs per SM must fit the SM's 228 KB of shared memory
// (1 KB of it reserved per CTA)
static_assert(FE3D_KC0_MINB * (sizeof(KSmem) + 1024) <= 228 * 1024, "triplet kernel: shared memory per SM");
static_assert(FE3D_KC0_MINB * (sizeof(KSmemCsr) + 1024) <= 228 * 1024, "CSR kernel: shared memory per SM");

// A staged element's scatter data in the stage's padding columns (24, 25):
// slots 0-23 the CSR position of each row's first entry (-1: fixed DOF),
// 24-27 the 16 block offsets (int16), 28-30 the rank of each column within
// its node (int8, -1: fixed DOF), 31 flags | assign bits << 32.
__device__ __forceinline__ long long *csr_meta(double *sv, int i) {
    return reinterpret_cast<long long *>(sv + (i >> 1) * KROW + 24 + (i & 1));
}
__device__ __forceinline__ const long long *csr_meta(const double *sv, int i) {
    return reinterpret_cast<const long long *>(sv + (i >> 1) * KROW + 24 + (i & 1));
}
__device__ __forceinline__ int csr_boff(const double *sv, int k) {
    return reinterpret_cast<const short *>(csr_meta(sv, 24 + (k >> 2)))[k & 3];
}
__device__ __forceinline__ int csr_colrank(const double *sv, int col) {
    return reinterpret_cast<const signed char *>(csr_meta(sv, 28 + (col >> 3)))[col & 7];
}

__device__ void kc0_phase_a_csr(const Q4Args &a, const CsrArgs &m, int64_t t, KElem &s, CsrElem &q) {
    s.flags = 0;
    const int64_t e = m.order ? (int64_t)m.order[t] : t;
    int32_t nd[4];
    bool ok = e >= 0 && e < a.E;
    if (ok) {
#pragma unroll
        for (int i = 0; i < 4; i++) {
            nd[i] = m.node[4 * e + i];
            ok &= nd[i] >= 0 && nd[i] < m.nnodes;
        }
    }
    if (!ok) {
        raise_error(a.err, kErrBounds);
        return;
    }
    long long c[4];
#pragma unroll
    for (int i = 0; i < 4; i++) {
        c[i] = 6LL * nd[i];
        const fe3d_noderow r = m.nr[nd[i]];
        s.c[i] = r.rs;
        q.Lf[i] = r.L | (r.fm << 16);
    }
    const int4 *bo = reinterpret_cast<const int4 *>(m.boff + 16 * e);
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const int4 v = bo[k];
        q.boff[4 * k] = (short)v.x;
        q.boff[4 * k + 1] = (short)v.y;
        q.boff[4 * k + 2] = (short)v.z;
        q.boff[4 * k + 3] = (short)v.w;
    }
    q.first = m.assign ? m.first[e] : 0u;
    s.init_k = 0;
    kc0_elem_setup(a, e, c, true, s);
}

__device__ __forceinline__ void csr_meta_build(const KElem &t, const CsrElem &q, double *sv, int lane) {
    if (lane < 24) {
        const int a = lane / 6, m = lane - 6 * a;
        const int Lf = q.Lf[a], fm = Lf >> 16, L = Lf & 0xffff;
        const bool fr = (fm >> m) & 1;
        const int rank = __popc(fm & ((1 << m) - 1));
        *csr_meta(sv, lane) = fr ? t.c[a] + (long long)rank * L : -1LL;
        reinterpret_cast<signed char *>(csr_meta(sv, 28 + (lane >> 3)))[lane & 7] =
            fr ? (signed char)rank : (signed char)-1;
    } else if (lane < 28) {
        *csr_meta(sv, lane) = reinterpret_cast<const long long *>(q.boff)[lane - 24];
    } else if (lane == 28) {
        *csr_meta(sv, 31) = (long long)(unsigned)t.flags | ((long long)q.first << 32);
    }
}

// The slots of a staged element that move: free row and column, and not an
// exact isotropic zero of a block that is added (assigned blocks store all).
// Lane l < 24 takes column l of the element for all 24 rows, so the column's
// rank, its block offsets and assign bits are hoisted out of the row loop;
// every row is one warp-wide access of its 4 runs of 6 entries.
template <class F>
__device__ __forceinline__ void csr_slots(const double *sv, int lane, F &&f) {
    if (lane >= 24) return;
    const long long fl = *csr_meta(sv, 31);
    const int flags = (int)(fl & 0xffffffffLL);
    if (!(flags & KF_VALID)) return;
    const int cr = csr_colrank(sv, lane);
    if (cr < 0) return;  // fixed column
    const unsigned first = (unsigned)((unsigned long long)fl >> 32);
    const int b = lane / 6, n = lane - 6 * b;
    const bool iso = flags & KF_ISO;
    const bool z_mid = iso && n < 2, z_out = iso && (n == 2 || n == 3);
    long long colpart[4];
    bool asg[4];
#pragma unroll
    for (int a = 0; a < 4; a++) {
        colpart[a] = csr_boff(sv, 4 * a + b) + cr;
        asg[a] = (first >> (4 * a + b)) & 1;
    }
#pragma unroll
    for (int row = 0; row < 24; row++) {
        const int a = row / 6, m = row - 6 * (row / 6);
        const long long rb = *csr_meta(sv, row);
        if (rb < 0) continue;
        const bool zero = (m >= 2 && m <= 4) ? z_mid : z_out;
        if (!asg[a] && zero) continue;
        f(row * KROW + lane, rb + colpart[a], asg[a]);
    }
}

__device__ __forceinline__ void csr_prefetch(const CsrArgs &m, double *sv, int lane, int *err) {
    csr_slots(sv, lane, [&](int si, long long pos, bool asg) {
        if (asg || m.atomic) {
            sv[si] = 0.;
        } else if (pos >= 0 && pos < m.nnz) {
            cp_async8(sv + si, m.vals + pos);
        } else {
            raise_error(err, kErrBounds);
        }
    });
}

__device__ __forceinline__ void csr_write(const CsrArgs &m, const double *sv, int lane) {
    csr_slots(sv, lane, [&](int si, long long pos, bool) {
        if (pos >= 0 && pos < m.nnz) {
            if (m.atomic) atomicAdd(m.vals + pos, sv[si]);
            else m.vals[pos] = sv[si];
        }
    });
}

__device__ __forceinline__ void kc0_round_csr(const Q4Args &a, const CsrArgs &m, KSmem &S, const CsrElem *cm,
                                              int el0, double (*stage)[24 * KROW], int lane) {
    const int half = lane >> 4, pair = lane & 15;
    const int na = pair >> 2, nb = pair & 3;
    const int el = el0 + half;
    double *st = stage[half];
#pragma unroll
    for (int hh = 0; hh < 2; hh++) csr_meta_build(S.el[el0 + hh], cm[el0 + hh], stage[hh], lane);
    __syncwarp();
#pragma unroll
    for (int hh = 0; hh < 2; hh++) csr_prefetch(m, stage[hh], lane, a.err);
    cp_async_commit();
    double H[3][3];
    pair_tensor(S, el, na, nb, H);
    cp_async_wait_all();
    __syncwarp();
    pair_add(S, el, na, nb, H, st);
    __syncwarp();
}

__global__ void __launch_bounds__(KNT, FE3D_KC0_MINB) quad4_kc0_csr_kernel(Q4Args a, CsrArgs m) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    KSmemCsr &SC = *reinterpret_cast<KSmemCsr *>(smem_raw);
    KSmem &S = SC.s;
    const int tid = threadIdx.x;
    kc0_tables(S, tid);
    const int64_t ntiles = (m.cnt + KT - 1) / KT;
    const int lane = tid & 31, warp = tid >> 5;
    bool pending = false;
    for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int64_t t0 = tile * KT;
        __syncthreads();
        if (tid < KT) {
            const int64_t t = t0 + tid;
            if (t < m.cnt) kc0_phase_a_csr(a, m, t, S.el[tid], SC.cm[tid]);
            else S.el[tid].flags = 0;
        } else if (pending) {
#pragma unroll
            for (int hh = 0; hh < 2; hh++) csr_write(m, S.stage[warp][hh], lane);
            __syncwarp();
            pending = false;
        }
        __syncthreads();
        for (int it = tid; it < KT * KPTS; it += KNT) {
            const int el = it / KPTS, g = it - el * KPTS;
            kc0_point(S, el, g);
        }
        __syncthreads();
        for (int round = 0; round < KT / KRND; round++) {
            kc0_round_csr(a, m, S, SC.cm, round * KRND + warp * 2, S.stage[warp], lane);
            // warps other than 0 write their last round while warp 0 runs the next phase A
            const bool defer = round == KT / KRND - 1 && warp != 0;
            if (!defer) {
#pragma unroll
                for (int hh = 0; hh < 2; hh++) csr_write(m, S.stage[warp][hh], lane);
            }
            pending = defer;
            __syncwarp();
        }
    }
    if (pending) {
#pragma unroll
        for (int hh = 0; hh < 2; hh++) csr_write(m, S.stage[warp][hh], lane);
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
                             (int)sizeof(KSmem)) != cudaSuccess ||
        cudaFuncSetAttribute(quad4_kc0_csr_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)sizeof(KSmemCsr)) != cudaSuccess)
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
    // 16-byte write-out for elements with an even init_k when the output
    // arrays are 16-byte aligned
    const auto al16 = [](const void *q) { return ((uintptr_t)q & 15u) == 0; };
    a.vec16 = al16(Kv) && (values_only || (al16(Kr) && al16(Kc)));
    const int64_t tiles = (E + KT - 1) / KT;
    const int64_t cap = (int64_t)kSMs * FE3D_KC0_MINB;
    const int grid = (int)(tiles < cap ? tiles : cap);
    quad4_kc0_ff_kernel<<<grid, KNT, sizeof(KSmem), as_stream(stream)>>>(a);
    FE3D_CHECK_LAUNCH();
    return FE3D_OK;
}

extern "C" int fe3d_quad4_kc0_csr(const fe3d_fmap *fm, int g, const double *x, int64_t nx, const double *xmat,
                                  int xmat_stride, const double *props, int64_t nprops, const int32_t *pid,
                                  double *vals, int mode, int *err, void *stream) {
    if (!fm || g < 0 || g >= fm->ngroups ||
        (mode != FE3D_CSR_ADD && mode != FE3D_CSR_ASSIGN && mode != FE3D_CSR_ATOMIC))
        return FE3D_ERR_ARG;
    const fe3d_fmap_group &G = fm->g[g];
    if (G.nn != 4) return FE3D_ERR_ARG;
    if (G.E == 0 || fm->pat->nnz == 0) return FE3D_OK;
    if (!x || !props || nprops <= 0 || !vals) return FE3D_ERR_ARG;
    if (xmat && xmat_stride != 0 && xmat_stride != 3) return FE3D_ERR_ARG;
    if (fm->pat->max_row_len > 32767) return FE3D_ERR_ARG;  // block offsets are staged as int16
    const int rc = upload_shape_table();
    if (rc) return rc;
    Q4Args a{G.E, nullptr, nullptr, x, nx, xmat, xmat_stride, nullptr, nullptr, nullptr, nullptr, props, nprops, pid,
             nullptr, nullptr, nullptr, 0, 1, err};
    a.vec16 = 0;
    const int64_t cap = (int64_t)kSMs * FE3D_KC0_MINB;
    if (mode == FE3D_CSR_ATOMIC) {
        CsrArgs m{nullptr, G.E, G.node, G.boff, G.first, fm->pat->noderow, fm->pat->nnodes,
                  vals, fm->pat->nnz, 0, 1};
        const int64_t tiles = (G.E + KT - 1) / KT;
        const int grid = (int)(tiles < cap ? tiles : cap);
        quad4_kc0_csr_kernel<<<grid, KNT, sizeof(KSmemCsr), as_stream(stream)>>>(a, m);
        FE3D_CHECK_LAUNCH();
        return FE3D_OK;
    }
    for (int c = 0; c < G.ncolors; c++) {
        const int64_t cnt = G.cstart[c + 1] - G.cstart[c];
        if (cnt == 0) continue;
        CsrArgs m{G.order + G.cstart[c], cnt, G.node, G.boff, G.first, fm->pat->noderow, fm->pat->nnodes,
                  vals, fm->pat->nnz, mode == FE3D_CSR_ASSIGN, 0};
        const int64_t tiles = (cnt + KT - 1) / KT;
        const int grid = (int)(tiles < cap ? tiles : cap);
        quad4_kc0_csr_kernel<<<grid, KNT, sizeof(KSmemCsr), as_stream(stream)>>>(a, m);
        FE3D_CHECK_LAUNCH();
    }
    return FE3D_OK;
}
