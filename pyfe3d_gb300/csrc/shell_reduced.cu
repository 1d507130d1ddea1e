// Reduced-integration shells: Tria3R (pyfe3d/tria3r.pyx) and Quad4R
// (pyfe3d/quad4r.pyx).
//
// Both elements evaluate membrane, bending and transverse shear at one
// centroid point and add a drilling penalty K6ROT 1e-6 A66 (rz - theta_z)^2
// integrated with a full rule (Tria3R: 3 points (2/3, 1/6, 1/6), weight 1/6;
// Quad4R: 2x2 Gauss).  Tria3R scales the transverse shear by
// 1 / (1 + alpha maxl^2 / h^2) (tria3r.pyx:2206-2210); Quad4R adds
// Brockman's hourglass stiffness on u, v, w, rx, ry with the twist mode
// gamma_a = N_a,xy at the centre (quad4r.pyx:1936-1981).
//
// KC0 kernels: phase A (one thread per element, plus one per Quad4R drilling
// point) stages the element's frame, constitutive data and shape-function
// derivatives in shared memory; phase B gives each thread one node pair
// a <= b, builds the 6x6 block (and its transpose) and stages it; phase C
// streams every element's (6 NN)^2 slots with all threads of the block,
// coalesced, adding onto the caller's values.  Flat elements in the XY
// plane (normal +z) are evaluated in the global frame (constitutive data and
// derivatives turned by the in-plane rotation) so their blocks need no
// element-to-global transformation; other elements are evaluated in the
// element frame and transformed with T = blockdiag(R, R).
//
// Quad4R's frame, probes, KG, KG of given stress and mass matrices are those
// of Quad4 (quad4r.pyx:286-548, 4681-12788 restate quad4.pyx:491-752,
// 1365-9489), served by the Quad4 entry points.
#include "ff.cuh"
#include "quad4_common.cuh"

namespace fe3d {
namespace {

constexpr int RNT = 128;  // threads per block of the reduced-shell kernels

struct RSArgs {
    int64_t E;
    const int64_t *cdof, *init_k;
    const double *x;
    int64_t nx;
    const double *xmat;
    int xmat_stride;
    const double *R, *m, *xe, *area;  // probe mode (x == NULL)
    const double *props;
    int64_t nprops;
    const int32_t *pid;
    const double *k6rot;
    int k6rot_stride;  // 0: one value for all elements, 1: per element
    const double *aux;  // Tria3R: alpha_shear_locking; Quad4R: 5 hourglass factors
    int aux_stride;     // 0 (shared) or 1 / 5 (per element)
    int64_t *Kr, *Kc;
    double *Kv;
    int64_t nk;
    int values_only;
    int *err;
};

// Projection of a material direction onto the element plane
// (tria3r.pyx:389-423, the same steps as quad4.pyx:587-624): m is left
// untouched when xmat does not project.
__device__ __forceinline__ void material_direction(const double *z, const double *xa, const double *y, double tol,
                                                   const double *xmat, double *m) {
    double xm[3] = {xmat[0], xmat[1], xmat[2]}, ym[3];
    const double xn = sqrt(xm[0] * xm[0] + xm[1] * xm[1] + xm[2] * xm[2]);
    xm[0] /= xn; xm[1] /= xn; xm[2] /= xn;
    if (!(xn > tol)) return;
    ym[0] = z[1] * xm[2] - z[2] * xm[1];
    ym[1] = z[2] * xm[0] - z[0] * xm[2];
    ym[2] = z[0] * xm[1] - z[1] * xm[0];
    double t = sqrt(ym[0] * ym[0] + ym[1] * ym[1] + ym[2] * ym[2]);
    ym[0] /= t; ym[1] /= t; ym[2] /= t;
    if (!(t > tol)) return;
    xm[0] = ym[1] * z[2] - ym[2] * z[1];
    xm[1] = ym[2] * z[0] - ym[0] * z[2];
    xm[2] = ym[0] * z[1] - ym[1] * z[0];
    t = sqrt(xm[0] * xm[0] + xm[1] * xm[1] + xm[2] * xm[2]);
    xm[0] /= t; xm[1] /= t; xm[2] /= t;
    const double cth = xm[0] * xa[0] + xm[1] * xa[1] + xm[2] * xa[2];
    m[0] = cth;
    m[3] = cth;
    m[1] = (xm[0] * y[0] + xm[1] * y[1] + xm[2] * y[2] > 0) ? -sqrt(1 - cth * cth) : sqrt(1 - cth * cth);
    m[2] = -m[1];
}

// Tria3R frame (tria3r.pyx:294-423): z = v12 x v13, x along v12, y = z x x.
__device__ __forceinline__ void t3_rotation(const double *p1, const double *p2, const double *p3,
                                            const double *xmat, double *R, double *m) {
    double v12[3], v13[3], z[3], xa[3], y[3], t;
#pragma unroll
    for (int i = 0; i < 3; i++) {
        v12[i] = p2[i] - p1[i];
        v13[i] = p3[i] - p1[i];
    }
    z[0] = v12[1] * v13[2] - v12[2] * v13[1];
    z[1] = v12[2] * v13[0] - v12[0] * v13[2];
    z[2] = v12[0] * v13[1] - v12[1] * v13[0];
    // normalisations by the reciprocal square root (FP64 square roots and
    // divisions are costly on this part; the frame agrees with the
    // reference's to rounding)
    const double zz = z[0] * z[0] + z[1] * z[1] + z[2] * z[2];
    t = rsqrt(zz);
    z[0] *= t; z[1] *= t; z[2] *= t;
    t = rsqrt(v12[0] * v12[0] + v12[1] * v12[1] + v12[2] * v12[2]);
    xa[0] = v12[0] * t; xa[1] = v12[1] * t; xa[2] = v12[2] * t;
    y[0] = z[1] * xa[2] - z[2] * xa[1];
    y[1] = z[2] * xa[0] - z[0] * xa[2];
    y[2] = z[0] * xa[1] - z[1] * xa[0];
    t = rsqrt(y[0] * y[0] + y[1] * y[1] + y[2] * y[2]);
    y[0] *= t; y[1] *= t; y[2] *= t;
#pragma unroll
    for (int i = 0; i < 3; i++) {
        R[3 * i + 0] = xa[i];
        R[3 * i + 1] = y[i];
        R[3 * i + 2] = z[i];
    }
    if (xmat) material_direction(z, xa, y, sqrt(zz) / 1e10, xmat, m);
}

// Tria3R area from the local coordinates (tria3r.pyx:530-547).
__device__ __forceinline__ double t3_area(const double *xy) {
    return fabs((-xy[0] + xy[2]) * (-xy[1] + xy[5]) / 2. + (xy[0] - xy[4]) * (-xy[1] + xy[3]) / 2.);
}

// Constant derivatives of the linear triangle (tria3r.pyx:2116-2121).
__device__ __forceinline__ void t3_derivs(const double *xy, double area, double *Nx, double *Ny) {
    const double id = 1. / (2 * area);  // one division for the six
    Nx[0] = (xy[3] - xy[5]) * id;
    Nx[1] = (-xy[1] + xy[5]) * id;
    Nx[2] = (xy[1] - xy[3]) * id;
    Ny[0] = (-xy[2] + xy[4]) * id;
    Ny[1] = (xy[0] - xy[4]) * id;
    Ny[2] = (-xy[0] + xy[2]) * id;
}

// A value of the Quad4R drilling rule: FP64, or float-float (RF_DFF).
union RSlot {
    double d;
    ff f;
};

template <int NN>
struct RSElem {
    static constexpr int NDP = NN == 4 ? 4 : 1;  // stored drilling points (Quad4R)
    double R[9];
    double abd[36];  // evaluation frame (RF_ISO: A11 A12 A66 D11 D12 D66)
    double es[3];    // E44 E45 E55, evaluation frame
    double Nx[NN], Ny[NN];  // centroid derivatives, evaluation frame
    double wc;              // w detJ of the centroid rule
    double kd;              // drilling coefficient 1e-6 K6ROT A66 (element axes)
    RSlot dw[NDP], dNx[NDP][NN], dNy[NDP][NN];  // Quad4R drilling rule (N: rs_shape_n)
    ff xyf[NN == 4 ? 8 : 1];  // RF_DFF (Quad4R): coordinates relative to node 1, float-float
    double gam[NN];  // hourglass mode (Quad4R)
    double hg[7];    // hourglass stiffness (uu, uv, vv, ww, xx, xy, yy), evaluation frame
    double xy[2 * NN];  // nodal coordinates in the evaluation frame
    double Ael[6];      // element-axes membrane stiffness (Quad4R hourglass)
    double ar, hth;     // area, thickness
    long long init_k;
    long long c[NN];
    int flags;
};

enum : int { RF_VALID = 1, RF_ROTATE = 2, RF_ISO = 4, RF_DFF = 8 };

__device__ __forceinline__ double arg_at(const double *a, int stride, int64_t e, int j) {
    return a[(int64_t)stride * e + j];
}

// Quad4R centre rule: derivatives at xi = eta = 0 in the evaluation frame,
// w detJ (weight 4), and the hourglass mode gamma_a = N_a,xy taken in the
// element axes (quad4r.pyx:1949-1981): in the global frame the centre
// inverse Jacobian is turned back (grad_local = R2^T grad_global).
template <int NN>
__device__ __forceinline__ void rs_quad_centre(RSElem<NN> &s) {
    if (NN != 4) return;
    double detJ, N[4];
    quad_derivs(s.xy, 0., 0., detJ, N, s.Nx, s.Ny);
    s.wc = detJ * 4.;
    const double *xy = s.xy;
    const double J11 = 0.25 * (-xy[0] + xy[2] + xy[4] - xy[6]), J12 = 0.25 * (-xy[1] + xy[3] + xy[5] - xy[7]);
    const double J21 = 0.25 * (-xy[0] - xy[2] + xy[4] + xy[6]), J22 = 0.25 * (-xy[1] - xy[3] + xy[5] + xy[7]);
    const double dj = J11 * J22 - J12 * J21;
    const double idj = 1. / dj;
    double j11 = J22 * idj, j12 = -J12 * idj, j21 = -J21 * idj, j22 = J11 * idj;
    if (!(s.flags & RF_ROTATE)) {
        const double r11 = s.R[0], r12 = s.R[1], r21 = s.R[3], r22 = s.R[4];
        const double l11 = r11 * j11 + r21 * j21, l12 = r11 * j12 + r21 * j22;
        const double l21 = r12 * j11 + r22 * j21, l22 = r12 * j12 + r22 * j22;
        j11 = l11; j12 = l12; j21 = l21; j22 = l22;
    }
    const double tw = 0.25 * (j11 * j22 + j12 * j21);
    s.gam[0] = tw;
    s.gam[1] = -tw;
    s.gam[2] = tw;
    s.gam[3] = -tw;
}

// Quad4R hourglass stiffness (quad4r.pyx:1936-1948): equivalent moduli of
// the element-axes A, E_u = f_u 0.1 E1eq h / (1 + 1 / area) and so on,
// turned to the evaluation frame (without the w detJ factor).
template <int NN>
__device__ __forceinline__ void rs_quad_hourglass(const RSArgs &a, int64_t e, RSElem<NN> &s) {
    if (NN != 4) return;
    const double *A = s.Ael;
    const double h = s.hth;
    const double den = -A[0] * A[3] * A[5] + A[0] * A[4] * A[4] + A[1] * A[1] * A[5] -
                       2 * A[1] * A[2] * A[4] + A[2] * A[2] * A[3];
    // a11 = n1 / den and a22 = n2 / den, so E1eq h = den / n1, E2eq h = den / n2,
    // and 1 / (1 + 1 / area) = area / (area + 1): one division for the four
    const double n1 = -A[3] * A[5] + A[4] * A[4], n2 = -A[0] * A[5] + A[2] * A[2];
    const double q = den * s.ar / (n1 * n2 * (s.ar + 1.));
    const double q1 = q * n2, q2 = q * n1;  // E1eq h / sa, E2eq h / sa
    const double *hf = a.aux ? a.aux + (int64_t)a.aux_stride * e : nullptr;
    const double f0 = hf ? hf[0] : 1., f1 = hf ? hf[1] : 1., f2 = hf ? hf[2] : 1., f3 = hf ? hf[3] : 1.,
                 f4 = hf ? hf[4] : 1.;
    const double Eu = f0 * 0.1 * q1, Ev = f1 * 0.1 * q2;
    const double Erx = f3 * 0.1 * q2 * h * h, Ery = f4 * 0.1 * q1 * h * h;
    const double Ew = f2 * 0.5 * (Erx + Ery);
    if (!(s.flags & RF_ROTATE)) {
        // diag(Eu, Ev) and diag(Erx, Ery) turned to the global axes
        const double r11 = s.R[0], r12 = s.R[1], r21 = s.R[3], r22 = s.R[4];
        s.hg[0] = r11 * r11 * Eu + r12 * r12 * Ev;
        s.hg[1] = r11 * r21 * Eu + r12 * r22 * Ev;
        s.hg[2] = r21 * r21 * Eu + r22 * r22 * Ev;
        s.hg[4] = r11 * r11 * Erx + r12 * r12 * Ery;
        s.hg[5] = r11 * r21 * Erx + r12 * r22 * Ery;
        s.hg[6] = r21 * r21 * Erx + r22 * r22 * Ery;
    } else {
        s.hg[0] = Eu;
        s.hg[1] = 0.;
        s.hg[2] = Ev;
        s.hg[4] = Erx;
        s.hg[5] = 0.;
        s.hg[6] = Ery;
    }
    s.hg[3] = Ew;
}

// Phase A of KC0 / fint for element e into s.  global_ok: flat elements of
// the fused mode are evaluated in the global frame (KC0); fint works in the
// element frame (its output is the local finte).  In the global frame the
// coordinates are taken relative to node 1 (no element-frame projection),
// an isotropic section needs no constitutive rotation, and Quad4R's
// hourglass mode (a component of the element-frame Hessian) is obtained by
// turning the centre inverse Jacobian back to the element axes.
template <int NN>
__device__ bool rs_phase_a(const RSArgs &a, int64_t e, RSElem<NN> &s, int size, bool global_ok) {
    s.flags = 0;
    bool ok = true;
#pragma unroll
    for (int i = 0; i < NN; i++) {
        s.c[i] = a.cdof[(int64_t)NN * e + i];
        if (s.c[i] < 0 || (a.x && s.c[i] / 2 + 3 > a.nx)) ok = false;
    }
    const long long k0 = a.init_k ? a.init_k[e] : 0;
    s.init_k = k0;
    if (a.init_k && (k0 < 0 || k0 + size > a.nk)) ok = false;
    const int64_t p = a.pid ? (int64_t)a.pid[e] : e;
    if (p < 0 || p >= a.nprops) ok = false;
    if (!ok) {
        raise_error(a.err, kErrBounds);
        return false;
    }
    double R[9], m[4] = {1., 0., 0., 1.}, ar;
    bool global_frame = false;
    if (a.x) {
        const double *pp[NN];
#pragma unroll
        for (int i = 0; i < NN; i++) pp[i] = a.x + s.c[i] / 2;
        const double *xm = a.xmat ? a.xmat + (int64_t)a.xmat_stride * e : nullptr;
        if (NN == 3)
            t3_rotation(pp[0], pp[1], pp[2], xm, R, m);
        else
            q4_rotation(pp[0], pp[1], pp[2], pp[3], xm, R, m);
        global_frame = global_ok && is_flat(R);
        if (global_frame) {
#pragma unroll
            for (int i = 0; i < NN; i++) {
                s.xy[2 * i] = pp[i][0] - pp[0][0];
                s.xy[2 * i + 1] = pp[i][1] - pp[0][1];
            }
        } else {
#pragma unroll
            for (int i = 0; i < NN; i++) {
                double q[3];
                to_local(R, pp[i], q);
                s.xy[2 * i] = q[0];
                s.xy[2 * i + 1] = q[1];
            }
        }
        ar = NN == 3 ? t3_area(s.xy) : shoelace(s.xy);
    } else {
#pragma unroll
        for (int i = 0; i < 9; i++) R[i] = a.R[9 * e + i];
#pragma unroll
        for (int i = 0; i < 4; i++) m[i] = a.m[4 * e + i];
#pragma unroll
        for (int i = 0; i < NN; i++) {
            s.xy[2 * i] = a.xe[3 * NN * e + 3 * i];
            s.xy[2 * i + 1] = a.xe[3 * NN * e + 3 * i + 1];
        }
        ar = a.area[e];
    }
#pragma unroll
    for (int i = 0; i < 9; i++) s.R[i] = R[i];
    const double *P = a.props + (int64_t)SP_STRIDE * p;
    const double h = P[SP_H];
    const double E44 = P[SP_E44] * P[SP_SCF23];
    const double E45 = P[SP_E45] * 0.5 * (P[SP_SCF13] + P[SP_SCF23]);
    const double E55 = P[SP_E55] * P[SP_SCF13];
    const bool iso = global_frame && iso_section(P, E44, E45, E55);
    // element-axes membrane stiffness: drilling coefficient, Quad4R's
    // equivalent moduli
    double A[6];
    if (m[1] == 0. || iso) {
#pragma unroll
        for (int i = 0; i < 6; i++) A[i] = P[SP_A11 + i];
    } else {
        rotate_plane(m[0], m[1], m[2], m[3], P + SP_A11, A);
    }
    if (iso) {
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
        q4_constitutive(P, m, R, global_frame, s.abd, s.es);
    }
    s.kd = 1e-6 * arg_at(a.k6rot, a.k6rot_stride, e, 0) * A[5];
    if (NN == 3) {
        t3_derivs(s.xy, ar, s.Nx, s.Ny);
        s.wc = 2 * ar * 0.5;
        // shear locking factor alpha maxl^2 / h^2 (tria3r.pyx:2195-2210)
        const double *xy = s.xy;
        const double l12 = (xy[0] - xy[2]) * (xy[0] - xy[2]) + (xy[1] - xy[3]) * (xy[1] - xy[3]);
        const double l23 = (xy[2] - xy[4]) * (xy[2] - xy[4]) + (xy[3] - xy[5]) * (xy[3] - xy[5]);
        const double l31 = (xy[4] - xy[0]) * (xy[4] - xy[0]) + (xy[5] - xy[1]) * (xy[5] - xy[1]);
        const double maxl2 = fmax(l12, fmax(l23, l31));
        // 1 / (1 + alpha maxl^2 / h^2) = h^2 / (h^2 + alpha maxl^2)
        const double sf = h * h / (h * h + arg_at(a.aux, a.aux_stride, e, 0) * maxl2);
#pragma unroll
        for (int i = 0; i < 3; i++) s.es[i] = sf * s.es[i];
#pragma unroll
        for (int i = 0; i < 7; i++) s.hg[i] = 0.;
#pragma unroll
        for (int i = 0; i < NN; i++) s.gam[i] = 0.;
    } else {
        // centre rule and hourglass data: rs_quad_centre, rs_quad_hourglass
#pragma unroll
        for (int i = 0; i < 6; i++) s.Ael[i] = A[i];
        s.ar = ar;
        s.hth = h;
    }
    bool dff = false;
    if (NN == 4) {
        // the drilling rule in float-float from coordinates relative to node 1
        dff = true;
        double d[2 * NN];
#pragma unroll
        for (int i = 0; i < NN; i++) {
            d[2 * i] = s.xy[2 * i] - s.xy[0];
            d[2 * i + 1] = s.xy[2 * i + 1] - s.xy[1];
            dff &= ff_safe(d[2 * i]) && ff_safe(d[2 * i + 1]);
        }
        if (dff)
#pragma unroll
            for (int i = 0; i < 2 * NN; i++) s.xyf[i] = ff_from_double(d[i]);
    }
    s.flags = RF_VALID | (global_frame ? 0 : RF_ROTATE) | (iso ? RF_ISO : 0) | (dff ? RF_DFF : 0);
    if (NN == 4) {
        rs_quad_centre<NN>(s);
        rs_quad_hourglass<NN>(a, e, s);
    }
    return true;
}

// Shape-function values and natural derivatives at the 2x2 Gauss points in
// float-float, [point][0: N, 1: dN/dxi, 2: dN/deta][node] (the expressions
// of quad_derivs), one copy per block.
__device__ __forceinline__ void rs_shape_table(ff (*sh)[3][4], int tid) {
    if (tid < 48) {
        const int g = tid / 12, t = (tid / 4) % 3, i = tid & 3;
        const double xi = (g & 2) ? kGauss : -kGauss, eta = (g & 1) ? kGauss : -kGauss;
        const double sx = (i == 1 || i == 2) ? 1. : -1., sy = (i >= 2) ? 1. : -1.;
        const double v = t == 0 ? 0.25 * (1 + sx * xi) * (1 + sy * eta)
                       : t == 1 ? 0.25 * sx * (1 + sy * eta) : 0.25 * sy * (1 + sx * xi);
        sh[g][t][i] = ff_from_double(v);
    }
}

// N_i at drilling point g in FP64 (the expression of quad_derivs).
__device__ __forceinline__ double rs_shape_n(int g, int i) {
    const double xi = (g & 2) ? kGauss : -kGauss, eta = (g & 1) ? kGauss : -kGauss;
    const double sx = (i == 1 || i == 2) ? 1. : -1., sy = (i >= 2) ? 1. : -1.;
    return 0.25 * (1 + sx * xi) * (1 + sy * eta);
}

// Quad4R drilling point g of a staged element (2x2 Gauss, unit weights,
// quad4r.pyx:3305-3360), from the evaluation-frame coordinates: detJ and the
// Cartesian derivatives, in float-float for RF_DFF elements (the drilling
// terms carry the factor 1e-6 K6ROT A66, far below the element's largest
// entries), else in FP64.
template <int NN>
__device__ __forceinline__ void rs_drill_point(RSElem<NN> &s, const ff (*sh)[3][4], int g) {
    if (NN != 4) return;
    const int q = g % RSElem<NN>::NDP;
    if (s.flags & RF_DFF) {
        const ff *x = s.xyf;
        ff J11 = ff_mul(x[0], sh[g][1][0]), J12 = ff_mul(x[1], sh[g][1][0]);
        ff J21 = ff_mul(x[0], sh[g][2][0]), J22 = ff_mul(x[1], sh[g][2][0]);
#pragma unroll
        for (int i = 1; i < NN; i++) {
            J11 = ff_fma(x[2 * i], sh[g][1][i], J11);
            J12 = ff_fma(x[2 * i + 1], sh[g][1][i], J12);
            J21 = ff_fma(x[2 * i], sh[g][2][i], J21);
            J22 = ff_fma(x[2 * i + 1], sh[g][2][i], J22);
        }
        const ff det = ff_fma(J11, J22, ff_neg(ff_mul(J12, J21)));
        const ff inv = ff_rcp(det);
        s.dw[q].f = det;
#pragma unroll
        for (int i = 0; i < NN; i++) {
            const ff dxi = sh[g][1][i], deta = sh[g][2][i];
            s.dNx[q][i].f = ff_mul(ff_fma(J22, dxi, ff_neg(ff_mul(J12, deta))), inv);
            s.dNy[q][i].f = ff_mul(ff_fma(J11, deta, ff_neg(ff_mul(J21, dxi))), inv);
        }
        return;
    }
    double detJ, N[4], Nx[4], Ny[4];
    const double xi = (g & 2) ? kGauss : -kGauss, eta = (g & 1) ? kGauss : -kGauss;
    quad_derivs(s.xy, xi, eta, detJ, N, Nx, Ny);
    s.dw[q].d = detJ;
#pragma unroll
    for (int i = 0; i < NN; i++) {
        s.dNx[q][i].d = Nx[i];
        s.dNy[q][i].d = Ny[i];
    }
}

// 6x6 block of node pair (a, b) in the evaluation frame.  kc0_rule: the
// Tria3R update_KC0 transformation (tria3r.pyx:2323-2960) keeps, of the
// drilling DOF rz, only the diagonal rz_a - rz_a terms (its couplings with
// u, v and with the rz of the other nodes do not reach KC0v), while
// update_probe_finte uses the whole local matrix.
template <int NN>
__device__ __forceinline__ void rs_block(const RSElem<NN> &s, const ff (*sh)[3][4], int a, int b, bool kc0_rule,
                                         double K[6][6]) {
    const double w = s.wc, Nc = NN == 3 ? 0.33333333333333333333 : 0.25;
    const double xa = s.Nx[a], ya = s.Ny[a], xb = s.Nx[b], yb = s.Ny[b];
    const double wxa = w * xa, wya = w * ya;
    const double H[2][2] = {{wxa * xb, wxa * yb}, {wya * xb, wya * yb}};
#pragma unroll
    for (int i = 0; i < 6; i++)
#pragma unroll
        for (int j = 0; j < 6; j++) K[i][j] = 0.;
    if (s.flags & RF_ISO) {
        // A16 = A26 = 0, A22 = A11, B = 0, D likewise
        const double A11 = s.abd[0], A12 = s.abd[1], A66 = s.abd[2];
        const double D11 = s.abd[3], D12 = s.abd[4], D66 = s.abd[5];
        K[0][0] = A11 * H[0][0] + A66 * H[1][1];
        K[0][1] = A12 * H[0][1] + A66 * H[1][0];
        K[1][0] = A12 * H[1][0] + A66 * H[0][1];
        K[1][1] = A66 * H[0][0] + A11 * H[1][1];
        K[3][3] = D66 * H[0][0] + D11 * H[1][1];
        K[3][4] = -(D66 * H[0][1] + D12 * H[1][0]);
        K[4][3] = -(D12 * H[0][1] + D66 * H[1][0]);
        K[4][4] = D11 * H[0][0] + D66 * H[1][1];
    } else {
        // membrane and bending: u -> (exx, gxy), v -> (gxy, eyy),
        // rx -> -(kxy, kyy), ry -> (kxx, kxy)
        const int dof[4] = {0, 1, 3, 4};
        const int sidx[4][2] = {{0, 2}, {2, 1}, {5, 4}, {3, 5}};
        const double sg[4] = {1., 1., -1., 1.};
#pragma unroll
        for (int mi = 0; mi < 4; mi++)
#pragma unroll
            for (int ni = 0; ni < 4; ni++) {
                double v = 0.;
#pragma unroll
                for (int p = 0; p < 2; p++)
#pragma unroll
                    for (int q = 0; q < 2; q++) v += s.abd[6 * sidx[mi][p] + sidx[ni][q]] * H[p][q];
                K[dof[mi]][dof[ni]] = sg[mi] * sg[ni] * v;
            }
    }
    // transverse shear at the centroid, (gyz, gxz) = (w_y - rx N, w_x + ry N)
    const double E44 = s.es[0], E45 = s.es[1], E55 = s.es[2];
    const double wNc = w * Nc;
    const double ya0 = wya * Nc, xa0 = wxa * Nc, y0b = wNc * yb, x0b = wNc * xb, nn0 = wNc * Nc;
    if (s.flags & RF_ISO) {
        // E45 = 0
        K[2][2] += E44 * H[1][1] + E55 * H[0][0];
        K[2][3] -= E44 * ya0;
        K[2][4] += E55 * xa0;
        K[3][2] -= E44 * y0b;
        K[4][2] += E55 * x0b;
        K[3][3] += E44 * nn0;
        K[4][4] += E55 * nn0;
    } else {
        K[2][2] += E44 * H[1][1] + E45 * (H[1][0] + H[0][1]) + E55 * H[0][0];
        K[2][3] -= E44 * ya0 + E45 * xa0;
        K[2][4] += E45 * ya0 + E55 * xa0;
        K[3][2] -= E44 * y0b + E45 * x0b;
        K[4][2] += E45 * y0b + E55 * x0b;
        K[3][3] += E44 * nn0;
        K[3][4] -= E45 * nn0;
        K[4][3] -= E45 * nn0;
        K[4][4] += E55 * nn0;
    }
    // drilling: d = u N_y/2 - v N_x/2 + rz N over the drilling rule
    double hnn, hnx, hny, hxn, hyn, hxx, hxy, hyx, hyy;
    if (NN == 3) {
        // constant derivatives; the 3-point rule (2/3, 1/6, 1/6) has
        // sum_g N_a = 1 and sum_g N_a N_b = 1/2 (a = b), 1/4 (a != b), with
        // total weight w = detJ / 2
        const double d3 = w * 0.33333333333333333333;
        hnn = d3 * (a == b ? 0.5 : 0.25);
        hnx = d3 * xb;
        hny = d3 * yb;
        hxn = d3 * xa;
        hyn = d3 * ya;
        hxx = H[0][0];
        hxy = H[0][1];
        hyx = H[1][0];
        hyy = H[1][1];
    } else if (s.flags & RF_DFF) {
        // the drilling rule's tensor sum_g w (N, N_x, N_y)_a (N, N_x, N_y)_b
        // in float-float
        ff h[3][3];
#pragma unroll
        for (int p = 0; p < 3; p++)
#pragma unroll
            for (int q = 0; q < 3; q++) h[p][q] = {0.f, 0.f};
#pragma unroll
        for (int g = 0; g < RSElem<NN>::NDP; g++) {
            const ff wg = s.dw[g].f;
            const ff va[3] = {ff_mul(wg, sh[g][0][a]), ff_mul(wg, s.dNx[g][a].f), ff_mul(wg, s.dNy[g][a].f)};
            const ff vb[3] = {sh[g][0][b], s.dNx[g][b].f, s.dNy[g][b].f};
#pragma unroll
            for (int p = 0; p < 3; p++)
#pragma unroll
                for (int q = 0; q < 3; q++) h[p][q] = ff_fma(va[p], vb[q], h[p][q]);
        }
        hnn = ff_to_double(h[0][0]);
        hnx = ff_to_double(h[0][1]);
        hny = ff_to_double(h[0][2]);
        hxn = ff_to_double(h[1][0]);
        hxx = ff_to_double(h[1][1]);
        hxy = ff_to_double(h[1][2]);
        hyn = ff_to_double(h[2][0]);
        hyx = ff_to_double(h[2][1]);
        hyy = ff_to_double(h[2][2]);
    } else {
        hnn = hnx = hny = hxn = hyn = hxx = hxy = hyx = hyy = 0.;
#pragma unroll
        for (int g = 0; g < RSElem<NN>::NDP; g++) {
            const double wg = s.dw[g].d;
            const double na = wg * rs_shape_n(g, a), nxa = wg * s.dNx[g][a].d, nya = wg * s.dNy[g][a].d;
            const double nb = rs_shape_n(g, b), nxb = s.dNx[g][b].d, nyb = s.dNy[g][b].d;
            hnn += na * nb;
            hnx += na * nxb;
            hny += na * nyb;
            hxn += nxa * nb;
            hyn += nya * nb;
            hxx += nxa * nxb;
            hxy += nxa * nyb;
            hyx += nya * nxb;
            hyy += nya * nyb;
        }
    }
    const double kd = s.kd;
    K[0][0] += kd * 0.25 * hyy;
    K[0][1] -= kd * 0.25 * hyx;
    K[1][0] -= kd * 0.25 * hxy;
    K[1][1] += kd * 0.25 * hxx;
    if (!(NN == 3 && kc0_rule)) {
        K[0][5] += kd * 0.5 * hyn;
        K[1][5] -= kd * 0.5 * hxn;
        K[5][0] += kd * 0.5 * hny;
        K[5][1] -= kd * 0.5 * hnx;
        K[5][5] += kd * hnn;
    } else if (a == b) {
        K[5][5] += kd * hnn;
    }
    if (NN == 4) {
        const double g = s.gam[a] * s.gam[b] * w;
        K[0][0] += g * s.hg[0];
        K[0][1] += g * s.hg[1];
        K[1][0] += g * s.hg[1];
        K[1][1] += g * s.hg[2];
        K[2][2] += g * s.hg[3];
        K[3][3] += g * s.hg[4];
        K[3][4] += g * s.hg[5];
        K[4][3] += g * s.hg[5];
        K[4][4] += g * s.hg[6];
    }
}

// elements staged per pass: 8 (Quad4R) and 9 (Tria3R) keep the shared memory
// of a block small enough for 3 and 4 blocks per SM (measured faster than
// 12 and 18 at 2 and 3 blocks per SM, whose passes keep more threads busy)
#ifndef FE3D_RS_TB4
#define FE3D_RS_TB4 8
#endif
#ifndef FE3D_RS_TB3
#define FE3D_RS_TB3 9
#endif
template <int NN>
struct RSTile {
    static constexpr int S = 6 * NN;                 // rows of the element matrix
    static constexpr int S2 = S * S;                 // slots per element
    // staged row and element strides (doubles): rows 16-byte aligned; the
    // node pairs of a warp's stage updates spread over the banks (at most
    // 2-way conflicts), consecutive elements shifted by 4 or 12 banks
    static constexpr int RS = NN == 4 ? 26 : S;
    static constexpr int SP = S * RS + 2;
    static constexpr int P = NN * (NN + 1) / 2;      // node pairs a <= b
    // TE elements per tile: phase A runs on one full warp (the FP64 pipe
    // charges a warp instruction whatever its active lanes); the blocks are
    // staged TB elements at a time
    static constexpr int TE = 32;
    static constexpr int TB = NN == 4 ? FE3D_RS_TB4 : FE3D_RS_TB3;
    static constexpr size_t smem = (size_t)TB * SP * sizeof(double) + (size_t)TE * sizeof(RSElem<NN>);
};

template <int NN>
__device__ __forceinline__ void pair_of(int p, int &a, int &b) {
    // p-th pair (a, b), a <= b, in row order
    a = 0;
    int rem = p;
    while (rem >= NN - a) {
        rem -= NN - a;
        a++;
    }
    b = a + rem;
}

// The caller's current values of elements e0 .. e0 + nel - 1, copied into
// the stage with cp.async (16-byte pieces where the element's slots are
// 16-byte aligned, else 8-byte pieces).
template <int NN>
__device__ __forceinline__ void rs_prefetch(const RSArgs &a, int64_t e0, int nel, double *stage, int tid) {
    using Tl = RSTile<NN>;
    constexpr int H = Tl::S2 / 2;  // 16-byte pieces per element
    for (int i = tid; i < nel * H; i += RNT) {
        const int el = i / H, j = i - el * H;
        const int64_t e = e0 + el;
        if (e >= a.E) break;
        const long long k0 = a.init_k[e];
        if (k0 < 0 || k0 + Tl::S2 > a.nk) continue;  // phase A reports it
        const int row = (2 * j) / Tl::S, col = 2 * j - row * Tl::S;
        const double *src = a.Kv + k0 + 2 * j;
        double *dst = stage + (size_t)el * Tl::SP + row * Tl::RS + col;
        if ((reinterpret_cast<uintptr_t>(src) & 15) == 0) {
            cp_async16(dst, src);
        } else {
            cp_async8(dst, src);
            cp_async8(dst + 1, src + 1);
        }
    }
    cp_async_commit();
}

template <int NN>
__global__ void __launch_bounds__(RNT) rs_kc0_kernel(RSArgs a) {
    using Tl = RSTile<NN>;
    extern __shared__ __align__(16) double rs_smem[];
    double *stage = rs_smem;
    RSElem<NN> *se = reinterpret_cast<RSElem<NN> *>(rs_smem + (size_t)Tl::TB * Tl::SP);
    __shared__ ff sh[4][3][4];
    const int tid = threadIdx.x;
    if (NN == 4) rs_shape_table(sh, tid);
    const int64_t ntiles = (a.E + Tl::TE - 1) / Tl::TE;
    for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int64_t e0 = tile * Tl::TE;
        __syncthreads();
        rs_prefetch<NN>(a, e0, Tl::TB, stage, tid);
        if (tid < Tl::TE) {
            se[tid].flags = 0;
            if (e0 + tid < a.E) rs_phase_a<NN>(a, e0 + tid, se[tid], Tl::S2, true);
        }
        if (NN == 4) {
            __syncthreads();
            if (tid < 4 * Tl::TE) {
                RSElem<NN> &s = se[tid >> 2];
                if (s.flags & RF_VALID) rs_drill_point<NN>(s, sh, tid & 3);
            }
        }
        for (int r0 = 0; r0 < Tl::TE; r0 += Tl::TB) {
            const int nb = Tl::TE - r0 < Tl::TB ? Tl::TE - r0 : Tl::TB;
            if (r0 > 0) {
                __syncthreads();  // the previous pass's write-out has read the stage
                rs_prefetch<NN>(a, e0 + r0, nb, stage, tid);
            }
            // the element data and (first pass of the tile) the prefetches of every thread
            cp_async_wait_all();
            __syncthreads();
            if (tid < nb * Tl::P) {
                const int el = tid / Tl::P;
                const RSElem<NN> &s = se[r0 + el];
                if (s.flags & RF_VALID) {
                    int pa, pb;
                    pair_of<NN>(tid - el * Tl::P, pa, pb);
                    double K[6][6];
                    rs_block<NN>(s, sh, pa, pb, true, K);
                    if (s.flags & RF_ROTATE) rotate_block(s.R, K);
                    double *st = stage + (size_t)el * Tl::SP;
                    // an isotropic block in the global frame couples (u, v,
                    // rz) and (w, rx, ry) only: the cross entries are exact
                    // zeros and the staged values there are left as they are
                    const bool iso = s.flags & RF_ISO;
#pragma unroll
                    for (int m = 0; m < 6; m++)
#pragma unroll
                        for (int n = 0; n < 6; n++) {
                            const bool gm = m >= 2 && m <= 4, gn = n >= 2 && n <= 4;
                            if (iso && gm != gn) continue;
                            st[(6 * pa + m) * Tl::RS + 6 * pb + n] += K[m][n];
                            if (pa != pb) st[(6 * pb + n) * Tl::RS + 6 * pa + m] += K[m][n];
                        }
                }
            }
            __syncthreads();
            for (int e2 = 0; e2 < nb; e2++) {
                const RSElem<NN> &s = se[r0 + e2];
                if (!(s.flags & RF_VALID)) continue;
                const long long k0 = s.init_k;
                const double *st = stage + (size_t)e2 * Tl::SP;
                double *kv = a.Kv + k0;
                if ((reinterpret_cast<uintptr_t>(kv) & 15) == 0) {
                    for (int i = tid; i < Tl::S2 / 2; i += RNT) {
                        const int q = 2 * i, row = q / Tl::S, col = q - row * Tl::S;
                        reinterpret_cast<double2 *>(kv)[i] =
                            *reinterpret_cast<const double2 *>(st + row * Tl::RS + col);
                    }
                } else {
                    for (int i = tid; i < Tl::S2; i += RNT) {
                        const int row = i / Tl::S, col = i - row * Tl::S;
                        kv[i] = st[row * Tl::RS + col];
                    }
                }
                if (!a.values_only) {
                    int64_t *kr = a.Kr + k0, *kc = a.Kc + k0;
                    const bool v2 = ((reinterpret_cast<uintptr_t>(kr) | reinterpret_cast<uintptr_t>(kc)) & 15) == 0;
                    if (v2) {
                        for (int i = tid; i < Tl::S2 / 2; i += RNT) {
                            const int q = 2 * i, row = q / Tl::S, col = q - row * Tl::S;
                            const long long r = s.c[row / 6] + row % 6, c0 = s.c[col / 6] + col % 6;
                            // col is even and S a multiple of 6: col + 1 stays in node col / 6
                            reinterpret_cast<longlong2 *>(kr)[i] = make_longlong2(r, r);
                            reinterpret_cast<longlong2 *>(kc)[i] = make_longlong2(c0, c0 + 1);
                        }
                    } else {
                        for (int i = tid; i < Tl::S2; i += RNT) {
                            const int row = i / Tl::S, col = i - row * Tl::S;
                            kr[i] = s.c[row / 6] + row % 6;
                            kc[i] = s.c[col / 6] + col % 6;
                        }
                    }
                }
            }
        }
    }
}

// finte = KC0e ue in the element frame (tria3r.pyx:549-947,
// quad4r.pyx:549-1143) and/or fint[c + .] += R finte (tria3r.pyx:2975-3017,
// quad4r.pyx:4620-4679).  One thread per node pair (a, b) forms Ke_ab ue_b;
// the partial products are summed per node row, rotated and added
// atomically (elements share nodes).
template <int NN>
__global__ void __launch_bounds__(RNT) rs_fint_kernel(RSArgs a, const double *ue, double *fint, int64_t nf,
                                                       double *finte) {
    constexpr int PP = NN * NN, T = RNT / PP;
    __shared__ RSElem<NN> se[T];
    __shared__ double part[T][NN][NN][6];
    __shared__ double fl[T][NN][6];
    __shared__ ff sh[4][3][4];
    const int tid = threadIdx.x;
    if (NN == 4) rs_shape_table(sh, tid);
    const int64_t ntiles = (a.E + T - 1) / T;
    for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int64_t e0 = tile * T;
        __syncthreads();
        if (tid < T) {
            se[tid].flags = 0;
            if (e0 + tid < a.E) rs_phase_a<NN>(a, e0 + tid, se[tid], 0, false);
        }
        __syncthreads();
        if (NN == 4 && tid < 4 * T) {
            RSElem<NN> &s = se[tid >> 2];
            if (s.flags & RF_VALID) rs_drill_point<NN>(s, sh, tid & 3);
        }
        __syncthreads();
        if (tid < T * PP) {
            const int el = tid / PP, pr = tid - el * PP, pa = pr / NN, pb = pr - pa * NN;
            const RSElem<NN> &s = se[el];
            if (s.flags & RF_VALID) {
                double K[6][6];
                rs_block<NN>(s, sh, pa, pb, false, K);
                const double *u = ue + 6 * NN * (e0 + el) + 6 * pb;
                double ub[6];
#pragma unroll
                for (int n = 0; n < 6; n++) ub[n] = u[n];
#pragma unroll
                for (int m = 0; m < 6; m++) {
                    double v = 0.;
#pragma unroll
                    for (int n = 0; n < 6; n++) v += K[m][n] * ub[n];
                    part[el][pa][pb][m] = v;
                }
            }
        }
        __syncthreads();
        for (int i = tid; i < T * NN * 6; i += RNT) {
            const int el = i / (NN * 6), r = i - el * NN * 6, na = r / 6, m = r - na * 6;
            if (se[el].flags & RF_VALID) {
                double v = 0.;
#pragma unroll
                for (int b = 0; b < NN; b++) v += part[el][na][b][m];
                fl[el][na][m] = v;
                if (finte) finte[6 * NN * (e0 + el) + 6 * na + m] = v;
            }
        }
        __syncthreads();
        for (int i = tid; fint && i < T * NN * 6; i += RNT) {
            const int el = i / (NN * 6), r = i - el * NN * 6, na = r / 6, m = r - na * 6;
            const RSElem<NN> &s = se[el];
            if (s.flags & RF_VALID) {
                const int g = m / 3, i = m % 3;
                const double *f = fl[el][na] + 3 * g;
                const double v = f[0] * s.R[3 * i + 0] + f[1] * s.R[3 * i + 1] + f[2] * s.R[3 * i + 2];
                const long long k = s.c[na] + m;
                if (k < 0 || k >= nf)
                    raise_error(a.err, kErrBounds);
                else
                    atomicAdd(fint + k, v);
            }
        }
    }
}

// --- Tria3R frame / probes (tria3r.pyx:294-547) ---------------------------
__global__ void t3_frame_kernel(int64_t E, const int64_t *cdof, const double *x, int64_t nx, const double *xmat,
                                int xmat_stride, const double *Rin, double *Ro, double *mo, double *xeo,
                                double *areao, int *err) {
    const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= E) return;
    long long c[3];
#pragma unroll
    for (int i = 0; i < 3; i++) {
        c[i] = cdof[3 * e + i];
        if (c[i] < 0 || c[i] / 2 + 3 > nx) {
            raise_error(err, kErrBounds);
            return;
        }
    }
    const double *pp[3] = {x + c[0] / 2, x + c[1] / 2, x + c[2] / 2};
    double R[9], m[4] = {1., 0., 0., 1.};
    if (Rin) {
        // probe update with the frame the element holds
#pragma unroll
        for (int i = 0; i < 9; i++) R[i] = Rin[9 * e + i];
    } else {
        if (mo)
#pragma unroll
            for (int i = 0; i < 4; i++) m[i] = mo[4 * e + i];
        t3_rotation(pp[0], pp[1], pp[2], xmat ? xmat + (int64_t)xmat_stride * e : nullptr, R, m);
        if (Ro)
#pragma unroll
            for (int i = 0; i < 9; i++) Ro[9 * e + i] = R[i];
        if (mo)
#pragma unroll
            for (int i = 0; i < 4; i++) mo[4 * e + i] = m[i];
    }
    double xe[9];
#pragma unroll
    for (int i = 0; i < 3; i++) to_local(R, pp[i], xe + 3 * i);
    if (xeo)
#pragma unroll
        for (int i = 0; i < 9; i++) xeo[9 * e + i] = xe[i];
    if (areao) {
        const double xy[6] = {xe[0], xe[1], xe[3], xe[4], xe[6], xe[7]};
        areao[e] = t3_area(xy);
    }
}

// --- Tria3R KG (tria3r.pyx:3020-4061) --------------------------------------
// One centroid point: the membrane resultants from ue (or given), then
// KG_ab = r_m3 r_n3 (grad N_a . Nmat . grad N_b) detJ / 2 on the
// translations, 81 slots row-major over (node, u v w).
struct T3KGElem {
    double r3[3];
    double Nx[3], Ny[3];
    double Nxx, Nyy, Nxy, w;
    long long init_k, c[3];
    int valid;
};

__global__ void __launch_bounds__(RNT) t3_kg_kernel(RSArgs a, const double *u, int64_t nu, const double *ue_in,
                                                    const double *nstress, int ns_stride) {
    __shared__ T3KGElem se[RNT];
    const int tid = threadIdx.x;
    const int64_t ntiles = (a.E + RNT - 1) / RNT;
    for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int64_t e0 = tile * RNT, e = e0 + tid;
        __syncthreads();
        T3KGElem &s = se[tid];
        s.valid = 0;
        if (e < a.E) {
            bool ok = true;
            for (int i = 0; i < 3; i++) {
                s.c[i] = a.cdof[3 * e + i];
                if (s.c[i] < 0 || (a.x && s.c[i] / 2 + 3 > a.nx) || (a.x && !nstress && s.c[i] + 6 > nu)) ok = false;
            }
            s.init_k = a.init_k[e];
            if (s.init_k < 0 || s.init_k + 81 > a.nk) ok = false;
            const int64_t p = a.pid ? (int64_t)a.pid[e] : e;
            if (!nstress && (p < 0 || p >= a.nprops)) ok = false;
            if (!ok) {
                raise_error(a.err, kErrBounds);
            } else {
                double R[9], m[4] = {1., 0., 0., 1.}, xy[6], ar;
                if (a.x) {
                    const double *pp[3] = {a.x + s.c[0] / 2, a.x + s.c[1] / 2, a.x + s.c[2] / 2};
                    t3_rotation(pp[0], pp[1], pp[2], a.xmat ? a.xmat + (int64_t)a.xmat_stride * e : nullptr, R, m);
                    for (int i = 0; i < 3; i++) {
                        double q[3];
                        to_local(R, pp[i], q);
                        xy[2 * i] = q[0];
                        xy[2 * i + 1] = q[1];
                    }
                    ar = t3_area(xy);
                } else {
                    for (int i = 0; i < 9; i++) R[i] = a.R[9 * e + i];
                    if (a.m)
                        for (int i = 0; i < 4; i++) m[i] = a.m[4 * e + i];
                    for (int i = 0; i < 3; i++) {
                        xy[2 * i] = a.xe[9 * e + 3 * i];
                        xy[2 * i + 1] = a.xe[9 * e + 3 * i + 1];
                    }
                    ar = a.area[e];
                }
                t3_derivs(xy, ar, s.Nx, s.Ny);
                s.r3[0] = R[2];
                s.r3[1] = R[5];
                s.r3[2] = R[8];
                s.w = 2 * ar * 0.5;
                if (nstress) {
                    s.Nxx = nstress[(int64_t)ns_stride * e + 0];
                    s.Nyy = nstress[(int64_t)ns_stride * e + 1];
                    s.Nxy = nstress[(int64_t)ns_stride * e + 2];
                } else {
                    double uel[18];
                    if (a.x) {
                        for (int j = 0; j < 3; j++) {
                            to_local(R, u + s.c[j], uel + 6 * j);
                            to_local(R, u + s.c[j] + 3, uel + 6 * j + 3);
                        }
                    } else {
                        for (int i = 0; i < 18; i++) uel[i] = ue_in[18 * e + i];
                    }
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
                    double exx = 0, eyy = 0, gxy = 0, kxx = 0, kyy = 0, kxy = 0;
                    for (int j = 0; j < 3; j++) {
                        const double *uj = uel + 6 * j;
                        exx += s.Nx[j] * uj[0];
                        eyy += s.Ny[j] * uj[1];
                        gxy += s.Ny[j] * uj[0] + s.Nx[j] * uj[1];
                        kxx += s.Nx[j] * uj[4];
                        kyy += -s.Ny[j] * uj[3];
                        kxy += -s.Nx[j] * uj[3] + s.Ny[j] * uj[4];
                    }
                    s.Nxx = A[0] * exx + A[1] * eyy + A[2] * gxy + B[0] * kxx + B[1] * kyy + B[2] * kxy;
                    s.Nyy = A[1] * exx + A[3] * eyy + A[4] * gxy + B[1] * kxx + B[3] * kyy + B[4] * kxy;
                    s.Nxy = A[2] * exx + A[4] * eyy + A[5] * gxy + B[2] * kxx + B[4] * kyy + B[5] * kxy;
                }
                s.valid = 1;
            }
        }
        __syncthreads();
        const int nel = (int)((a.E - e0) < RNT ? (a.E - e0) : RNT);
        // in batches of 8 slots per thread: the caller's values first (all
        // loads in flight), then the stores
        for (int i0 = tid; i0 < nel * 81; i0 += 8 * RNT) {
            double old[8];
#pragma unroll
            for (int u = 0; u < 8; u++) {
                const int i = i0 + u * RNT, el = i / 81;
                old[u] = (i < nel * 81 && se[el].valid) ? a.Kv[se[el].init_k + (i - el * 81)] : 0.;
            }
#pragma unroll
            for (int u = 0; u < 8; u++) {
                const int i = i0 + u * RNT;
                if (i >= nel * 81) break;
                const int el = i / 81, j = i - el * 81;
                const T3KGElem &t = se[el];
                if (!t.valid) continue;
                const int row = j / 9, col = j - row * 9;
                const int na = row / 3, mm = row % 3, nb = col / 3, nn = col % 3;
                const double g = (t.Nx[nb] * (t.Nx[na] * t.Nxx + t.Ny[na] * t.Nxy) +
                                  t.Ny[nb] * (t.Nx[na] * t.Nxy + t.Ny[na] * t.Nyy)) *
                                 t.w;
                const long long k = t.init_k + j;
                a.Kv[k] = old[u] + t.r3[mm] * t.r3[nn] * g;
                if (!a.values_only) {
                    a.Kr[k] = t.c[na] + mm;
                    a.Kc[k] = t.c[nb] + nn;
                }
            }
        }
    }
}

// --- Tria3R mass (tria3r.pyx:4063-7723) -------------------------------------
// h_ab from the 3-point rule (mtype 0), detJ/18 (mtype 1) or the vertex rule
// (mtype 2, like-kind DOF pairs only) times the nodal 6x6 pattern of
// intrho / intrhoz / intrhoz2 turned to the global axes.
struct T3MElem {
    double h[9];
    double G[36];
    long long init_k, c[3];
    int valid;
};

__global__ void __launch_bounds__(RNT) t3_m_kernel(RSArgs a, int mtype) {
    constexpr int TM = 32;
    __shared__ T3MElem se[TM];
    const int tid = threadIdx.x;
    const int ncol = mtype == 2 ? 9 : 15, size = 18 * ncol;
    const int64_t ntiles = (a.E + TM - 1) / TM;
    for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int64_t e0 = tile * TM;
        __syncthreads();
        if (tid < TM) {
            T3MElem &s = se[tid];
            s.valid = 0;
            const int64_t e = e0 + tid;
            if (e < a.E) {
                bool ok = true;
                for (int i = 0; i < 3; i++) {
                    s.c[i] = a.cdof[3 * e + i];
                    if (s.c[i] < 0 || (a.x && s.c[i] / 2 + 3 > a.nx)) ok = false;
                }
                s.init_k = a.init_k[e];
                if (s.init_k < 0 || s.init_k + size > a.nk) ok = false;
                const int64_t p = a.pid ? (int64_t)a.pid[e] : e;
                if (p < 0 || p >= a.nprops) ok = false;
                if (!ok) {
                    raise_error(a.err, kErrBounds);
                } else {
                    double R[9], ar;
                    if (a.x) {
                        double m[4] = {1., 0., 0., 1.}, xy[6];
                        const double *pp[3] = {a.x + s.c[0] / 2, a.x + s.c[1] / 2, a.x + s.c[2] / 2};
                        t3_rotation(pp[0], pp[1], pp[2], nullptr, R, m);
                        for (int i = 0; i < 3; i++) {
                            double q[3];
                            to_local(R, pp[i], q);
                            xy[2 * i] = q[0];
                            xy[2 * i + 1] = q[1];
                        }
                        ar = t3_area(xy);
                    } else {
                        for (int i = 0; i < 9; i++) R[i] = a.R[9 * e + i];
                        ar = a.area[e];
                    }
                    const double detJ = 2 * ar;
                    if (mtype == 1) {
                        for (int i = 0; i < 9; i++) s.h[i] = detJ / 18.;
                    } else {
                        const double p0 = mtype == 2 ? 1. : 0.66666666666666666667;
                        const double p1 = mtype == 2 ? 0. : 0.16666666666666666667;
                        const double pts[3][3] = {{p0, p1, p1}, {p1, p1, p0}, {p1, p0, p1}};
                        for (int i = 0; i < 9; i++) s.h[i] = 0.;
                        for (int g = 0; g < 3; g++)
                            for (int i = 0; i < 3; i++)
                                for (int j = 0; j < 3; j++)
                                    s.h[3 * i + j] += pts[g][i] * pts[g][j] * detJ * (0.5 * 0.33333333333333333333);
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
                    s.valid = 1;
                }
            }
        }
        __syncthreads();
        const int nel = (int)((a.E - e0) < TM ? (a.E - e0) : TM);
        // in batches of 8 slots per thread: the caller's values first (all
        // loads in flight), then the stores
        for (int i0 = tid; i0 < nel * size; i0 += 8 * RNT) {
            double old[8];
#pragma unroll
            for (int u = 0; u < 8; u++) {
                const int i = i0 + u * RNT, el = i / size;
                old[u] = (i < nel * size && se[el].valid) ? a.Kv[se[el].init_k + (i - el * size)] : 0.;
            }
#pragma unroll
            for (int u = 0; u < 8; u++) {
                const int i = i0 + u * RNT;
                if (i >= nel * size) break;
                const int el = i / size, j = i - el * size;
                const T3MElem &s = se[el];
                if (!s.valid) continue;
                const int row = j / ncol, jj = j - row * ncol;
                const int na = row / 6, mm = row % 6;
                int nb, nn;
                if (mtype == 2) {
                    nb = jj / 3;
                    nn = (mm < 3 ? 0 : 3) + jj % 3;
                } else {
                    nb = jj / 5;
                    const int q = jj % 5, skip = (mm + 3) % 6;
                    nn = q + (q >= skip ? 1 : 0);
                }
                const long long k = s.init_k + j;
                a.Kv[k] = old[u] + s.h[3 * na + nb] * s.G[6 * mm + nn];
                a.Kr[k] = s.c[na] + mm;
                a.Kc[k] = s.c[nb] + nn;
            }
        }
    }
}

inline int rs_grid(int64_t E, int per_block, int per_sm) {
    int64_t g = (E + per_block - 1) / per_block;
    const int64_t cap = (int64_t)kSMs * per_sm;
    if (g > cap) g = cap;
    if (g < 1) g = 1;
    return (int)g;
}

template <int NN>
int launch_rs_kc0(const RSArgs &a, cudaStream_t st) {
    using Tl = RSTile<NN>;
    static bool attr = false;
    static int per_sm = 1;  // resident blocks per SM (registers and shared memory)
    if (!attr) {
        FE3D_CUDA(cudaFuncSetAttribute(rs_kc0_kernel<NN>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)Tl::smem));
        int n = 0;
        FE3D_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, rs_kc0_kernel<NN>, RNT, Tl::smem));
        per_sm = n > 0 ? n : 1;
        attr = true;
    }
    rs_kc0_kernel<NN><<<rs_grid(a.E, Tl::TE, per_sm), RNT, Tl::smem, st>>>(a);
    FE3D_CHECK_LAUNCH();
    return FE3D_OK;
}

int rs_check_common(int64_t E, const int64_t *cdof, const double *x, const double *xmat, int xmat_stride,
                    const double *R, const double *m, const double *xe, const double *area, const double *props,
                    int64_t nprops, const double *k6rot, int k6rot_stride) {
    if (!cdof || !props || nprops <= 0 || !k6rot) return FE3D_ERR_ARG;
    if (k6rot_stride != 0 && k6rot_stride != 1) return FE3D_ERR_ARG;
    if (!x && (!R || !m || !xe || !area)) return FE3D_ERR_ARG;
    if (xmat && xmat_stride != 0 && xmat_stride != 3) return FE3D_ERR_ARG;
    (void)E;
    return FE3D_OK;
}

}  // namespace
}  // namespace fe3d

using namespace fe3d;

extern "C" int fe3d_tria3r_frame(int64_t E, const int64_t *cdof, const double *x, int64_t nx, const double *xmat,
                                 int xmat_stride, double *R, double *m, double *xe, double *area, int *err,
                                 void *stream) {
    if (E < 0) return FE3D_ERR_ARG;
    if (E == 0) return FE3D_OK;
    if (!cdof || !x) return FE3D_ERR_ARG;
    if (xmat && xmat_stride != 0 && xmat_stride != 3) return FE3D_ERR_ARG;
    t3_frame_kernel<<<(unsigned)((E + 127) / 128), 128, 0, as_stream(stream)>>>(E, cdof, x, nx, xmat, xmat_stride,
                                                                               nullptr, R, m, xe, area, err);
    FE3D_CHECK_LAUNCH();
    return FE3D_OK;
}

extern "C" int fe3d_tria3r_probe_xe(int64_t E, const int64_t *cdof, const double *x, int64_t nx, const double *R,
                                    double *xe, double *area, int *err, void *stream) {
    if (E < 0) return FE3D_ERR_ARG;
    if (E == 0) return FE3D_OK;
    if (!cdof || !x || !R) return FE3D_ERR_ARG;
    t3_frame_kernel<<<(unsigned)((E + 127) / 128), 128, 0, as_stream(stream)>>>(E, cdof, x, nx, nullptr, 0, R,
                                                                               nullptr, nullptr, xe, area, err);
    FE3D_CHECK_LAUNCH();
    return FE3D_OK;
}

extern "C" int fe3d_tria3r_probe_ue(int64_t E, const int64_t *cdof, const double *u, int64_t nu, const double *R,
                                    double *ue, int *err, void *stream) {
    if (E < 0) return FE3D_ERR_ARG;
    if (E == 0) return FE3D_OK;
    if (!cdof || !u || !R || !ue) return FE3D_ERR_ARG;
    probe_ue_kernel<3><<<(unsigned)((E + 127) / 128), 128, 0, as_stream(stream)>>>(E, cdof, u, nu, R, ue, err);
    FE3D_CHECK_LAUNCH();
    return FE3D_OK;
}

extern "C" int fe3d_tria3r_kc0(int64_t E, const int64_t *cdof, const int64_t *init_k, const double *x, int64_t nx,
                               const double *xmat, int xmat_stride, const double *R, const double *m,
                               const double *xe, const double *area, const double *props, int64_t nprops,
                               const int32_t *pid, const double *k6rot, int k6rot_stride, const double *alpha,
                               int alpha_stride, int64_t *Kr, int64_t *Kc, double *Kv, int64_t nk, int values_only,
                               int *err, void *stream) {
    if (E < 0) return FE3D_ERR_ARG;
    if (E == 0) return FE3D_OK;
    int rc = rs_check_common(E, cdof, x, xmat, xmat_stride, R, m, xe, area, props, nprops, k6rot, k6rot_stride);
    if (rc) return rc;
    if (!init_k || !Kv || !alpha || (alpha_stride != 0 && alpha_stride != 1)) return FE3D_ERR_ARG;
    if (!values_only && (!Kr || !Kc)) return FE3D_ERR_ARG;
    RSArgs a{E, cdof, init_k, x, nx, xmat, xmat_stride, R, m, xe, area, props, nprops, pid, k6rot, k6rot_stride,
             alpha, alpha_stride, Kr, Kc, Kv, nk, values_only, err};
    return launch_rs_kc0<3>(a, as_stream(stream));
}

extern "C" int fe3d_quad4r_kc0(int64_t E, const int64_t *cdof, const int64_t *init_k, const double *x, int64_t nx,
                               const double *xmat, int xmat_stride, const double *R, const double *m,
                               const double *xe, const double *area, const double *props, int64_t nprops,
                               const int32_t *pid, const double *k6rot, int k6rot_stride, const double *hgfactors,
                               int hg_stride, int64_t *Kr, int64_t *Kc, double *Kv, int64_t nk, int values_only,
                               int *err, void *stream) {
    if (E < 0) return FE3D_ERR_ARG;
    if (E == 0) return FE3D_OK;
    int rc = rs_check_common(E, cdof, x, xmat, xmat_stride, R, m, xe, area, props, nprops, k6rot, k6rot_stride);
    if (rc) return rc;
    if (!init_k || !Kv || (hgfactors && hg_stride != 0 && hg_stride != 5)) return FE3D_ERR_ARG;
    if (!values_only && (!Kr || !Kc)) return FE3D_ERR_ARG;
    RSArgs a{E, cdof, init_k, x, nx, xmat, xmat_stride, R, m, xe, area, props, nprops, pid, k6rot, k6rot_stride,
             hgfactors, hg_stride, Kr, Kc, Kv, nk, values_only, err};
    return launch_rs_kc0<4>(a, as_stream(stream));
}

extern "C" int fe3d_tria3r_finte(int64_t E, const int64_t *cdof, const double *R, const double *m, const double *xe,
                                 const double *area, const double *ue, const double *props, int64_t nprops,
                                 const int32_t *pid, const double *k6rot, int k6rot_stride, const double *alpha,
                                 int alpha_stride, double *fint, int64_t nf, double *finte, int *err, void *stream) {
    if (E < 0) return FE3D_ERR_ARG;
    if (E == 0) return FE3D_OK;
    int rc = rs_check_common(E, cdof, nullptr, nullptr, 0, R, m, xe, area, props, nprops, k6rot, k6rot_stride);
    if (rc) return rc;
    if (!ue || (!fint && !finte) || !alpha || (alpha_stride != 0 && alpha_stride != 1)) return FE3D_ERR_ARG;
    RSArgs a{E, cdof, nullptr, nullptr, 0, nullptr, 0, R, m, xe, area, props, nprops, pid, k6rot, k6rot_stride,
             alpha, alpha_stride, nullptr, nullptr, nullptr, INT64_MAX, 1, err};
    rs_fint_kernel<3><<<rs_grid(E, RNT / 9, 4), RNT, 0, as_stream(stream)>>>(a, ue, fint, nf, finte);
    FE3D_CHECK_LAUNCH();
    return FE3D_OK;
}

extern "C" int fe3d_quad4r_finte(int64_t E, const int64_t *cdof, const double *R, const double *m, const double *xe,
                                 const double *area, const double *ue, const double *props, int64_t nprops,
                                 const int32_t *pid, const double *k6rot, int k6rot_stride, const double *hgfactors,
                                 int hg_stride, double *fint, int64_t nf, double *finte, int *err, void *stream) {
    if (E < 0) return FE3D_ERR_ARG;
    if (E == 0) return FE3D_OK;
    int rc = rs_check_common(E, cdof, nullptr, nullptr, 0, R, m, xe, area, props, nprops, k6rot, k6rot_stride);
    if (rc) return rc;
    if (!ue || (!fint && !finte) || (hgfactors && hg_stride != 0 && hg_stride != 5)) return FE3D_ERR_ARG;
    RSArgs a{E, cdof, nullptr, nullptr, 0, nullptr, 0, R, m, xe, area, props, nprops, pid, k6rot, k6rot_stride,
             hgfactors, hg_stride, nullptr, nullptr, nullptr, INT64_MAX, 1, err};
    rs_fint_kernel<4><<<rs_grid(E, RNT / 16, 4), RNT, 0, as_stream(stream)>>>(a, ue, fint, nf, finte);
    FE3D_CHECK_LAUNCH();
    return FE3D_OK;
}

extern "C" int fe3d_tria3r_kg(int64_t E, const int64_t *cdof, const int64_t *init_k, const double *x, int64_t nx,
                              const double *xmat, int xmat_stride, const double *u, int64_t nu, const double *R,
                              const double *m, const double *xe, const double *area, const double *ue,
                              const double *props, int64_t nprops, const int32_t *pid, int64_t *Kr, int64_t *Kc,
                              double *Kv, int64_t nk, int values_only, int *err, void *stream) {
    if (E < 0) return FE3D_ERR_ARG;
    if (E == 0) return FE3D_OK;
    if (!cdof || !init_k || !props || nprops <= 0 || !Kv) return FE3D_ERR_ARG;
    if (!values_only && (!Kr || !Kc)) return FE3D_ERR_ARG;
    if (x && !u) return FE3D_ERR_ARG;
    if (!x && (!R || !m || !xe || !area || !ue)) return FE3D_ERR_ARG;
    if (xmat && xmat_stride != 0 && xmat_stride != 3) return FE3D_ERR_ARG;
    RSArgs a{E, cdof, init_k, x, nx, xmat, xmat_stride, R, m, xe, area, props, nprops, pid, nullptr, 0,
             nullptr, 0, Kr, Kc, Kv, nk, values_only, err};
    t3_kg_kernel<<<rs_grid(E, RNT, 4), RNT, 0, as_stream(stream)>>>(a, u, nu, ue, nullptr, 0);
    FE3D_CHECK_LAUNCH();
    return FE3D_OK;
}

extern "C" int fe3d_tria3r_kg_given_stress(int64_t E, const int64_t *cdof, const int64_t *init_k, const double *x,
                                           int64_t nx, const double *R, const double *xe, const double *area,
                                           const double *nstress, int nstress_stride, int64_t *Kr, int64_t *Kc,
                                           double *Kv, int64_t nk, int values_only, int *err, void *stream) {
    if (E < 0) return FE3D_ERR_ARG;
    if (E == 0) return FE3D_OK;
    if (!cdof || !init_k || !nstress || !Kv) return FE3D_ERR_ARG;
    if (nstress_stride != 0 && nstress_stride != 3) return FE3D_ERR_ARG;
    if (!values_only && (!Kr || !Kc)) return FE3D_ERR_ARG;
    if (!x && (!R || !xe || !area)) return FE3D_ERR_ARG;
    RSArgs a{E, cdof, init_k, x, nx, nullptr, 0, R, nullptr, xe, area, nullptr, 0, nullptr, nullptr, 0,
             nullptr, 0, Kr, Kc, Kv, nk, values_only, err};
    t3_kg_kernel<<<rs_grid(E, RNT, 4), RNT, 0, as_stream(stream)>>>(a, nullptr, 0, nullptr, nstress,
                                                                     nstress_stride);
    FE3D_CHECK_LAUNCH();
    return FE3D_OK;
}

extern "C" int fe3d_tria3r_m(int64_t E, const int64_t *cdof, const int64_t *init_k, const double *x, int64_t nx,
                             const double *R, const double *area, const double *props, int64_t nprops,
                             const int32_t *pid, int64_t *Kr, int64_t *Kc, double *Kv, int64_t nk, int mtype, int *err,
                             void *stream) {
    if (E < 0) return FE3D_ERR_ARG;
    if (mtype < 0 || mtype > 2) return FE3D_ERR_ARG;
    if (E == 0) return FE3D_OK;
    if (!cdof || !init_k || !props || nprops <= 0 || !Kr || !Kc || !Kv) return FE3D_ERR_ARG;
    if (!x && (!R || !area)) return FE3D_ERR_ARG;
    RSArgs a{E, cdof, init_k, x, nx, nullptr, 0, R, nullptr, nullptr, area, props, nprops, pid, nullptr, 0,
             nullptr, 0, Kr, Kc, Kv, nk, 0, err};
    t3_m_kernel<<<rs_grid(E, 32, 8), RNT, 0, as_stream(stream)>>>(a, mtype);
    FE3D_CHECK_LAUNCH();
    return FE3D_OK;
}
