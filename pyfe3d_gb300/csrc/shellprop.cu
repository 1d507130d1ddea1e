// Isotropic ShellProp records built on the device, one thread per record:
// shellprop_utils.isotropic_plate (pyfe3d/shellprop_utils.py) -> the
// single-ply laminate integration of shellprop.pyx:568-621 with the lamina
// stiffness of shellprop.pyx:278-341 (a 0-degree ply) and the shear
// correction of shellprop.pyx:485-549, so per-element property fields
// (thickness, modulus, density per element) need no host-side record
// construction.  Inputs are arrays with stride 1 or broadcast scalars
// (stride 0).
#include "common.cuh"

namespace fe3d {
namespace {

__global__ void isotropic_records_kernel(int64_t n, const double *h_, int sh, const double *E_, int sE,
                                         const double *nu_, int snu, const double *rho_, int srho,
                                         const double *off_, int soff, int calc_scf, double *rec) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double h = h_[sh * i], E = E_[sE * i], nu = nu_[snu * i];
    const double rho = rho_ ? rho_[srho * i] : 0., offset = off_ ? off_[soff * i] : 0.;
    const double g = E / (2. * (1. + nu));
    const double nu21 = nu * E / E;
    const double q11 = E / (1. - nu * nu21), q12 = nu * E / (1. - nu * nu21), q22 = E / (1. - nu * nu21);
    // a single ply at 0 degrees (cos = 1, sin = 0)
    const double q[6] = {q11, q12, 0., q22, 0., g};
    const double hk_1 = -h / 2. + offset, hk = hk_1 + h;
    const double d1 = hk - hk_1, d2 = hk * hk - hk_1 * hk_1, d3 = hk * hk * hk - hk_1 * hk_1 * hk_1;
    double *r = rec + (int64_t)SP_STRIDE * i;
    for (int k = 0; k < 6; k++) {
        r[k] = q[k] * d1;
        r[6 + k] = 0.5 * q[k] * d2;
        r[12 + k] = q[k] * d3 / 3.;
    }
    r[SP_E44] = g * d1;
    r[SP_E45] = 0.;
    r[SP_E55] = g * d1;
    if (calc_scf) {
        const double zbot = -h / 2. + offset, z1 = zbot, z2 = zbot + h;
        const double D1 = E / (1. - nu * nu21);
        const double poly = 15. * offset * z1 * z1 * z1 * z1 + 30. * offset * z1 * z1 * zbot * (2. * offset - zbot) -
                            15. * offset * z2 * z2 * z2 * z2 + 30. * offset * z2 * z2 * zbot * (-2. * offset + zbot) -
                            3. * z1 * z1 * z1 * z1 * z1 +
                            10. * z1 * z1 * z1 * (-2. * offset * offset - 2. * offset * zbot + zbot * zbot) -
                            15. * z1 * zbot * zbot * (4. * offset * offset - 4. * offset * zbot + zbot * zbot) +
                            3. * z2 * z2 * z2 * z2 * z2 +
                            10. * z2 * z2 * z2 * (2. * offset * offset + 2. * offset * zbot - zbot * zbot) +
                            15. * z2 * zbot * zbot * (4. * offset * offset - 4. * offset * zbot + zbot * zbot);
        const double a1 = z2 - offset, a0 = z1 - offset;
        const double R1 = D1 * (a1 * a1 * a1 / 3. - a0 * a0 * a0 / 3.);
        const double den1 = g * h * (h / h) * D1 * D1 * poly / (60. * g);
        const double scf = R1 * R1 / den1;
        r[SP_SCF13] = scf;
        r[SP_SCF23] = scf;
    } else {
        r[SP_SCF13] = 5. / 6.;
        r[SP_SCF23] = 5. / 6.;
    }
    r[SP_H] = h;
    r[SP_H + 1] = rho * d1;
    r[SP_H + 2] = rho * (hk * hk / 2. - hk_1 * hk_1 / 2.);
    r[SP_H + 3] = rho * (hk * hk * hk / 3. - hk_1 * hk_1 * hk_1 / 3.);
    for (int k = SP_H + 4; k < SP_STRIDE; k++) r[k] = 0.;
}

// Laminated records, one thread per record: for every ply the lamina
// stiffness (shellprop_utils.read_laminaprop and MatLamina.rebuild,
// pyfe3d/shellprop_utils.py:13-93, shellprop.pyx:128-196) turned to the ply
// angle (Lamina.rebuild, shellprop.pyx:278-341), the ply integration of ABD,
// E and the density integrals (ShellProp.calc_constitutive_matrix,
// shellprop.pyx:568-621) and the Vlachoutsis shear correction
// (ShellProp.calc_scf, shellprop.pyx:485-549), in the reference's order of
// operations.  Ply data: angle (degrees), thickness, density and the six
// lamina constants E11 E22 nu12 G12 G13 G23; each array holds one stack
// shared by every record (record stride 0) or one stack per record.
__global__ void laminate_records_kernel(int64_t n, int nply, const double *theta, int64_t th_rs,
                                        const double *plyt, int64_t pt_rs, const double *lam, int64_t lam_rs,
                                        const double *rho_, int64_t rho_rs, const double *off_, int64_t off_rs,
                                        int calc_scf, double *rec) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double *th = theta + th_rs * i, *pt = plyt + pt_rs * i, *lp = lam + lam_rs * i;
    const double *rh = rho_ ? rho_ + rho_rs * i : nullptr;
    const double offset = off_ ? off_[off_rs * i] : 0.;
    const double pi = 4. * atan(1.);
    double h = 0.;
    for (int k = 0; k < nply; k++) h += pt[k];
    double acc[21];
    for (int k = 0; k < 21; k++) acc[k] = 0.;
    double rho0 = 0., rho1 = 0., rho2 = 0.;
    double h0 = -h / 2. + offset;
    for (int k = 0; k < nply; k++) {
        const double *L = lp + 6 * k;
        const double e1 = L[0], e2 = L[1], nu12 = L[2], g12 = L[3], g13 = L[4], g23 = L[5];
        const double nu21 = nu12 * e2 / e1;
        const double t = th[k] * pi / 180.;
        const double c = cos(t), sn = sin(t);
        const double c2 = c * c, c3 = c2 * c, c4 = c3 * c, s2 = sn * sn, s3 = s2 * sn, s4 = s3 * sn;
        const double q11 = e1 / (1. - nu12 * nu21), q12 = nu12 * e2 / (1. - nu12 * nu21),
                     q22 = e2 / (1. - nu12 * nu21), q44 = g23, q55 = g13, q66 = g12;
        double q[9];
        q[0] = q11 * c4 + 2. * (q12 + 2. * q66) * s2 * c2 + q22 * s4;                        // 11
        q[1] = (q11 + q22 - 4. * q66) * s2 * c2 + q12 * (s4 + c4);                          // 12
        q[2] = (q11 - q12 - 2. * q66) * sn * c3 + (q12 - q22 + 2. * q66) * s3 * c;            // 16
        q[3] = q11 * s4 + 2. * (q12 + 2. * q66) * s2 * c2 + q22 * c4;                        // 22
        q[4] = (q11 - q12 - 2. * q66) * s3 * c + (q12 - q22 + 2. * q66) * sn * c3;            // 26
        q[5] = (q11 + q22 - 2. * q12 - 2. * q66) * s2 * c2 + q66 * (s4 + c4);                // 66
        q[6] = q44 * c2 + q55 * s2;                                                           // 44
        q[7] = (q55 - q44) * sn * c;                                                          // 45
        q[8] = q55 * c2 + q44 * s2;                                                           // 55
        const double hk_1 = h0;
        h0 += pt[k];
        const double hk = h0;
        const double r = rh ? rh[k] : 0.;
        rho0 += r * (hk - hk_1);
        rho1 += r * (hk * hk / 2. - hk_1 * hk_1 / 2.);
        rho2 += r * (hk * hk * hk / 3. - hk_1 * hk_1 * hk_1 / 3.);
        const double d1 = hk - hk_1, d2 = hk * hk - hk_1 * hk_1, d3 = hk * hk * hk - hk_1 * hk_1 * hk_1;
        for (int m = 0; m < 6; m++) {
            acc[m] += q[m] * d1;
            acc[6 + m] += 1. / 2. * q[m] * d2;
            acc[12 + m] += 1. / 3. * q[m] * d3;
        }
        acc[18] += q[6] * d1;
        acc[19] += q[7] * d1;
        acc[20] += q[8] * d1;
    }
    double *o = rec + (int64_t)SP_STRIDE * i;
    for (int k = 0; k < 21; k++) o[k] = acc[k];
    double k13 = 5. / 6., k23 = 5. / 6.;
    if (calc_scf) {
        double D1 = 0., R1 = 0., den1 = 0., D2 = 0., R2 = 0., den2 = 0.;
        const double zbot = -h / 2. + offset;
        double z1 = zbot;
        for (int k = 0; k < nply; k++) {
            const double *L = lp + 6 * k;
            const double E1 = L[0], E2 = L[1], n12 = L[2], g13 = L[4], g23 = L[5];
            const double n21 = n12 * E2 / E1;
            const double z2 = z1 + pt[k];
            const double t = th[k] * pi / 180.;
            const double ct = cos(t), st = sin(t);
            const double e1 = E1 * ct + E2 * st, e2 = E2 * ct + E1 * st;
            const double nu12 = n12 * ct + n21 * st, nu21 = n21 * ct + n12 * st;
            const double poly = 15. * offset * z1 * z1 * z1 * z1 + 30. * offset * z1 * z1 * zbot * (2. * offset - zbot) -
                                15. * offset * z2 * z2 * z2 * z2 + 30. * offset * z2 * z2 * zbot * (-2. * offset + zbot) -
                                3. * z1 * z1 * z1 * z1 * z1 +
                                10. * z1 * z1 * z1 * (-2. * offset * offset - 2. * offset * zbot + zbot * zbot) -
                                15. * z1 * zbot * zbot * (4. * offset * offset - 4. * offset * zbot + zbot * zbot) +
                                3. * z2 * z2 * z2 * z2 * z2 +
                                10. * z2 * z2 * z2 * (2. * offset * offset + 2. * offset * zbot - zbot * zbot) +
                                15. * z2 * zbot * zbot * (4. * offset * offset - 4. * offset * zbot + zbot * zbot);
            const double a1 = z2 - offset, a0 = z1 - offset;
            D1 += e1 / (1. - nu12 * nu21);
            R1 += D1 * (a1 * a1 * a1 / 3. - a0 * a0 * a0 / 3.);
            den1 += g13 * pt[k] * (h / pt[k]) * D1 * D1 * poly / (60. * g13);
            D2 += e2 / (1. - nu12 * nu21);
            R2 += D2 * (a1 * a1 * a1 / 3. - a0 * a0 * a0 / 3.);
            den2 += g23 * pt[k] * (h / pt[k]) * D2 * D2 * poly / (60. * g23);
            z1 = z2;
        }
        k13 = R1 * R1 / den1;
        k23 = R2 * R2 / den2;
    }
    o[SP_SCF13] = k13;
    o[SP_SCF23] = k23;
    o[SP_H] = h;
    o[SP_H + 1] = rho0;
    o[SP_H + 2] = rho1;
    o[SP_H + 3] = rho2;
    for (int k = SP_H + 4; k < SP_STRIDE; k++) o[k] = 0.;
}

}  // namespace
}  // namespace fe3d

using namespace fe3d;

extern "C" int fe3d_laminate_records(int64_t n, int nply, const double *theta, int64_t theta_rs, const double *plyt,
                                     int64_t plyt_rs, const double *lam, int64_t lam_rs, const double *rho,
                                     int64_t rho_rs, const double *offset, int64_t offset_rs, int calc_scf,
                                     double *records, void *stream) {
    if (n < 0 || nply < 1) return FE3D_ERR_ARG;
    if (n == 0) return FE3D_OK;
    if (!theta || !plyt || !lam || !records) return FE3D_ERR_ARG;
    if ((theta_rs != 0 && theta_rs < nply) || (plyt_rs != 0 && plyt_rs < nply) ||
        (lam_rs != 0 && lam_rs < 6 * (int64_t)nply) || (rho && rho_rs != 0 && rho_rs < nply) ||
        (offset && offset_rs != 0 && offset_rs != 1))
        return FE3D_ERR_ARG;
    laminate_records_kernel<<<(unsigned)((n + 127) / 128), 128, 0, as_stream(stream)>>>(
        n, nply, theta, theta_rs, plyt, plyt_rs, lam, lam_rs, rho, rho_rs, offset, offset_rs, calc_scf, records);
    FE3D_CHECK_LAUNCH();
    return FE3D_OK;
}

extern "C" int fe3d_isotropic_plate_records(int64_t n, const double *h, int h_stride, const double *E,
                                            int E_stride, const double *nu, int nu_stride, const double *rho,
                                            int rho_stride, const double *offset, int offset_stride,
                                            int calc_scf, double *records, void *stream) {
    if (n < 0) return FE3D_ERR_ARG;
    if (n == 0) return FE3D_OK;
    if (!h || !E || !nu || !records) return FE3D_ERR_ARG;
    for (int s : {h_stride, E_stride, nu_stride, rho_stride, offset_stride})
        if (s != 0 && s != 1) return FE3D_ERR_ARG;
    isotropic_records_kernel<<<(unsigned)((n + 255) / 256), 256, 0, as_stream(stream)>>>(
        n, h, h_stride, E, E_stride, nu, nu_stride, rho, rho_stride, offset, offset_stride, calc_scf, records);
    FE3D_CHECK_LAUNCH();
    return FE3D_OK;
}
