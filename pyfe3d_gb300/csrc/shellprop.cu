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

}  // namespace
}  // namespace fe3d

using namespace fe3d;

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
