/*
 * fe3d_oracle.c -- CPU oracle for the pyfe3d element-assembly path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker: tests, the smoke
 * check and the CPU-baseline leg of the benchmark load it to compare the
 * CUDA library against.  The product path (pyfe3d_gb300) never links,
 * imports or calls it.
 *
 * It is a plain FP64 restatement of the reference's per-element algorithms,
 * written in the same order of operations as the reference wherever that
 * order matters for rounding (the 24x24 Gauss-point loops of Quad4 KC0, the
 * element-to-global transformation Kg = R Ke R^T).  Every function cites the
 * reference routine it restates (paths are relative to the pyfe3d project).
 * The restatement is pinned against fixtures produced by running the
 * reference itself (tests/golden/make_golden.py).
 *
 * Property records are flat double arrays:
 *   shell (Q4P_STRIDE=28): A11 A12 A16 A22 A26 A66 B11 B12 B16 B22 B26 B66
 *                          D11 D12 D16 D22 D26 D66 E44 E45 E55 scf_k13
 *                          scf_k23 h intrho intrhoz intrhoz2 (pad)
 *   beam (BCP_STRIDE=16):  A E G Iyy Izz Iyz J Ay Az intrho intrhoy intrhoz
 *                          intrhoy2 intrhoz2 intrhoyz (pad)
 */
#include <math.h>
#include <stdint.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define Q4P_STRIDE 28
#define BCP_STRIDE 16

enum { P_A11, P_A12, P_A16, P_A22, P_A26, P_A66, P_B11, P_B12, P_B16, P_B22,
       P_B26, P_B66, P_D11, P_D12, P_D16, P_D22, P_D26, P_D66, P_E44, P_E45,
       P_E55, P_SCF13, P_SCF23, P_H, P_RHO, P_RHOZ, P_RHOZ2 };
enum { BP_A, BP_E, BP_G, BP_IYY, BP_IZZ, BP_IYZ, BP_J, BP_AY, BP_AZ, BP_RHO,
       BP_RHOY, BP_RHOZ, BP_RHOY2, BP_RHOZ2, BP_RHOYZ };

static const double GP = 0.5773502691896257645092;

/* ------------------------------------------------------------------ */
/* Quad4 frame: pyfe3d/quad4.pyx:491-624 (update_rotation_matrix).      */
/* R is row-major r11 r12 r13 r21 ... r33; m = m11 m12 m21 m22 is       */
/* in/out: it is only overwritten when the material vector projects.    */
/* ------------------------------------------------------------------ */
void orc_q4_rotation(const double *x, const int64_t *c, const double *xmat,
                     double *R, double *m)
{
    const double *p1 = x + c[0] / 2, *p2 = x + c[1] / 2, *p3 = x + c[2] / 2,
                 *p4 = x + c[3] / 2;
    double v13[3], v42[3], z[3], xa[3], y[3], t;
    for (int i = 0; i < 3; i++) { v13[i] = p3[i] - p1[i]; v42[i] = p2[i] - p4[i]; }
    z[0] = v42[1] * v13[2] - v42[2] * v13[1];
    z[1] = -v42[0] * v13[2] + v42[2] * v13[0];
    z[2] = v42[0] * v13[1] - v42[1] * v13[0];
    t = sqrt(z[0] * z[0] + z[1] * z[1] + z[2] * z[2]);
    for (int i = 0; i < 3; i++) z[i] /= t;
    double tol = t / 1e10;
    for (int i = 0; i < 3; i++) xa[i] = (v13[i] + v42[i]) / 2.;
    t = sqrt(xa[0] * xa[0] + xa[1] * xa[1] + xa[2] * xa[2]);
    for (int i = 0; i < 3; i++) xa[i] /= t;
    y[0] = z[1] * xa[2] - z[2] * xa[1];
    y[1] = z[2] * xa[0] - z[0] * xa[2];
    y[2] = z[0] * xa[1] - z[1] * xa[0];
    t = sqrt(y[0] * y[0] + y[1] * y[1] + y[2] * y[2]);
    for (int i = 0; i < 3; i++) y[i] /= t;
    for (int i = 0; i < 3; i++) { R[3 * i + 0] = xa[i]; R[3 * i + 1] = y[i]; R[3 * i + 2] = z[i]; }
    if (!xmat) return;
    double xm[3] = {xmat[0], xmat[1], xmat[2]}, ym[3];
    double xn = sqrt(xm[0] * xm[0] + xm[1] * xm[1] + xm[2] * xm[2]);
    for (int i = 0; i < 3; i++) xm[i] /= xn;
    if (xn > tol) {
        ym[0] = z[1] * xm[2] - z[2] * xm[1];
        ym[1] = z[2] * xm[0] - z[0] * xm[2];
        ym[2] = z[0] * xm[1] - z[1] * xm[0];
        t = sqrt(ym[0] * ym[0] + ym[1] * ym[1] + ym[2] * ym[2]);
        for (int i = 0; i < 3; i++) ym[i] /= t;
        if (t > tol) {
            xm[0] = ym[1] * z[2] - ym[2] * z[1];
            xm[1] = ym[2] * z[0] - ym[0] * z[2];
            xm[2] = ym[0] * z[1] - ym[1] * z[0];
            t = sqrt(xm[0] * xm[0] + xm[1] * xm[1] + xm[2] * xm[2]);
            for (int i = 0; i < 3; i++) xm[i] /= t;
            double cth = xm[0] * xa[0] + xm[1] * xa[1] + xm[2] * xa[2];
            m[0] = cth; m[3] = cth;
            if (xm[0] * y[0] + xm[1] * y[1] + xm[2] * y[2] > 0) m[1] = -sqrt(1 - cth * cth);
            else m[1] = sqrt(1 - cth * cth);
            m[2] = -m[1];
        }
    }
}

/* pyfe3d/quad4.pyx:682-752 (update_probe_xe + update_area) */
void orc_q4_probe_xe(const double *x, const int64_t *c, const double *R,
                     double *xe, double *area)
{
    for (int j = 0; j < 4; j++) {
        const double *p = x + c[j] / 2;
        for (int k = 0; k < 3; k++) {
            double s = 0;
            for (int i = 0; i < 3; i++) s += R[3 * i + k] * p[i];
            xe[3 * j + k] = s;
        }
    }
    double x1 = xe[0], y1 = xe[1], x2 = xe[3], y2 = xe[4], x3 = xe[6], y3 = xe[7],
           x4 = xe[9], y4 = xe[10];
    *area = 0.5 * fabs((x1 * y2 + x2 * y3 + x3 * y4 + x4 * y1) -
                       (x2 * y1 + x3 * y2 + x4 * y3 + x1 * y4));
}

/* pyfe3d/quad4.pyx:627-679 (update_probe_ue); also BeamC with nn=2 */
static void probe_ue_n(int nn, const double *u, const int64_t *c, const double *R,
                       double *ue)
{
    for (int j = 0; j < nn; j++) {
        for (int g = 0; g < 2; g++) {
            const double *p = u + c[j] + 3 * g;
            for (int k = 0; k < 3; k++) {
                double s = 0;
                for (int i = 0; i < 3; i++) s += R[3 * i + k] * p[i];
                ue[6 * j + 3 * g + k] = s;
            }
        }
    }
}
void orc_q4_probe_ue(const double *u, const int64_t *c, const double *R, double *ue)
{
    probe_ue_n(4, u, c, R, ue);
}

/* ABD rotation to the element axes, quad4.pyx:845-899: X' = T X T^T with
 * rows a=(m11^2, m12^2, 2 m11 m12), b=(m21^2, m22^2, 2 m21 m22),
 * c=(m11 m21, m12 m22, m11 m22 + m12 m21). */
static void rot3(const double *m, double X11, double X12, double X16, double X22,
                 double X26, double X66, double *out /* 11 12 16 22 26 66 */)
{
    double T[3][3] = {{m[0] * m[0], m[1] * m[1], 2 * m[0] * m[1]},
                      {m[2] * m[2], m[3] * m[3], 2 * m[2] * m[3]},
                      {m[0] * m[2], m[1] * m[3], m[0] * m[3] + m[1] * m[2]}};
    double X[3][3] = {{X11, X12, X16}, {X12, X22, X26}, {X16, X26, X66}};
    double Y[3][3];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            double s = 0;
            for (int k = 0; k < 3; k++)
                for (int l = 0; l < 3; l++) s += T[i][k] * X[k][l] * T[j][l];
            Y[i][j] = s;
        }
    out[0] = Y[0][0]; out[1] = Y[1][0]; out[2] = Y[2][0];
    out[3] = Y[1][1]; out[4] = Y[2][1]; out[5] = Y[2][2];
}

static void shape_derivs(const double *xe, double xi, double eta, double *detJ,
                         double *N, double *Nx, double *Ny)
{
    double x1 = xe[0], y1 = xe[1], x2 = xe[3], y2 = xe[4], x3 = xe[6], y3 = xe[7],
           x4 = xe[9], y4 = xe[10];
    double J11 = -0.5 * x1 + 0.5 * x2 + 0.5 * (eta + 1) * (0.5 * x1 - 0.5 * x2 + 0.5 * x3 - 0.5 * x4);
    double J12 = -0.5 * y1 + 0.5 * y2 + 0.5 * (eta + 1) * (0.5 * y1 - 0.5 * y2 + 0.5 * y3 - 0.5 * y4);
    double J21 = -0.5 * x1 + 0.5 * x4 - 0.25 * (-x1 + x2) * (xi + 1) + 0.25 * (x3 - x4) * (xi + 1);
    double J22 = -0.5 * y1 + 0.5 * y4 - 0.25 * (xi + 1) * (-y1 + y2) + 0.25 * (xi + 1) * (y3 - y4);
    double d = J11 * J22 - J12 * J21;
    *detJ = d;
    double j11 = J22 / d, j12 = -J12 / d, j21 = -J21 / d, j22 = J11 / d;
    /* natural derivatives of the bilinear shape functions */
    double dxi[4] = {0.25 * (eta - 1), 0.25 * (1 - eta), 0.25 * (eta + 1), -0.25 * (eta + 1)};
    double det[4] = {0.25 * (xi - 1), -0.25 * (xi + 1), 0.25 * (xi + 1), 0.25 * (1 - xi)};
    double sx[4] = {-1, 1, 1, -1}, sy[4] = {-1, -1, 1, 1};
    for (int a = 0; a < 4; a++) {
        N[a] = 0.25 * (1 + sx[a] * xi) * (1 + sy[a] * eta);
        Nx[a] = j11 * dxi[a] + j12 * det[a];
        Ny[a] = j21 * dxi[a] + j22 * det[a];
    }
}

/* Local 24x24 constitutive stiffness, quad4.pyx:755-1171
 * (_update_probe_KC0ve).  Drilling has unit weight (quad4.pyx:1053-1073). */
void orc_q4_kc0_local(const double *m, const double *xe, double area,
                      const double *P, double *Ke)
{
    double Am[6], Bm[6], Dm[6];
    if (m[1] == 0) {
        for (int i = 0; i < 6; i++) { Am[i] = P[P_A11 + i]; Bm[i] = P[P_B11 + i]; Dm[i] = P[P_D11 + i]; }
    } else {
        rot3(m, P[P_A11], P[P_A12], P[P_A16], P[P_A22], P[P_A26], P[P_A66], Am);
        rot3(m, P[P_B11], P[P_B12], P[P_B16], P[P_B22], P[P_B26], P[P_B66], Bm);
        rot3(m, P[P_D11], P[P_D12], P[P_D16], P[P_D22], P[P_D26], P[P_D66], Dm);
    }
    double ABD[6][6] = {
        {Am[0], Am[1], Am[2], Bm[0], Bm[1], Bm[2]},
        {Am[1], Am[3], Am[4], Bm[1], Bm[3], Bm[4]},
        {Am[2], Am[4], Am[5], Bm[2], Bm[4], Bm[5]},
        {Bm[0], Bm[1], Bm[2], Dm[0], Dm[1], Dm[2]},
        {Bm[1], Bm[3], Bm[4], Dm[1], Dm[3], Dm[4]},
        {Bm[2], Bm[4], Bm[5], Dm[2], Dm[4], Dm[5]}};
    double E44 = P[P_E44] * P[P_SCF23];
    double E45 = P[P_E45] * 0.5 * (P[P_SCF13] + P[P_SCF23]);
    double E55 = P[P_E55] * P[P_SCF13];
    int thick = P[P_H] / sqrt(area) >= 1.;
    memset(Ke, 0, sizeof(double) * 576);
    double N[4], Nx[4], Ny[4], detJ;
    double pts[2] = {-GP, GP};
    for (int pi = 0; pi < 2; pi++)
        for (int pj = 0; pj < 2; pj++) {
            shape_derivs(xe, pts[pi], pts[pj], &detJ, N, Nx, Ny);
            double Bl[6][24], gy[24], gx[24], dr[24];
            memset(Bl, 0, sizeof(Bl)); memset(gy, 0, sizeof(gy));
            memset(gx, 0, sizeof(gx)); memset(dr, 0, sizeof(dr));
            for (int a = 0; a < 4; a++) {
                int o = 6 * a;
                Bl[0][o + 0] = Nx[a];
                Bl[1][o + 1] = Ny[a];
                Bl[2][o + 0] = Ny[a]; Bl[2][o + 1] = Nx[a];
                Bl[3][o + 4] = Nx[a];
                Bl[4][o + 3] = -Ny[a];
                Bl[5][o + 3] = -Nx[a]; Bl[5][o + 4] = Ny[a];
                gy[o + 2] = Ny[a]; gx[o + 2] = Nx[a];
                dr[o + 0] = Ny[a] / 2.; dr[o + 1] = -Nx[a] / 2.; dr[o + 5] = N[a];
            }
            for (int i = 0; i < 24; i++)
                for (int j = 0; j < 24; j++) {
                    double s = 0;
                    for (int p = 0; p < 6; p++)
                        for (int q = 0; q < 6; q++) s += Bl[p][i] * ABD[p][q] * Bl[q][j];
                    Ke[24 * i + j] += detJ * s;
                }
            if (thick)
                for (int i = 0; i < 24; i++)
                    for (int j = 0; j < 24; j++)
                        Ke[24 * i + j] += detJ * (gy[i] * E44 * gy[j] + gy[i] * E45 * gx[j] +
                                                  gx[i] * E45 * gy[j] + gx[i] * E55 * gx[j]);
            for (int i = 0; i < 24; i++)
                for (int j = 0; j < 24; j++) Ke[24 * i + j] += detJ * dr[i] * dr[j];
        }
    /* one-point centre rule for transverse shear, quad4.pyx:1075-1171 */
    shape_derivs(xe, 0., 0., &detJ, N, Nx, Ny);
    double gyg[24], gyr[24], gxg[24], gxr[24];
    memset(gyg, 0, sizeof(gyg)); memset(gyr, 0, sizeof(gyr));
    memset(gxg, 0, sizeof(gxg)); memset(gxr, 0, sizeof(gxr));
    for (int a = 0; a < 4; a++) {
        int o = 6 * a;
        gyg[o + 2] = Ny[a]; gyr[o + 3] = -N[a];
        gxg[o + 2] = Nx[a]; gxr[o + 4] = N[a];
    }
    for (int i = 0; i < 24; i++)
        for (int j = 0; j < 24; j++) {
            double s = 0;
            if (!thick)
                s += gyg[i] * E44 * gyg[j] + gyg[i] * E45 * gxg[j] + gxg[i] * E45 * gyg[j] + gxg[i] * E55 * gxg[j];
            s += gyg[i] * E44 * gyr[j] + gyg[i] * E45 * gxr[j] + gxg[i] * E45 * gyr[j] + gxg[i] * E55 * gxr[j];
            s += gyr[i] * E44 * gyg[j] + gyr[i] * E45 * gxg[j] + gxr[i] * E45 * gyg[j] + gxr[i] * E55 * gxg[j];
            s += gyr[i] * E44 * gyr[j] + gyr[i] * E45 * gxr[j] + gxr[i] * E45 * gyr[j] + gxr[i] * E55 * gxr[j];
            Ke[24 * i + j] += 4. * detJ * s;
        }
}

/* Kg = T Ke T^T with T = blockdiag(R, R, ..), scattered row-major at
 * init_k (quad4.pyx:1278-1313; beamc.pyx:626-1352).  nn = nodes. */
static void scatter_rotated(int nn, const double *R, const double *Ke, const int64_t *c,
                            int64_t init_k, int64_t *Kr, int64_t *Kc, double *Kv,
                            int write_idx)
{
    int n = 6 * nn;
    for (int ni = 0; ni < nn; ni++)
        for (int mm = 0; mm < 6; mm++)
            for (int nj = 0; nj < nn; nj++)
                for (int nn2 = 0; nn2 < 6; nn2++) {
                    int64_t k = init_k + (int64_t)n * (6 * ni + mm) + 6 * nj + nn2;
                    if (write_idx) { Kr[k] = c[ni] + mm; Kc[k] = c[nj] + nn2; }
                    int gm = mm / 3, im = mm % 3, gn = nn2 / 3, in = nn2 % 3;
                    double s = 0;
                    for (int i = 0; i < 3; i++)
                        for (int j = 0; j < 3; j++)
                            s += R[3 * im + i] * Ke[n * (6 * ni + 3 * gm + i) + 6 * nj + 3 * gn + j] * R[3 * in + j];
                    Kv[k] += s;
                }
}

/* pyfe3d/quad4.pyx:1204-1313 (update_KC0) */
void orc_q4_kc0(const double *R, const double *m, const double *xe, double area,
                const double *P, const int64_t *c, int64_t init_k, int64_t *Kr,
                int64_t *Kc, double *Kv, int values_only)
{
    double Ke[576];
    orc_q4_kc0_local(m, xe, area, P, Ke);
    scatter_rotated(4, R, Ke, c, init_k, Kr, Kc, Kv, values_only == 0);
}

/* pyfe3d/quad4.pyx:1174-1201 (update_probe_finte): finte = KC0e ue, local */
void orc_q4_finte(const double *m, const double *xe, double area, const double *P,
                  const double *ue, double *fe)
{
    double Ke[576];
    orc_q4_kc0_local(m, xe, area, P, Ke);
    for (int i = 0; i < 24; i++) {
        double s = 0;
        for (int j = 0; j < 24; j++) s += Ke[24 * i + j] * ue[j];
        fe[i] = s;
    }
}

/* pyfe3d/quad4.pyx:1316-1362 (update_fint): fint[c + .] += R finte */
void orc_q4_fint(const double *R, const double *m, const double *xe, double area,
                 const double *P, const int64_t *c, const double *ue, double *fint)
{
    double fe[24];
    orc_q4_finte(m, xe, area, P, ue, fe);
    for (int a = 0; a < 4; a++)
        for (int g = 0; g < 2; g++)
            for (int i = 0; i < 3; i++) {
                double s = 0;
                for (int j = 0; j < 3; j++) s += fe[6 * a + 3 * g + j] * R[3 * i + j];
                fint[c[a] + 3 * g + i] += s;
            }
}

/* pyfe3d/quad4.pyx:1365-2257 (update_KG): 144 entries, row-major 12x12 over
 * the translational DOFs; value = r_m3 r_n3 (grad N_a . Nmat . grad N_b) detJ */
void orc_q4_kg(const double *R, const double *m, const double *xe, const double *ue,
               const double *P, const int64_t *c, int64_t init_k, int64_t *Kr,
               int64_t *Kc, double *Kv)
{
    double A[6], B[6];
    if (m[1] == 0) {
        for (int i = 0; i < 6; i++) { A[i] = P[P_A11 + i]; B[i] = P[P_B11 + i]; }
    } else {
        rot3(m, P[P_A11], P[P_A12], P[P_A16], P[P_A22], P[P_A26], P[P_A66], A);
        rot3(m, P[P_B11], P[P_B12], P[P_B16], P[P_B22], P[P_B26], P[P_B66], B);
    }
    for (int a = 0; a < 4; a++)
        for (int mm = 0; mm < 3; mm++)
            for (int b = 0; b < 4; b++)
                for (int nn = 0; nn < 3; nn++) {
                    int64_t k = init_k + 12 * (3 * a + mm) + 3 * b + nn;
                    Kr[k] = c[a] + mm; Kc[k] = c[b] + nn;
                }
    double pts[2] = {-GP, GP};
    double N[4], Nx[4], Ny[4], detJ;
    for (int pi = 0; pi < 2; pi++)
        for (int pj = 0; pj < 2; pj++) {
            shape_derivs(xe, pts[pi], pts[pj], &detJ, N, Nx, Ny);
            double exx = 0, eyy = 0, gxy = 0, kxx = 0, kyy = 0, kxy = 0;
            for (int a = 0; a < 4; a++) {
                const double *u = ue + 6 * a;
                exx += Nx[a] * u[0];
                eyy += Ny[a] * u[1];
                gxy += Ny[a] * u[0] + Nx[a] * u[1];
                kxx += Nx[a] * u[4];
                kyy += -Ny[a] * u[3];
                kxy += -Nx[a] * u[3] + Ny[a] * u[4];
            }
            double Nxx = A[0] * exx + A[1] * eyy + A[2] * gxy + B[0] * kxx + B[1] * kyy + B[2] * kxy;
            double Nyy = A[1] * exx + A[3] * eyy + A[4] * gxy + B[1] * kxx + B[3] * kyy + B[4] * kxy;
            double Nxy = A[2] * exx + A[4] * eyy + A[5] * gxy + B[2] * kxx + B[4] * kyy + B[5] * kxy;
            for (int a = 0; a < 4; a++)
                for (int b = 0; b < 4; b++) {
                    double g = (Nx[b] * (Nx[a] * Nxx + Ny[a] * Nxy) + Ny[b] * (Nx[a] * Nxy + Ny[a] * Nyy)) * detJ;
                    for (int mm = 0; mm < 3; mm++)
                        for (int nn = 0; nn < 3; nn++)
                            Kv[init_k + 12 * (3 * a + mm) + 3 * b + nn] += R[3 * mm + 2] * R[3 * nn + 2] * g;
                }
        }
}

/* pyfe3d/quad4.pyx:2259-3081 (update_KG_given_stress): as update_KG with the
 * constant resultants Nxx, Nyy, Nxy at the 2x2 Gauss points (unit weights). */
void orc_q4_kg_given_stress(const double *R, const double *xe, double Nxx, double Nyy, double Nxy,
                            const int64_t *c, int64_t init_k, int64_t *Kr, int64_t *Kc, double *Kv)
{
    for (int a = 0; a < 4; a++)
        for (int mm = 0; mm < 3; mm++)
            for (int b = 0; b < 4; b++)
                for (int nn = 0; nn < 3; nn++) {
                    int64_t k = init_k + 12 * (3 * a + mm) + 3 * b + nn;
                    Kr[k] = c[a] + mm; Kc[k] = c[b] + nn;
                }
    double pts[2] = {-GP, GP};
    double N[4], Nx[4], Ny[4], detJ;
    for (int pi = 0; pi < 2; pi++)
        for (int pj = 0; pj < 2; pj++) {
            shape_derivs(xe, pts[pi], pts[pj], &detJ, N, Nx, Ny);
            for (int a = 0; a < 4; a++)
                for (int b = 0; b < 4; b++) {
                    double g = (Nx[b] * (Nx[a] * Nxx + Ny[a] * Nxy) + Ny[b] * (Nx[a] * Nxy + Ny[a] * Nyy)) * detJ;
                    for (int mm = 0; mm < 3; mm++)
                        for (int nn = 0; nn < 3; nn++)
                            Kv[init_k + 12 * (3 * a + mm) + 3 * b + nn] += R[3 * mm + 2] * R[3 * nn + 2] * g;
                }
        }
}

/* pyfe3d/quad4.pyx:3083-9489 (update_M).  Local mass per node pair: h_ab
 * times [intrho I3 on translations; (u,ry)=+intrhoz, (v,rx)=-intrhoz;
 * intrhoz2 on (rx,rx),(ry,ry)], rotated by R.  mtype 0: 2x2 Gauss h_ab
 * (480 entries: pairs with |m-n| == 3 skipped); mtype 1: h_ab = area/16
 * (same 480 pattern); mtype 2: 2x2 Lobatto h_ab, translation-translation
 * and rotation-rotation blocks only (288 entries). */
void orc_q4_m(const double *R, const double *xe, double area, const double *P,
              const int64_t *c, int64_t init_k, int64_t *Kr, int64_t *Kc,
              double *Kv, int mtype)
{
    double h[4][4];
    memset(h, 0, sizeof(h));
    if (mtype == 1) {
        for (int a = 0; a < 4; a++) for (int b = 0; b < 4; b++) h[a][b] = 0.0625 * area;
    } else {
        double pts[2] = {-GP, GP};
        if (mtype == 2) { pts[0] = -1.; pts[1] = 1.; }
        double N[4], Nx[4], Ny[4], detJ;
        for (int pi = 0; pi < 2; pi++)
            for (int pj = 0; pj < 2; pj++) {
                shape_derivs(xe, pts[pi], pts[pj], &detJ, N, Nx, Ny);
                for (int a = 0; a < 4; a++)
                    for (int b = 0; b < 4; b++) h[a][b] += N[a] * N[b] * detJ;
            }
    }
    double rho = P[P_RHO], rz = P[P_RHOZ], rz2 = P[P_RHOZ2];
    double L[6][6];
    memset(L, 0, sizeof(L));
    L[0][0] = L[1][1] = L[2][2] = rho;
    L[0][4] = L[4][0] = rz;
    L[1][3] = L[3][1] = -rz;
    L[3][3] = L[4][4] = rz2;
    double G[6][6];
    for (int mm = 0; mm < 6; mm++)
        for (int nn = 0; nn < 6; nn++) {
            int gm = mm / 3, im = mm % 3, gn = nn / 3, in = nn % 3;
            double s = 0;
            for (int i = 0; i < 3; i++)
                for (int j = 0; j < 3; j++)
                    s += R[3 * im + i] * L[3 * gm + i][3 * gn + j] * R[3 * in + j];
            G[mm][nn] = s;
        }
    int64_t k = init_k;
    for (int a = 0; a < 4; a++)
        for (int mm = 0; mm < 6; mm++)
            for (int b = 0; b < 4; b++)
                for (int nn = 0; nn < 6; nn++) {
                    if (mtype == 2) { if ((mm < 3) != (nn < 3)) continue; }
                    else if (mm - nn == 3 || nn - mm == 3) continue;
                    Kr[k] = c[a] + mm; Kc[k] = c[b] + nn;
                    Kv[k] += h[a][b] * G[mm][nn];
                    k++;
                }
}

/* ------------------------------------------------------------------ */
/* BeamC: pyfe3d/beamc.pyx                                              */
/* ------------------------------------------------------------------ */

/* beamc.pyx:158-231 (update_rotation_matrix) */
void orc_bc_rotation(const double *x, const int64_t *c, const double *vxy, double *R)
{
    const double *p1 = x + c[0] / 2, *p2 = x + c[1] / 2;
    double xa[3], z[3], y[3], t;
    for (int i = 0; i < 3; i++) xa[i] = p2[i] - p1[i];
    t = sqrt(xa[0] * xa[0] + xa[1] * xa[1] + xa[2] * xa[2]);
    for (int i = 0; i < 3; i++) xa[i] /= t;
    z[0] = xa[1] * vxy[2] - xa[2] * vxy[1];
    z[1] = -xa[0] * vxy[2] + xa[2] * vxy[0];
    z[2] = xa[0] * vxy[1] - xa[1] * vxy[0];
    t = sqrt(z[0] * z[0] + z[1] * z[1] + z[2] * z[2]);
    for (int i = 0; i < 3; i++) z[i] /= t;
    y[0] = -xa[1] * z[2] + xa[2] * z[1];
    y[1] = xa[0] * z[2] - xa[2] * z[0];
    y[2] = -xa[0] * z[1] + xa[1] * z[0];
    t = sqrt(y[0] * y[0] + y[1] * y[1] + y[2] * y[2]);
    for (int i = 0; i < 3; i++) y[i] /= t;
    for (int i = 0; i < 3; i++) { R[3 * i + 0] = xa[i]; R[3 * i + 1] = y[i]; R[3 * i + 2] = z[i]; }
}

/* beamc.pyx:287-349 (update_probe_xe + update_length) */
void orc_bc_probe_xe(const double *x, const int64_t *c, const double *R, double *xe,
                     double *length)
{
    for (int j = 0; j < 2; j++) {
        const double *p = x + c[j] / 2;
        for (int k = 0; k < 3; k++) {
            double s = 0;
            for (int i = 0; i < 3; i++) s += R[3 * i + k] * p[i];
            xe[3 * j + k] = s;
        }
    }
    double dx = xe[3] - xe[0], dy = xe[4] - xe[1], dz = xe[5] - xe[2];
    *length = sqrt(dx * dx + dy * dy + dz * dz);
}

/* beamc.pyx:234-284 */
void orc_bc_probe_ue(const double *u, const int64_t *c, const double *R, double *ue)
{
    probe_ue_n(2, u, c, R, ue);
}

static void sym_set(double *K, int i, int j, double v) { K[12 * i + j] = v; K[12 * j + i] = v; }

/* Local 12x12 KC0 of the consistent Timoshenko beam (Luo 2008), closed
 * forms of beamc.pyx:543-624; DOFs u v w rx ry rz per node. */
void orc_bc_kc0_local(double L, const double *P, double *K)
{
    double A = P[BP_A], E = P[BP_E], G = P[BP_G], Iyy = P[BP_IYY], Izz = P[BP_IZZ],
           Iyz = P[BP_IYZ], J = P[BP_J], Ay = P[BP_AY], Az = P[BP_AZ];
    double ay = 12 * E * Izz / (G * A * L * L), az = 12 * E * Iyy / (G * A * L * L);
    double by = 1 / (1. - ay), bz = 1 / (1. - az);
    memset(K, 0, sizeof(double) * 144);
    double L2 = L * L, L3 = L2 * L;
    double ka = A * E / L, kt = G * J / L;
    double sy = A * G * L2 * ay * ay + 12 * E * Izz;  /* y-plane (v, rz) */
    double sz = A * G * L2 * az * az + 12 * E * Iyy;  /* z-plane (w, ry) */
    double cvv = by * by * sy / L3, cvr = by * by * sy / (2 * L2);
    double cww = bz * bz * sz / L3, cwr = bz * bz * sz / (2 * L2);
    double rzz1 = by * by * (A * G * L2 * ay * ay / 4 + E * Izz * ay * ay - 2 * E * Izz * ay + 4 * E * Izz) / L;
    double rzz2 = by * by * (A * G * L2 * ay * ay / 4 - E * Izz * ay * ay + 2 * E * Izz * ay + 2 * E * Izz) / L;
    double ryy1 = bz * bz * (A * G * L2 * az * az / 4 + E * Iyy * az * az - 2 * E * Iyy * az + 4 * E * Iyy) / L;
    double ryy2 = bz * bz * (A * G * L2 * az * az / 4 - E * Iyy * az * az + 2 * E * Iyy * az + 2 * E * Iyy) / L;
    double c3 = 12 * E * Iyz * by * bz / L3, c2 = 6 * E * Iyz * by * bz / L2;
    double c1a = E * Iyz * by * bz * (-ay * az + ay + az - 4) / L;
    double c1b = E * Iyz * by * bz * (ay * az - ay - az - 2) / L;
    double oz = Az * E * bz * (1 - az) / L, oy = Ay * E * by * (1 - ay) / L;
    double tz = Az * G * ay * by / L, ty = Ay * G * az * bz / L;
    double tz2 = Az * G * ay * by / 2, ty2 = Ay * G * az * bz / 2;
    /* axial + torsion */
    sym_set(K, 0, 0, ka); sym_set(K, 6, 6, ka); sym_set(K, 0, 6, -ka);
    sym_set(K, 3, 3, kt); sym_set(K, 9, 9, kt); sym_set(K, 3, 9, -kt);
    /* axial-bending offsets */
    sym_set(K, 0, 4, oz); sym_set(K, 0, 10, -oz); sym_set(K, 4, 6, -oz); sym_set(K, 6, 10, oz);
    sym_set(K, 0, 5, -oy); sym_set(K, 0, 11, oy); sym_set(K, 5, 6, oy); sym_set(K, 6, 11, -oy);
    /* bending in the x-y plane */
    sym_set(K, 1, 1, cvv); sym_set(K, 7, 7, cvv); sym_set(K, 1, 7, -cvv);
    sym_set(K, 1, 5, cvr); sym_set(K, 1, 11, cvr); sym_set(K, 5, 7, -cvr); sym_set(K, 7, 11, -cvr);
    sym_set(K, 5, 5, rzz1); sym_set(K, 11, 11, rzz1); sym_set(K, 5, 11, rzz2);
    /* bending in the x-z plane */
    sym_set(K, 2, 2, cww); sym_set(K, 8, 8, cww); sym_set(K, 2, 8, -cww);
    sym_set(K, 2, 4, -cwr); sym_set(K, 2, 10, -cwr); sym_set(K, 4, 8, cwr); sym_set(K, 8, 10, cwr);
    sym_set(K, 4, 4, ryy1); sym_set(K, 10, 10, ryy1); sym_set(K, 4, 10, ryy2);
    /* product of inertia coupling */
    sym_set(K, 1, 2, c3); sym_set(K, 1, 8, -c3); sym_set(K, 2, 7, -c3); sym_set(K, 7, 8, c3);
    sym_set(K, 1, 4, -c2); sym_set(K, 1, 10, -c2); sym_set(K, 2, 5, c2); sym_set(K, 2, 11, c2);
    sym_set(K, 4, 7, c2); sym_set(K, 5, 8, -c2); sym_set(K, 7, 10, c2); sym_set(K, 8, 11, -c2);
    sym_set(K, 4, 5, c1a); sym_set(K, 10, 11, c1a); sym_set(K, 4, 11, c1b); sym_set(K, 5, 10, c1b);
    /* torsion-shear couplings through the section first moments */
    sym_set(K, 1, 3, tz); sym_set(K, 1, 9, -tz); sym_set(K, 3, 7, -tz); sym_set(K, 7, 9, tz);
    sym_set(K, 2, 3, -ty); sym_set(K, 2, 9, ty); sym_set(K, 3, 8, ty); sym_set(K, 8, 9, -ty);
    sym_set(K, 3, 4, ty2); sym_set(K, 3, 10, ty2); sym_set(K, 4, 9, -ty2); sym_set(K, 9, 10, -ty2);
    sym_set(K, 3, 5, tz2); sym_set(K, 3, 11, tz2); sym_set(K, 5, 9, -tz2); sym_set(K, 9, 11, -tz2);
}

/* beamc.pyx:489-1352 (update_KC0) */
void orc_bc_kc0(const double *R, double L, const double *P, const int64_t *c,
                int64_t init_k, int64_t *Kr, int64_t *Kc, double *Kv, int values_only)
{
    double K[144];
    orc_bc_kc0_local(L, P, K);
    scatter_rotated(2, R, K, c, init_k, Kr, Kc, Kv, values_only == 0);
}

/* beamc.pyx:352-486 (update_probe_finte): finte = KC0e ue, local; and
 * beamc.pyx:1354-1390 (update_fint): fint[c + .] += R finte (fint may be NULL) */
void orc_bc_fint(const double *R, double L, const double *P, const int64_t *c, const double *ue,
                 double *fe, double *fint)
{
    double K[144];
    orc_bc_kc0_local(L, P, K);
    for (int i = 0; i < 12; i++) {
        double s = 0;
        for (int j = 0; j < 12; j++) s += K[12 * i + j] * ue[j];
        fe[i] = s;
    }
    if (!fint) return;
    for (int a = 0; a < 2; a++)
        for (int g = 0; g < 2; g++)
            for (int i = 0; i < 3; i++) {
                double s = 0;
                for (int j = 0; j < 3; j++) s += fe[6 * a + 3 * g + j] * R[3 * i + j];
                fint[c[a] + 3 * g + i] += s;
            }
}

/* Local 12x12 geometric stiffness, beamc.pyx:1889-2179: axial force
 * N = A E (u2 - u1)/L times, per pair of bending planes p, q, the 4x4 form
 * on (d1, t1, d2, t2) with t = rz for the x-y plane and t = -ry for x-z. */
void orc_bc_kg_local(double L, const double *P, const double *ue, double *K)
{
    double A = P[BP_A], E = P[BP_E], G = P[BP_G], Iyy = P[BP_IYY], Izz = P[BP_IZZ];
    double ay = 12 * E * Izz / (G * A * L * L), az = 12 * E * Iyy / (G * A * L * L);
    double by = 1 / (1. - ay), bz = 1 / (1. - az);
    double N = A * E * (-ue[0] + ue[6]) / L;
    memset(K, 0, sizeof(double) * 144);
    int dofs[2][4] = {{1, 5, 7, 11}, {2, 4, 8, 10}};
    double sgn[2][4] = {{1, 1, 1, 1}, {1, -1, 1, -1}};
    double al[2] = {ay, az}, be[2] = {by, bz};
    for (int p = 0; p < 2; p++)
        for (int q = 0; q < 2; q++) {
            double bb = be[p] * be[q], t = 5 * al[p] * al[q] - 5 * al[p] - 5 * al[q];
            double a = bb * (t + 6) / (5 * L), b = bb / 10, cc = L * bb * (t + 8) / 60,
                   e = -L * bb * (t + 2) / 60;
            double S[4][4] = {{a, b, -a, b}, {b, cc, -b, e}, {-a, -b, a, -b}, {b, e, -b, cc}};
            for (int i = 0; i < 4; i++)
                for (int j = 0; j < 4; j++)
                    K[12 * dofs[p][i] + dofs[q][j]] = N * sgn[p][i] * sgn[q][j] * S[i][j];
        }
}

/* beamc.pyx:1392-2179 (update_KG): indices are written when the flag is 0
 * (the code's behaviour, beamc.pyx:1451). */
void orc_bc_kg(const double *R, double L, const double *P, const double *ue,
               const int64_t *c, int64_t init_k, int64_t *Kr, int64_t *Kc, double *Kv,
               int values_only)
{
    double K[144];
    orc_bc_kg_local(L, P, ue, K);
    scatter_rotated(2, R, K, c, init_k, Kr, Kc, Kv, values_only == 0);
}

/* Local consistent mass (mtype 0), closed forms of beamc.pyx:2246-2968. */
void orc_bc_m0_local(double L, const double *P, double *M)
{
    double A = P[BP_A], E = P[BP_E], G = P[BP_G], Iyy = P[BP_IYY], Izz = P[BP_IZZ];
    double r = P[BP_RHO], ry = P[BP_RHOY], rz = P[BP_RHOZ], ry2 = P[BP_RHOY2],
           rz2 = P[BP_RHOZ2], ryz = P[BP_RHOYZ];
    double ay = 12 * E * Izz / (G * A * L * L), az = 12 * E * Iyy / (G * A * L * L);
    double by = 1 / (1. - ay), bz = 1 / (1. - az);
    double L2 = L * L;
    memset(M, 0, sizeof(double) * 144);
    /* axial */
    sym_set(M, 0, 0, L * r / 3); sym_set(M, 6, 6, L * r / 3); sym_set(M, 0, 6, L * r / 6);
    /* axial - lateral through the first moments */
    sym_set(M, 0, 1, by * ry / 2); sym_set(M, 0, 7, -by * ry / 2);
    sym_set(M, 1, 6, by * ry / 2); sym_set(M, 6, 7, -by * ry / 2);
    sym_set(M, 0, 2, bz * rz / 2); sym_set(M, 0, 8, -bz * rz / 2);
    sym_set(M, 2, 6, bz * rz / 2); sym_set(M, 6, 8, -bz * rz / 2);
    sym_set(M, 0, 4, L * bz * rz * (1 - 4 * az) / 12); sym_set(M, 6, 10, L * bz * rz * (1 - 4 * az) / 12);
    sym_set(M, 0, 10, -L * bz * rz * (2 * az + 1) / 12); sym_set(M, 4, 6, -L * bz * rz * (2 * az + 1) / 12);
    sym_set(M, 0, 5, L * by * ry * (4 * ay - 1) / 12); sym_set(M, 6, 11, L * by * ry * (4 * ay - 1) / 12);
    sym_set(M, 0, 11, L * by * ry * (2 * ay + 1) / 12); sym_set(M, 5, 6, L * by * ry * (2 * ay + 1) / 12);
    /* translation, x-y plane (v, rz) */
    double vv = by * by * (70 * L2 * ay * ay * r - 147 * L2 * ay * r + 78 * L2 * r + 252 * ry2) / (210 * L);
    double vv2 = by * by * (35 * L2 * ay * ay * r - 63 * L2 * ay * r + 27 * L2 * r - 252 * ry2) / (210 * L);
    double vr = by * by * (35 * L2 * ay * ay * r - 77 * L2 * ay * r + 44 * L2 * r + 420 * ay * ry2 + 84 * ry2) / 840;
    double vr2 = by * by * (-35 * L2 * ay * ay * r + 63 * L2 * ay * r - 26 * L2 * r + 420 * ay * ry2 + 84 * ry2) / 840;
    double rr = L * by * by * (7 * L2 * ay * ay * r - 14 * L2 * ay * r + 8 * L2 * r + 280 * ay * ay * ry2 - 140 * ay * ry2 + 112 * ry2) / 840;
    double rr2 = L * by * by * (-7 * L2 * ay * ay * r + 14 * L2 * ay * r - 6 * L2 * r + 140 * ay * ay * ry2 + 140 * ay * ry2 - 28 * ry2) / 840;
    sym_set(M, 1, 1, vv); sym_set(M, 7, 7, vv); sym_set(M, 1, 7, vv2);
    sym_set(M, 1, 5, vr); sym_set(M, 7, 11, -vr); sym_set(M, 1, 11, vr2); sym_set(M, 5, 7, -vr2);
    sym_set(M, 5, 5, rr); sym_set(M, 11, 11, rr); sym_set(M, 5, 11, rr2);
    /* translation, x-z plane (w, ry) */
    double ww = bz * bz * (70 * L2 * az * az * r - 147 * L2 * az * r + 78 * L2 * r + 252 * rz2) / (210 * L);
    double ww2 = bz * bz * (35 * L2 * az * az * r - 63 * L2 * az * r + 27 * L2 * r - 252 * rz2) / (210 * L);
    double wr = bz * bz * (-35 * L2 * az * az * r + 77 * L2 * az * r - 44 * L2 * r - 420 * az * rz2 - 84 * rz2) / 840;
    double wr2 = bz * bz * (35 * L2 * az * az * r - 63 * L2 * az * r + 26 * L2 * r - 420 * az * rz2 - 84 * rz2) / 840;
    double ss = L * bz * bz * (7 * L2 * az * az * r - 14 * L2 * az * r + 8 * L2 * r + 280 * az * az * rz2 - 140 * az * rz2 + 112 * rz2) / 840;
    double ss2 = L * bz * bz * (-7 * L2 * az * az * r + 14 * L2 * az * r - 6 * L2 * r + 140 * az * az * rz2 + 140 * az * rz2 - 28 * rz2) / 840;
    sym_set(M, 2, 2, ww); sym_set(M, 8, 8, ww); sym_set(M, 2, 8, ww2);
    sym_set(M, 2, 4, wr); sym_set(M, 8, 10, -wr); sym_set(M, 2, 10, wr2); sym_set(M, 4, 8, -wr2);
    sym_set(M, 4, 4, ss); sym_set(M, 10, 10, ss); sym_set(M, 4, 10, ss2);
    /* product-of-inertia coupling between the planes */
    double p1 = 6 * by * bz * ryz / (5 * L);
    sym_set(M, 1, 2, p1); sym_set(M, 7, 8, p1); sym_set(M, 1, 8, -p1); sym_set(M, 2, 7, -p1);
    double pz = by * bz * ryz * (5 * az + 1) / 10, py = by * bz * ryz * (5 * ay + 1) / 10;
    sym_set(M, 1, 4, -pz); sym_set(M, 1, 10, -pz); sym_set(M, 4, 7, pz); sym_set(M, 7, 10, pz);
    sym_set(M, 2, 5, py); sym_set(M, 2, 11, py); sym_set(M, 5, 8, -py); sym_set(M, 8, 11, -py);
    double q1 = L * by * bz * ryz * (-20 * ay * az + 5 * ay + 5 * az - 8) / 60;
    double q2 = L * by * bz * ryz * (-10 * ay * az - 5 * ay - 5 * az + 2) / 60;
    sym_set(M, 4, 5, q1); sym_set(M, 10, 11, q1); sym_set(M, 4, 11, q2); sym_set(M, 5, 10, q2);
    /* torsion */
    double rp = ry2 + rz2;
    sym_set(M, 3, 3, L * rp / 3); sym_set(M, 9, 9, L * rp / 3); sym_set(M, 3, 9, L * rp / 6);
    /* torsion - lateral through the first moments */
    sym_set(M, 1, 3, L * by * rz * (20 * ay - 21) / 60); sym_set(M, 7, 9, L * by * rz * (20 * ay - 21) / 60);
    sym_set(M, 1, 9, L * by * rz * (10 * ay - 9) / 60); sym_set(M, 3, 7, L * by * rz * (10 * ay - 9) / 60);
    sym_set(M, 2, 3, L * bz * ry * (21 - 20 * az) / 60); sym_set(M, 8, 9, L * bz * ry * (21 - 20 * az) / 60);
    sym_set(M, 2, 9, L * bz * ry * (9 - 10 * az) / 60); sym_set(M, 3, 8, L * bz * ry * (9 - 10 * az) / 60);
    sym_set(M, 3, 4, L2 * bz * ry * (5 * az - 6) / 120); sym_set(M, 9, 10, L2 * bz * ry * (6 - 5 * az) / 120);
    sym_set(M, 3, 10, L2 * bz * ry * (4 - 5 * az) / 120); sym_set(M, 4, 9, L2 * bz * ry * (5 * az - 4) / 120);
    sym_set(M, 3, 5, L2 * by * rz * (5 * ay - 6) / 120); sym_set(M, 9, 11, L2 * by * rz * (6 - 5 * ay) / 120);
    sym_set(M, 3, 11, L2 * by * rz * (4 - 5 * ay) / 120); sym_set(M, 5, 9, L2 * by * rz * (5 * ay - 4) / 120);
}

/* Local lumped mass (mtype 1), beamc.pyx:2969-3152: diagonal. */
void orc_bc_m1_local(double L, const double *P, double *M)
{
    double A = P[BP_A], E = P[BP_E], G = P[BP_G], Iyy = P[BP_IYY], Izz = P[BP_IZZ];
    double r = P[BP_RHO], ry2 = P[BP_RHOY2], rz2 = P[BP_RHOZ2];
    double ay = 12 * E * Izz / (G * A * L * L), az = 12 * E * Iyy / (G * A * L * L);
    double by = 1 / (1. - ay), bz = 1 / (1. - az);
    double fy = by * by * (ay * ay - 2 * ay + 1), fz = bz * bz * (az * az - 2 * az + 1);
    memset(M, 0, sizeof(double) * 144);
    for (int n = 0; n < 2; n++) {
        int o = 6 * n;
        M[13 * (o + 0)] = L * r / 2;
        M[13 * (o + 1)] = L * fy * r / 2;
        M[13 * (o + 2)] = L * fz * r / 2;
        M[13 * (o + 3)] = L * (ry2 + rz2) / 2;
        M[13 * (o + 4)] = L * fz * rz2 / 2;
        M[13 * (o + 5)] = L * fy * ry2 / 2;
    }
}

/* beamc.pyx:2181-3152 (update_M): mtype 0 writes the full 12x12 (144);
 * mtype 1 writes the four 3x3 diagonal blocks (36 entries). */
void orc_bc_m(const double *R, double L, const double *P, const int64_t *c,
              int64_t init_k, int64_t *Kr, int64_t *Kc, double *Kv, int mtype)
{
    double M[144];
    if (mtype == 0) {
        orc_bc_m0_local(L, P, M);
        scatter_rotated(2, R, M, c, init_k, Kr, Kc, Kv, 1);
        return;
    }
    orc_bc_m1_local(L, P, M);
    int64_t k = init_k;
    for (int blk = 0; blk < 4; blk++) {
        int node = blk / 2, g = blk % 2;
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) {
                double s = 0;
                for (int p = 0; p < 3; p++)
                    for (int q = 0; q < 3; q++)
                        s += R[3 * i + p] * M[12 * (6 * node + 3 * g + p) + 6 * node + 3 * g + q] * R[3 * j + q];
                Kr[k] = c[node] + 3 * g + i;
                Kc[k] = c[node] + 3 * g + j;
                Kv[k] += s;
                k++;
            }
    }
}

/* ------------------------------------------------------------------ */
/* Reduced-integration shells: pyfe3d/tria3r.pyx, pyfe3d/quad4r.pyx     */
/* ------------------------------------------------------------------ */

/* Material-direction projection shared by the shell frames
 * (tria3r.pyx:389-423, quad4r.pyx:381-419): m is only overwritten when
 * xmat projects onto the element plane. */
static void mat_direction(const double *z, const double *xa, const double *y, double tol,
                          const double *xmat, double *m)
{
    double xm[3] = {xmat[0], xmat[1], xmat[2]}, ym[3], t;
    double xn = sqrt(xm[0] * xm[0] + xm[1] * xm[1] + xm[2] * xm[2]);
    for (int i = 0; i < 3; i++) xm[i] /= xn;
    if (!(xn > tol)) return;
    ym[0] = z[1] * xm[2] - z[2] * xm[1];
    ym[1] = z[2] * xm[0] - z[0] * xm[2];
    ym[2] = z[0] * xm[1] - z[1] * xm[0];
    t = sqrt(ym[0] * ym[0] + ym[1] * ym[1] + ym[2] * ym[2]);
    for (int i = 0; i < 3; i++) ym[i] /= t;
    if (!(t > tol)) return;
    xm[0] = ym[1] * z[2] - ym[2] * z[1];
    xm[1] = ym[2] * z[0] - ym[0] * z[2];
    xm[2] = ym[0] * z[1] - ym[1] * z[0];
    t = sqrt(xm[0] * xm[0] + xm[1] * xm[1] + xm[2] * xm[2]);
    for (int i = 0; i < 3; i++) xm[i] /= t;
    double cth = xm[0] * xa[0] + xm[1] * xa[1] + xm[2] * xa[2];
    m[0] = cth; m[3] = cth;
    if (xm[0] * y[0] + xm[1] * y[1] + xm[2] * y[2] > 0) m[1] = -sqrt(1 - cth * cth);
    else m[1] = sqrt(1 - cth * cth);
    m[2] = -m[1];
}

/* Tria3R frame, tria3r.pyx:294-423: z = v12 x v13, x along v12, y = z x x. */
void orc_t3_rotation(const double *x, const int64_t *c, const double *xmat,
                     double *R, double *m)
{
    const double *p1 = x + c[0] / 2, *p2 = x + c[1] / 2, *p3 = x + c[2] / 2;
    double v12[3], v13[3], z[3], xa[3], y[3], t;
    for (int i = 0; i < 3; i++) { v12[i] = p2[i] - p1[i]; v13[i] = p3[i] - p1[i]; }
    z[0] = v12[1] * v13[2] - v12[2] * v13[1];
    z[1] = v12[2] * v13[0] - v12[0] * v13[2];
    z[2] = v12[0] * v13[1] - v12[1] * v13[0];
    t = sqrt(z[0] * z[0] + z[1] * z[1] + z[2] * z[2]);
    for (int i = 0; i < 3; i++) z[i] /= t;
    double tol = t / 1e10;
    t = sqrt(v12[0] * v12[0] + v12[1] * v12[1] + v12[2] * v12[2]);
    for (int i = 0; i < 3; i++) xa[i] = v12[i] / t;
    y[0] = z[1] * xa[2] - z[2] * xa[1];
    y[1] = z[2] * xa[0] - z[0] * xa[2];
    y[2] = z[0] * xa[1] - z[1] * xa[0];
    t = sqrt(y[0] * y[0] + y[1] * y[1] + y[2] * y[2]);
    for (int i = 0; i < 3; i++) y[i] /= t;
    for (int i = 0; i < 3; i++) { R[3 * i + 0] = xa[i]; R[3 * i + 1] = y[i]; R[3 * i + 2] = z[i]; }
    if (xmat) mat_direction(z, xa, y, tol, xmat, m);
}

/* tria3r.pyx:480-547 (update_probe_xe + update_area) */
void orc_t3_probe_xe(const double *x, const int64_t *c, const double *R,
                     double *xe, double *area)
{
    for (int j = 0; j < 3; j++) {
        const double *p = x + c[j] / 2;
        for (int k = 0; k < 3; k++) {
            double s = 0;
            for (int i = 0; i < 3; i++) s += R[3 * i + k] * p[i];
            xe[3 * j + k] = s;
        }
    }
    double x1 = xe[0], y1 = xe[1], x2 = xe[3], y2 = xe[4], x3 = xe[6], y3 = xe[7];
    *area = fabs((-x1 + x2) * (-y1 + y3) / 2. + (x1 - x3) * (-y1 + y2) / 2.);
}

/* tria3r.pyx:426-477 (update_probe_ue) */
void orc_t3_probe_ue(const double *u, const int64_t *c, const double *R, double *ue)
{
    probe_ue_n(3, u, c, R, ue);
}

/* ABD in the element (material-rotated) axes: quad4.pyx:845-899 and the
 * identical blocks of tria3r.pyx / quad4r.pyx. */
static void element_abd(const double *m, const double *P, double *A, double *B, double *D)
{
    if (m[1] == 0) {
        for (int i = 0; i < 6; i++) { A[i] = P[P_A11 + i]; B[i] = P[P_B11 + i]; D[i] = P[P_D11 + i]; }
    } else {
        rot3(m, P[P_A11], P[P_A12], P[P_A16], P[P_A22], P[P_A26], P[P_A66], A);
        rot3(m, P[P_B11], P[P_B12], P[P_B16], P[P_B22], P[P_B26], P[P_B66], B);
        rot3(m, P[P_D11], P[P_D12], P[P_D16], P[P_D22], P[P_D26], P[P_D66], D);
    }
}

/* Constant-strain part of a reduced shell at one point (weight wd = w detJ):
 * membrane/bending Bl^T ABD Bl and transverse shear with
 * (gyz, gxz) = (w_y - rx N, w_x + ry N). n = 6 nn. */
static void reduced_point(int nn, const double *A, const double *B, const double *D,
                          double E44, double E45, double E55, const double *N,
                          const double *Nx, const double *Ny, double wd, double *Ke)
{
    int n = 6 * nn;
    double ABD[6][6] = {
        {A[0], A[1], A[2], B[0], B[1], B[2]},
        {A[1], A[3], A[4], B[1], B[3], B[4]},
        {A[2], A[4], A[5], B[2], B[4], B[5]},
        {B[0], B[1], B[2], D[0], D[1], D[2]},
        {B[1], B[3], B[4], D[1], D[3], D[4]},
        {B[2], B[4], B[5], D[2], D[4], D[5]}};
    double Bl[6][24], gy[24], gx[24];
    memset(Bl, 0, sizeof(Bl)); memset(gy, 0, sizeof(gy)); memset(gx, 0, sizeof(gx));
    for (int a = 0; a < nn; a++) {
        int o = 6 * a;
        Bl[0][o + 0] = Nx[a];
        Bl[1][o + 1] = Ny[a];
        Bl[2][o + 0] = Ny[a]; Bl[2][o + 1] = Nx[a];
        Bl[3][o + 4] = Nx[a];
        Bl[4][o + 3] = -Ny[a];
        Bl[5][o + 3] = -Nx[a]; Bl[5][o + 4] = Ny[a];
        gy[o + 2] = Ny[a]; gy[o + 3] = -N[a];
        gx[o + 2] = Nx[a]; gx[o + 4] = N[a];
    }
    for (int i = 0; i < n; i++)
        for (int j = 0; j < n; j++) {
            double s = 0;
            for (int p = 0; p < 6; p++)
                for (int q = 0; q < 6; q++) s += Bl[p][i] * ABD[p][q] * Bl[q][j];
            s += gy[i] * E44 * gy[j] + gy[i] * E45 * gx[j] + gx[i] * E45 * gy[j] + gx[i] * E55 * gx[j];
            Ke[n * i + j] += wd * s;
        }
}

/* Drilling penalty K6ROT 1e-6 A66 (rz - theta_z)^2 at one point, with
 * d = u N_y/2 - v N_x/2 + rz N (tria3r.pyx:69-103). */
static void drilling_point(int nn, double kd, const double *N, const double *Nx,
                           const double *Ny, double wd, double *Ke)
{
    int n = 6 * nn;
    double dr[24];
    memset(dr, 0, sizeof(dr));
    for (int a = 0; a < nn; a++) {
        dr[6 * a + 0] = Ny[a] / 2.; dr[6 * a + 1] = -Nx[a] / 2.; dr[6 * a + 5] = N[a];
    }
    for (int i = 0; i < n; i++)
        for (int j = 0; j < n; j++) Ke[n * i + j] += kd * wd * dr[i] * dr[j];
}

/* Constant derivatives of the linear triangle (tria3r.pyx:2116-2121). */
static void tria_derivs(const double *xe, double area, double *Nx, double *Ny)
{
    double x1 = xe[0], y1 = xe[1], x2 = xe[3], y2 = xe[4], x3 = xe[6], y3 = xe[7];
    Nx[0] = (y2 - y3) / (2 * area); Nx[1] = (-y1 + y3) / (2 * area); Nx[2] = (y1 - y2) / (2 * area);
    Ny[0] = (-x2 + x3) / (2 * area); Ny[1] = (x1 - x3) / (2 * area); Ny[2] = (-x1 + x2) / (2 * area);
}

/* Local 18x18 Tria3R stiffness, tria3r.pyx:950-2322: one centroid point
 * (weight 1/2) for membrane, bending and transverse shear, the shear terms
 * scaled by 1 / (1 + alpha maxl^2 / h^2); drilling by the 3-point rule
 * (2/3, 1/6, 1/6) with weight 1/6. */
void orc_t3_kc0_local(const double *m, const double *xe, double area, const double *P,
                      double k6rot, double alpha, double *Ke)
{
    double A[6], B[6], D[6];
    element_abd(m, P, A, B, D);
    double E44 = P[P_E44] * P[P_SCF23];
    double E45 = P[P_E45] * 0.5 * (P[P_SCF13] + P[P_SCF23]);
    double E55 = P[P_E55] * P[P_SCF13];
    double x1 = xe[0], y1 = xe[1], x2 = xe[3], y2 = xe[4], x3 = xe[6], y3 = xe[7];
    double l12 = sqrt((x1 - x2) * (x1 - x2) + (y1 - y2) * (y1 - y2));
    double l23 = sqrt((x2 - x3) * (x2 - x3) + (y2 - y3) * (y2 - y3));
    double l31 = sqrt((x3 - x1) * (x3 - x1) + (y3 - y1) * (y3 - y1));
    double maxl = l12;
    if (l23 > maxl) maxl = l23;
    if (l31 > maxl) maxl = l31;
    double factor = alpha * maxl * maxl / (P[P_H] * P[P_H]);
    E44 = 1 / (1 + factor) * E44;
    E45 = 1 / (1 + factor) * E45;
    E55 = 1 / (1 + factor) * E55;
    double detJ = 2 * area;
    double Nx[3], Ny[3];
    tria_derivs(xe, area, Nx, Ny);
    memset(Ke, 0, sizeof(double) * 324);
    double Nc[3] = {1. / 3, 1. / 3, 1. / 3};
    reduced_point(3, A, B, D, E44, E45, E55, Nc, Nx, Ny, detJ * 0.5, Ke);
    double kd = 1e-6 * k6rot * A[5];
    const double p0 = 2. / 3, p1 = 1. / 6;
    double pts[3][2] = {{p0, p1}, {p1, p1}, {p1, p0}};
    for (int g = 0; g < 3; g++) {
        double N[3] = {pts[g][0], pts[g][1], 1 - pts[g][0] - pts[g][1]};
        drilling_point(3, kd, N, Nx, Ny, detJ * (0.5 / 3), Ke);
    }
}

/* tria3r.pyx:950-2960 (update_KC0) */
void orc_t3_kc0(const double *R, const double *m, const double *xe, double area,
                const double *P, double k6rot, double alpha, const int64_t *c,
                int64_t init_k, int64_t *Kr, int64_t *Kc, double *Kv, int values_only)
{
    double Ke[324];
    orc_t3_kc0_local(m, xe, area, P, k6rot, alpha, Ke);
    /* the element-to-global transformation of update_KC0
     * (tria3r.pyx:2323-2960) keeps, of the local drilling DOF rz, only its
     * diagonal terms rz_a - rz_a: the couplings of rz with u, v and with the
     * rz of the other nodes, present in the local matrix (and used by
     * update_probe_finte), do not reach KC0v; they are left out here the
     * same way */
    for (int i = 0; i < 18; i++)
        for (int j = 0; j < 18; j++)
            if ((i % 6 == 5 || j % 6 == 5) && i != j) Ke[18 * i + j] = 0.;
    scatter_rotated(3, R, Ke, c, init_k, Kr, Kc, Kv, values_only == 0);
}

static void local_times(int n, const double *Ke, const double *ue, double *fe)
{
    for (int i = 0; i < n; i++) {
        double s = 0;
        for (int j = 0; j < n; j++) s += Ke[n * i + j] * ue[j];
        fe[i] = s;
    }
}

static void fint_rotated(int nn, const double *R, const int64_t *c, const double *fe, double *fint)
{
    for (int a = 0; a < nn; a++)
        for (int g = 0; g < 2; g++)
            for (int i = 0; i < 3; i++) {
                double s = 0;
                for (int j = 0; j < 3; j++) s += fe[6 * a + 3 * g + j] * R[3 * i + j];
                fint[c[a] + 3 * g + i] += s;
            }
}

/* tria3r.pyx:549-947 (update_probe_finte): finte = KC0e ue, local */
void orc_t3_finte(const double *m, const double *xe, double area, const double *P,
                  double k6rot, double alpha, const double *ue, double *fe)
{
    double Ke[324];
    orc_t3_kc0_local(m, xe, area, P, k6rot, alpha, Ke);
    local_times(18, Ke, ue, fe);
}

/* tria3r.pyx:2975-3017 (update_fint) */
void orc_t3_fint(const double *R, const double *m, const double *xe, double area,
                 const double *P, double k6rot, double alpha, const int64_t *c,
                 const double *ue, double *fint)
{
    double fe[18];
    orc_t3_finte(m, xe, area, P, k6rot, alpha, ue, fe);
    fint_rotated(3, R, c, fe, fint);
}

/* Geometric stiffness of a constant membrane state on the translations,
 * 9x9 row-major: r_m3 r_n3 (grad N_a . Nmat . grad N_b) detJ / 2. */
static void t3_kg_scatter(const double *R, const double *Nx, const double *Ny, double detJ,
                          double Nxx, double Nyy, double Nxy, const int64_t *c, int64_t init_k,
                          int64_t *Kr, int64_t *Kc, double *Kv, int values_only)
{
    for (int a = 0; a < 3; a++)
        for (int mm = 0; mm < 3; mm++)
            for (int b = 0; b < 3; b++)
                for (int nn = 0; nn < 3; nn++) {
                    int64_t k = init_k + 9 * (3 * a + mm) + 3 * b + nn;
                    if (!values_only) { Kr[k] = c[a] + mm; Kc[k] = c[b] + nn; }
                    double g = (Nx[b] * (Nx[a] * Nxx + Ny[a] * Nxy) + Ny[b] * (Nx[a] * Nxy + Ny[a] * Nyy)) *
                               detJ * 0.5;
                    Kv[k] += R[3 * mm + 2] * R[3 * nn + 2] * g;
                }
}

/* tria3r.pyx:3020-3574 (update_KG): resultants from ue at the centroid;
 * indices written when values_only == 0 */
void orc_t3_kg(const double *R, const double *m, const double *xe, double area,
               const double *ue, const double *P, const int64_t *c, int64_t init_k,
               int64_t *Kr, int64_t *Kc, double *Kv, int values_only)
{
    double A[6], B[6], D[6];
    element_abd(m, P, A, B, D);
    double Nx[3], Ny[3];
    tria_derivs(xe, area, Nx, Ny);
    double exx = 0, eyy = 0, gxy = 0, kxx = 0, kyy = 0, kxy = 0;
    for (int a = 0; a < 3; a++) {
        const double *u = ue + 6 * a;
        exx += Nx[a] * u[0];
        eyy += Ny[a] * u[1];
        gxy += Ny[a] * u[0] + Nx[a] * u[1];
        kxx += Nx[a] * u[4];
        kyy += -Ny[a] * u[3];
        kxy += -Nx[a] * u[3] + Ny[a] * u[4];
    }
    double Nxx = A[0] * exx + A[1] * eyy + A[2] * gxy + B[0] * kxx + B[1] * kyy + B[2] * kxy;
    double Nyy = A[1] * exx + A[3] * eyy + A[4] * gxy + B[1] * kxx + B[3] * kyy + B[4] * kxy;
    double Nxy = A[2] * exx + A[4] * eyy + A[5] * gxy + B[2] * kxx + B[4] * kyy + B[5] * kxy;
    t3_kg_scatter(R, Nx, Ny, 2 * area, Nxx, Nyy, Nxy, c, init_k, Kr, Kc, Kv, values_only);
}

/* tria3r.pyx:3576-4061 (update_KG_given_stress) */
void orc_t3_kg_given_stress(const double *R, const double *xe, double area, double Nxx,
                            double Nyy, double Nxy, const int64_t *c, int64_t init_k,
                            int64_t *Kr, int64_t *Kc, double *Kv, int values_only)
{
    double Nx[3], Ny[3];
    tria_derivs(xe, area, Nx, Ny);
    t3_kg_scatter(R, Nx, Ny, 2 * area, Nxx, Nyy, Nxy, c, init_k, Kr, Kc, Kv, values_only);
}

/* tria3r.pyx:4063-7723 (update_M): h_ab from the 3-point rule (mtype 0,
 * 270 entries), detJ/18 (mtype 1, same pattern) or the vertex rule
 * (mtype 2, 162 entries of like-kind DOF pairs); the nodal 6x6 pattern of
 * the Quad4 mass. */
void orc_t3_m(const double *R, double area, const double *P, const int64_t *c,
              int64_t init_k, int64_t *Kr, int64_t *Kc, double *Kv, int mtype)
{
    double h[3][3], detJ = 2 * area;
    memset(h, 0, sizeof(h));
    if (mtype == 1) {
        for (int a = 0; a < 3; a++) for (int b = 0; b < 3; b++) h[a][b] = detJ / 18.;
    } else {
        const double p0 = mtype == 2 ? 1. : 2. / 3, p1 = mtype == 2 ? 0. : 1. / 6;
        double pts[3][3] = {{p0, p1, p1}, {p1, p1, p0}, {p1, p0, p1}};
        for (int g = 0; g < 3; g++)
            for (int a = 0; a < 3; a++)
                for (int b = 0; b < 3; b++) h[a][b] += pts[g][a] * pts[g][b] * detJ * (0.5 / 3);
    }
    double rho = P[P_RHO], rz = P[P_RHOZ], rz2 = P[P_RHOZ2];
    double L[6][6];
    memset(L, 0, sizeof(L));
    L[0][0] = L[1][1] = L[2][2] = rho;
    L[0][4] = L[4][0] = rz;
    L[1][3] = L[3][1] = -rz;
    L[3][3] = L[4][4] = rz2;
    double G[6][6];
    for (int mm = 0; mm < 6; mm++)
        for (int nn = 0; nn < 6; nn++) {
            int gm = mm / 3, im = mm % 3, gn = nn / 3, in = nn % 3;
            double s = 0;
            for (int i = 0; i < 3; i++)
                for (int j = 0; j < 3; j++) s += R[3 * im + i] * L[3 * gm + i][3 * gn + j] * R[3 * in + j];
            G[mm][nn] = s;
        }
    int64_t k = init_k;
    for (int a = 0; a < 3; a++)
        for (int mm = 0; mm < 6; mm++)
            for (int b = 0; b < 3; b++)
                for (int nn = 0; nn < 6; nn++) {
                    if (mtype == 2) { if ((mm < 3) != (nn < 3)) continue; }
                    else if (mm - nn == 3 || nn - mm == 3) continue;
                    Kr[k] = c[a] + mm; Kc[k] = c[b] + nn;
                    Kv[k] += h[a][b] * G[mm][nn];
                    k++;
                }
}

/* Local 24x24 Quad4R stiffness, quad4r.pyx:1145-3780: one centre point
 * (weight 4) for membrane, bending and transverse shear; Brockman's
 * hourglass stiffness on u, v, w, rx, ry with gamma_a = N_a,xy at the centre
 * (quad4r.pyx:1936-1981); drilling by the 2x2 Gauss rule (quad4r.pyx:3305-3780).
 * hg = hgfactor_u, _v, _w, _rx, _ry. */
void orc_q4r_kc0_local(const double *m, const double *xe, double area, const double *P,
                       double k6rot, const double *hg, double *Ke)
{
    double A[6], B[6], D[6];
    element_abd(m, P, A, B, D);
    double den = -A[0] * A[3] * A[5] + A[0] * A[4] * A[4] + A[1] * A[1] * A[5] -
                 2 * A[1] * A[2] * A[4] + A[2] * A[2] * A[3];
    double a11 = (-A[3] * A[5] + A[4] * A[4]) / den;
    double a22 = (-A[0] * A[5] + A[2] * A[2]) / den;
    double h = P[P_H];
    double E1eq = 1. / (h * a11), E2eq = 1. / (h * a22);
    double E44 = P[P_E44] * P[P_SCF23];
    double E45 = P[P_E45] * 0.5 * (P[P_SCF13] + P[P_SCF23]);
    double E55 = P[P_E55] * P[P_SCF13];
    double s = 1.0 + 1.0 / area;
    double Eu = hg[0] * 0.1 * E1eq * h / s;
    double Ev = hg[1] * 0.1 * E2eq * h / s;
    double Erx = hg[3] * 0.1 * E2eq * h * h * h / s;
    double Ery = hg[4] * 0.1 * E1eq * h * h * h / s;
    double Ew = hg[2] * 0.5 * (Erx + Ery);
    memset(Ke, 0, sizeof(double) * 576);
    double N[4], Nx[4], Ny[4], detJ;
    shape_derivs(xe, 0., 0., &detJ, N, Nx, Ny);
    reduced_point(4, A, B, D, E44, E45, E55, N, Nx, Ny, detJ * 4., Ke);
    /* N_a,xy at the centre: the xi-eta twist of N_a pushed by the inverse
     * Jacobian, (j11 j22 + j12 j21) / 4 with signs + - + - */
    double x1 = xe[0], y1 = xe[1], x2 = xe[3], y2 = xe[4], x3 = xe[6], y3 = xe[7],
           x4 = xe[9], y4 = xe[10];
    double J11 = 0.25 * (-x1 + x2 + x3 - x4), J12 = 0.25 * (-y1 + y2 + y3 - y4);
    double J21 = 0.25 * (-x1 - x2 + x3 + x4), J22 = 0.25 * (-y1 - y2 + y3 + y4);
    double dj = J11 * J22 - J12 * J21;
    double j11 = J22 / dj, j12 = -J12 / dj, j21 = -J21 / dj, j22 = J11 / dj;
    double tw = 0.25 * (j11 * j22 + j12 * j21);
    double gam[4] = {tw, -tw, tw, -tw};
    double Ehg[5] = {Eu, Ev, Ew, Erx, Ery};
    for (int a = 0; a < 4; a++)
        for (int b = 0; b < 4; b++)
            for (int d = 0; d < 5; d++) Ke[24 * (6 * a + d) + 6 * b + d] += detJ * 4. * Ehg[d] * gam[a] * gam[b];
    double kd = 1e-6 * k6rot * A[5];
    double pts[2] = {-GP, GP};
    for (int pi = 0; pi < 2; pi++)
        for (int pj = 0; pj < 2; pj++) {
            shape_derivs(xe, pts[pi], pts[pj], &detJ, N, Nx, Ny);
            drilling_point(4, kd, N, Nx, Ny, detJ, Ke);
        }
}

/* quad4r.pyx:1145-4618 (update_KC0) */
void orc_q4r_kc0(const double *R, const double *m, const double *xe, double area,
                 const double *P, double k6rot, const double *hg, const int64_t *c,
                 int64_t init_k, int64_t *Kr, int64_t *Kc, double *Kv, int values_only)
{
    double Ke[576];
    orc_q4r_kc0_local(m, xe, area, P, k6rot, hg, Ke);
    scatter_rotated(4, R, Ke, c, init_k, Kr, Kc, Kv, values_only == 0);
}

/* quad4r.pyx:549-1143 (update_probe_finte): finte = KC0e ue, local */
void orc_q4r_finte(const double *m, const double *xe, double area, const double *P,
                   double k6rot, const double *hg, const double *ue, double *fe)
{
    double Ke[576];
    orc_q4r_kc0_local(m, xe, area, P, k6rot, hg, Ke);
    local_times(24, Ke, ue, fe);
}

/* quad4r.pyx:4620-4679 (update_fint) */
void orc_q4r_fint(const double *R, const double *m, const double *xe, double area,
                  const double *P, double k6rot, const double *hg, const int64_t *c,
                  const double *ue, double *fint)
{
    double fe[24];
    orc_q4r_finte(m, xe, area, P, k6rot, hg, ue, fe);
    fint_rotated(4, R, c, fe, fint);
}

/* ------------------------------------------------------------------ */
/* Batched drivers (frame + matrices for E elements, OpenMP over         */
/* elements).  These time the CPU path and generate full-size parity     */
/* data; every element follows the per-element sequence of the           */
/* reference tests: rotation -> probe_xe -> update_KC0.                   */
/* ------------------------------------------------------------------ */
int orc_num_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void orc_set_threads(int n)
{
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

void orc_q4_kc0_batch(int64_t E, const int64_t *cdof, const int64_t *init_k,
                      const double *x, const double *xmat, const double *props,
                      const int32_t *pid, int64_t *Kr, int64_t *Kc, double *Kv,
                      int values_only)
{
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < E; e++) {
        double R[9], m[4] = {1, 0, 0, 1}, xe[12], area;
        const int64_t *c = cdof + 4 * e;
        orc_q4_rotation(x, c, xmat ? xmat + 3 * e : 0, R, m);
        orc_q4_probe_xe(x, c, R, xe, &area);
        const double *P = props + Q4P_STRIDE * (pid ? pid[e] : e);
        orc_q4_kc0(R, m, xe, area, P, c, init_k[e], Kr, Kc, Kv, values_only);
    }
}

void orc_q4_kg_batch(int64_t E, const int64_t *cdof, const int64_t *init_k,
                     const double *x, const double *xmat, const double *u,
                     const double *props, const int32_t *pid, int64_t *Kr,
                     int64_t *Kc, double *Kv)
{
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < E; e++) {
        double R[9], m[4] = {1, 0, 0, 1}, xe[12], area, ue[24];
        const int64_t *c = cdof + 4 * e;
        orc_q4_rotation(x, c, xmat ? xmat + 3 * e : 0, R, m);
        orc_q4_probe_xe(x, c, R, xe, &area);
        orc_q4_probe_ue(u, c, R, ue);
        const double *P = props + Q4P_STRIDE * (pid ? pid[e] : e);
        orc_q4_kg(R, m, xe, ue, P, c, init_k[e], Kr, Kc, Kv);
    }
}

void orc_q4_m_batch(int64_t E, const int64_t *cdof, const int64_t *init_k,
                    const double *x, const double *props, const int32_t *pid,
                    int64_t *Kr, int64_t *Kc, double *Kv, int mtype)
{
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < E; e++) {
        double R[9], m[4] = {1, 0, 0, 1}, xe[12], area;
        const int64_t *c = cdof + 4 * e;
        orc_q4_rotation(x, c, 0, R, m);
        orc_q4_probe_xe(x, c, R, xe, &area);
        const double *P = props + Q4P_STRIDE * (pid ? pid[e] : e);
        orc_q4_m(R, xe, area, P, c, init_k[e], Kr, Kc, Kv, mtype);
    }
}

void orc_bc_kc0_batch(int64_t E, const int64_t *cdof, const int64_t *init_k,
                      const double *x, const double *vxy, const double *props,
                      const int32_t *pid, int64_t *Kr, int64_t *Kc, double *Kv,
                      int values_only)
{
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < E; e++) {
        double R[9], xe[6], L;
        const int64_t *c = cdof + 2 * e;
        orc_bc_rotation(x, c, vxy + 3 * e, R);
        orc_bc_probe_xe(x, c, R, xe, &L);
        const double *P = props + BCP_STRIDE * (pid ? pid[e] : e);
        orc_bc_kc0(R, L, P, c, init_k[e], Kr, Kc, Kv, values_only);
    }
}

void orc_t3_kc0_batch(int64_t E, const int64_t *cdof, const int64_t *init_k,
                      const double *x, const double *xmat, const double *props,
                      const int32_t *pid, const double *k6rot, const double *alpha,
                      int64_t *Kr, int64_t *Kc, double *Kv, int values_only)
{
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < E; e++) {
        double R[9], m[4] = {1, 0, 0, 1}, xe[9], area;
        const int64_t *c = cdof + 3 * e;
        orc_t3_rotation(x, c, xmat ? xmat + 3 * e : 0, R, m);
        orc_t3_probe_xe(x, c, R, xe, &area);
        const double *P = props + Q4P_STRIDE * (pid ? pid[e] : e);
        orc_t3_kc0(R, m, xe, area, P, k6rot[e], alpha[e], c, init_k[e], Kr, Kc, Kv, values_only);
    }
}

void orc_q4r_kc0_batch(int64_t E, const int64_t *cdof, const int64_t *init_k,
                       const double *x, const double *xmat, const double *props,
                       const int32_t *pid, const double *k6rot, const double *hg,
                       int64_t *Kr, int64_t *Kc, double *Kv, int values_only)
{
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < E; e++) {
        double R[9], m[4] = {1, 0, 0, 1}, xe[12], area;
        const int64_t *c = cdof + 4 * e;
        orc_q4_rotation(x, c, xmat ? xmat + 3 * e : 0, R, m);
        orc_q4_probe_xe(x, c, R, xe, &area);
        const double *P = props + Q4P_STRIDE * (pid ? pid[e] : e);
        orc_q4r_kc0(R, m, xe, area, P, k6rot[e], hg + 5 * e, c, init_k[e], Kr, Kc, Kv, values_only);
    }
}
