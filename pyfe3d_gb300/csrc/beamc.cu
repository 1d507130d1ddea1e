// BeamC (consistent Timoshenko beam, Luo 2008) kernels: frame, probe ue,
// KC0, KG, M.  Local 12x12 matrices follow the closed forms of
// pyfe3d/beamc.pyx (cited per function); the global matrix is R Ke R^T on
// the 3x3 sub-blocks.  Matrix kernel, per tile of 32 elements: all threads
// clear the local matrices, one full warp forms their non-zero terms in
// shared memory; each warp then turns one upper 3x3 block of the 32
// elements to the global axes in place (the matrices are symmetric: each
// transformed block is also written transposed; for KC0 and KG four of the
// ten blocks follow from the others with a sign), and every element's slots
// are streamed out with coalesced += over the whole tile.
#include "common.cuh"

namespace fe3d {
namespace {

constexpr int BNT = 64;   // threads per CTA (per-element kernels)
constexpr int BMT = 128;  // threads per CTA of the matrix kernel

struct BeamShape {  // alpha/beta of the two bending planes
    double ay, az, by, bz;
};

__device__ __forceinline__ BeamShape beam_shape(const double *P, double L) {
    BeamShape s;
    // one division for the two alphas and one for the two betas (FP64
    // divisions are costly on this part; the results agree to rounding)
    const double f = 12 * P[BP_E] / (P[BP_G] * P[BP_A] * L * L);
    s.ay = f * P[BP_IZZ];
    s.az = f * P[BP_IYY];
    const double d = 1. / ((1. - s.ay) * (1. - s.az));
    s.by = (1. - s.az) * d;
    s.bz = (1. - s.ay) * d;
    return s;
}

__device__ __forceinline__ void put(double *K, int i, int j, double v) {
    K[12 * i + j] = v;
    K[12 * j + i] = v;
}

// beamc.pyx:543-624: the 66 non-zero upper-triangle terms of KC0e.  The
// local matrices below are written into a zeroed 12x12 array.
__device__ void beam_kc0_local(double L, const double *P, double *K) {
    const double A = P[BP_A], E = P[BP_E], G = P[BP_G], Iyy = P[BP_IYY], Izz = P[BP_IZZ];
    const double Iyz = P[BP_IYZ], J = P[BP_J], Ay = P[BP_AY], Az = P[BP_AZ];
    const BeamShape s = beam_shape(P, L);
    const double ay = s.ay, az = s.az, by = s.by, bz = s.bz;
    const double L2 = L * L, iL = 1. / L, iL2 = iL * iL, iL3 = iL2 * iL;
    const double ka = A * E * iL, kt = G * J * iL;
    const double gy = A * G * L2 * ay * ay, gz = A * G * L2 * az * az;
    const double cvv = by * by * (gy + 12 * E * Izz) * iL3, cvr = by * by * (gy + 12 * E * Izz) * (0.5 * iL2);
    const double cww = bz * bz * (gz + 12 * E * Iyy) * iL3, cwr = bz * bz * (gz + 12 * E * Iyy) * (0.5 * iL2);
    const double rz1 = by * by * (gy * 0.25 + E * Izz * ay * ay - 2 * E * Izz * ay + 4 * E * Izz) * iL;
    const double rz2 = by * by * (gy * 0.25 - E * Izz * ay * ay + 2 * E * Izz * ay + 2 * E * Izz) * iL;
    const double ry1 = bz * bz * (gz * 0.25 + E * Iyy * az * az - 2 * E * Iyy * az + 4 * E * Iyy) * iL;
    const double ry2 = bz * bz * (gz * 0.25 - E * Iyy * az * az + 2 * E * Iyy * az + 2 * E * Iyy) * iL;
    const double c3 = 12 * E * Iyz * by * bz * iL3, c2 = 6 * E * Iyz * by * bz * iL2;
    const double c1a = E * Iyz * by * bz * (-ay * az + ay + az - 4) * iL;
    const double c1b = E * Iyz * by * bz * (ay * az - ay - az - 2) * iL;
    const double oz = Az * E * bz * (1 - az) * iL, oy = Ay * E * by * (1 - ay) * iL;
    const double tz = Az * G * ay * by * iL, ty = Ay * G * az * bz * iL;
    const double tz2 = Az * G * ay * by * 0.5, ty2 = Ay * G * az * bz * 0.5;
    put(K, 0, 0, ka); put(K, 6, 6, ka); put(K, 0, 6, -ka);
    put(K, 3, 3, kt); put(K, 9, 9, kt); put(K, 3, 9, -kt);
    put(K, 0, 4, oz); put(K, 0, 10, -oz); put(K, 4, 6, -oz); put(K, 6, 10, oz);
    put(K, 0, 5, -oy); put(K, 0, 11, oy); put(K, 5, 6, oy); put(K, 6, 11, -oy);
    put(K, 1, 1, cvv); put(K, 7, 7, cvv); put(K, 1, 7, -cvv);
    put(K, 1, 5, cvr); put(K, 1, 11, cvr); put(K, 5, 7, -cvr); put(K, 7, 11, -cvr);
    put(K, 5, 5, rz1); put(K, 11, 11, rz1); put(K, 5, 11, rz2);
    put(K, 2, 2, cww); put(K, 8, 8, cww); put(K, 2, 8, -cww);
    put(K, 2, 4, -cwr); put(K, 2, 10, -cwr); put(K, 4, 8, cwr); put(K, 8, 10, cwr);
    put(K, 4, 4, ry1); put(K, 10, 10, ry1); put(K, 4, 10, ry2);
    put(K, 1, 2, c3); put(K, 1, 8, -c3); put(K, 2, 7, -c3); put(K, 7, 8, c3);
    put(K, 1, 4, -c2); put(K, 1, 10, -c2); put(K, 2, 5, c2); put(K, 2, 11, c2);
    put(K, 4, 7, c2); put(K, 5, 8, -c2); put(K, 7, 10, c2); put(K, 8, 11, -c2);
    put(K, 4, 5, c1a); put(K, 10, 11, c1a); put(K, 4, 11, c1b); put(K, 5, 10, c1b);
    put(K, 1, 3, tz); put(K, 1, 9, -tz); put(K, 3, 7, -tz); put(K, 7, 9, tz);
    put(K, 2, 3, -ty); put(K, 2, 9, ty); put(K, 3, 8, ty); put(K, 8, 9, -ty);
    put(K, 3, 4, ty2); put(K, 3, 10, ty2); put(K, 4, 9, -ty2); put(K, 9, 10, -ty2);
    put(K, 3, 5, tz2); put(K, 3, 11, tz2); put(K, 5, 9, -tz2); put(K, 9, 11, -tz2);
}

// beamc.pyx:1889-2179: N = A E (u2 - u1) / L times, for each pair of bending
// planes (p, q), the 4x4 form on (d1, t1, d2, t2), t = rz (x-y) or -ry (x-z).
__device__ void beam_kg_local(double L, const double *P, const double *ue, double *K) {
    const BeamShape s = beam_shape(P, L);
    const double iL = 1. / L;
    const double N = P[BP_A] * P[BP_E] * (-ue[0] + ue[6]) * iL;
    const int dofs[2][4] = {{1, 5, 7, 11}, {2, 4, 8, 10}};
    const double sg[2][4] = {{1., 1., 1., 1.}, {1., -1., 1., -1.}};
    const double al[2] = {s.ay, s.az}, be[2] = {s.by, s.bz};
#pragma unroll
    for (int p = 0; p < 2; p++)
#pragma unroll
        for (int q = 0; q < 2; q++) {
            const double bb = be[p] * be[q], t = 5 * al[p] * al[q] - 5 * al[p] - 5 * al[q];
            const double va = bb * (t + 6) * (0.2 * iL), vb = bb * 0.1, vc = L * bb * (t + 8) * (1. / 60),
                         ve = -L * bb * (t + 2) * (1. / 60);
            const double S[4][4] = {{va, vb, -va, vb}, {vb, vc, -vb, ve}, {-va, -vb, va, -vb}, {vb, ve, -vb, vc}};
#pragma unroll
            for (int i = 0; i < 4; i++)
#pragma unroll
                for (int j = 0; j < 4; j++) K[12 * dofs[p][i] + dofs[q][j]] = N * sg[p][i] * sg[q][j] * S[i][j];
        }
}

// beamc.pyx:2246-2968: consistent mass (mtype 0).
__device__ void beam_m0_local(double L, const double *P, double *M) {
    const BeamShape s = beam_shape(P, L);
    const double ay = s.ay, az = s.az, by = s.by, bz = s.bz;
    const double r = P[BP_RHO], ry = P[BP_RHOY], rz = P[BP_RHOZ], ry2 = P[BP_RHOY2];
    const double rz2 = P[BP_RHOZ2], ryz = P[BP_RHOYZ];
    const double L2 = L * L, iL = 1. / L;
    put(M, 0, 0, L * r * (1. / 3)); put(M, 6, 6, L * r * (1. / 3)); put(M, 0, 6, L * r * (1. / 6));
    put(M, 0, 1, by * ry * 0.5); put(M, 0, 7, -by * ry * 0.5); put(M, 1, 6, by * ry * 0.5); put(M, 6, 7, -by * ry * 0.5);
    put(M, 0, 2, bz * rz * 0.5); put(M, 0, 8, -bz * rz * 0.5); put(M, 2, 6, bz * rz * 0.5); put(M, 6, 8, -bz * rz * 0.5);
    const double f04 = L * bz * rz * (1 - 4 * az) * (1. / 12), f010 = -L * bz * rz * (2 * az + 1) * (1. / 12);
    put(M, 0, 4, f04); put(M, 6, 10, f04); put(M, 0, 10, f010); put(M, 4, 6, f010);
    const double f05 = L * by * ry * (4 * ay - 1) * (1. / 12), f011 = L * by * ry * (2 * ay + 1) * (1. / 12);
    put(M, 0, 5, f05); put(M, 6, 11, f05); put(M, 0, 11, f011); put(M, 5, 6, f011);
    const double py = L2 * ay * ay * r, qy = L2 * ay * r, ly = L2 * r;
    const double vv = by * by * (70 * py - 147 * qy + 78 * ly + 252 * ry2) * ((1. / 210) * iL);
    const double vv2 = by * by * (35 * py - 63 * qy + 27 * ly - 252 * ry2) * ((1. / 210) * iL);
    const double vr = by * by * (35 * py - 77 * qy + 44 * ly + 420 * ay * ry2 + 84 * ry2) * (1. / 840);
    const double vr2 = by * by * (-35 * py + 63 * qy - 26 * ly + 420 * ay * ry2 + 84 * ry2) * (1. / 840);
    const double rr = L * by * by * (7 * py - 14 * qy + 8 * ly + 280 * ay * ay * ry2 - 140 * ay * ry2 + 112 * ry2) * (1. / 840);
    const double rr2 = L * by * by * (-7 * py + 14 * qy - 6 * ly + 140 * ay * ay * ry2 + 140 * ay * ry2 - 28 * ry2) * (1. / 840);
    put(M, 1, 1, vv); put(M, 7, 7, vv); put(M, 1, 7, vv2);
    put(M, 1, 5, vr); put(M, 7, 11, -vr); put(M, 1, 11, vr2); put(M, 5, 7, -vr2);
    put(M, 5, 5, rr); put(M, 11, 11, rr); put(M, 5, 11, rr2);
    const double pz = L2 * az * az * r, qz = L2 * az * r;
    const double ww = bz * bz * (70 * pz - 147 * qz + 78 * ly + 252 * rz2) * ((1. / 210) * iL);
    const double ww2 = bz * bz * (35 * pz - 63 * qz + 27 * ly - 252 * rz2) * ((1. / 210) * iL);
    const double wr = bz * bz * (-35 * pz + 77 * qz - 44 * ly - 420 * az * rz2 - 84 * rz2) * (1. / 840);
    const double wr2 = bz * bz * (35 * pz - 63 * qz + 26 * ly - 420 * az * rz2 - 84 * rz2) * (1. / 840);
    const double ss = L * bz * bz * (7 * pz - 14 * qz + 8 * ly + 280 * az * az * rz2 - 140 * az * rz2 + 112 * rz2) * (1. / 840);
    const double ss2 = L * bz * bz * (-7 * pz + 14 * qz - 6 * ly + 140 * az * az * rz2 + 140 * az * rz2 - 28 * rz2) * (1. / 840);
    put(M, 2, 2, ww); put(M, 8, 8, ww); put(M, 2, 8, ww2);
    put(M, 2, 4, wr); put(M, 8, 10, -wr); put(M, 2, 10, wr2); put(M, 4, 8, -wr2);
    put(M, 4, 4, ss); put(M, 10, 10, ss); put(M, 4, 10, ss2);
    const double p1 = 6 * by * bz * ryz * (0.2 * iL);
    put(M, 1, 2, p1); put(M, 7, 8, p1); put(M, 1, 8, -p1); put(M, 2, 7, -p1);
    const double cz = by * bz * ryz * (5 * az + 1) * (1. / 10), cy = by * bz * ryz * (5 * ay + 1) * (1. / 10);
    put(M, 1, 4, -cz); put(M, 1, 10, -cz); put(M, 4, 7, cz); put(M, 7, 10, cz);
    put(M, 2, 5, cy); put(M, 2, 11, cy); put(M, 5, 8, -cy); put(M, 8, 11, -cy);
    const double q1 = L * by * bz * ryz * (-20 * ay * az + 5 * ay + 5 * az - 8) * (1. / 60);
    const double q2 = L * by * bz * ryz * (-10 * ay * az - 5 * ay - 5 * az + 2) * (1. / 60);
    put(M, 4, 5, q1); put(M, 10, 11, q1); put(M, 4, 11, q2); put(M, 5, 10, q2);
    const double rp = ry2 + rz2;
    put(M, 3, 3, L * rp * (1. / 3)); put(M, 9, 9, L * rp * (1. / 3)); put(M, 3, 9, L * rp * (1. / 6));
    const double t13 = L * by * rz * (20 * ay - 21) * (1. / 60), t19 = L * by * rz * (10 * ay - 9) * (1. / 60);
    put(M, 1, 3, t13); put(M, 7, 9, t13); put(M, 1, 9, t19); put(M, 3, 7, t19);
    const double t23 = L * bz * ry * (21 - 20 * az) * (1. / 60), t29 = L * bz * ry * (9 - 10 * az) * (1. / 60);
    put(M, 2, 3, t23); put(M, 8, 9, t23); put(M, 2, 9, t29); put(M, 3, 8, t29);
    put(M, 3, 4, L2 * bz * ry * (5 * az - 6) * (1. / 120)); put(M, 9, 10, L2 * bz * ry * (6 - 5 * az) * (1. / 120));
    put(M, 3, 10, L2 * bz * ry * (4 - 5 * az) * (1. / 120)); put(M, 4, 9, L2 * bz * ry * (5 * az - 4) * (1. / 120));
    put(M, 3, 5, L2 * by * rz * (5 * ay - 6) * (1. / 120)); put(M, 9, 11, L2 * by * rz * (6 - 5 * ay) * (1. / 120));
    put(M, 3, 11, L2 * by * rz * (4 - 5 * ay) * (1. / 120)); put(M, 5, 9, L2 * by * rz * (5 * ay - 4) * (1. / 120));
}

// beamc.pyx:2969-3152: lumped mass (mtype 1), diagonal in the element frame.
__device__ void beam_m1_local(double L, const double *P, double *M) {
    const BeamShape s = beam_shape(P, L);
    const double fy = s.by * s.by * (s.ay * s.ay - 2 * s.ay + 1);
    const double fz = s.bz * s.bz * (s.az * s.az - 2 * s.az + 1);
    for (int n = 0; n < 2; n++) {
        const int o = 6 * n;
        M[13 * (o + 0)] = L * P[BP_RHO] / 2;
        M[13 * (o + 1)] = L * fy * P[BP_RHO] / 2;
        M[13 * (o + 2)] = L * fz * P[BP_RHO] / 2;
        M[13 * (o + 3)] = L * (P[BP_RHOY2] + P[BP_RHOZ2]) / 2;
        M[13 * (o + 4)] = L * fz * P[BP_RHOZ2] / 2;
        M[13 * (o + 5)] = L * fy * P[BP_RHOY2] / 2;
    }
}

// value of (T K T^T)[i][j], T = blockdiag(R, R, R, R)
__device__ __forceinline__ double rotated(const double *R, const double *K, int i, int j) {
    const int bi = i / 3, ii = i % 3, bj = j / 3, jj = j % 3;
    double s = 0.;
#pragma unroll
    for (int p = 0; p < 3; p++) {
        double t = 0.;
#pragma unroll
        for (int q = 0; q < 3; q++) t += K[12 * (3 * bi + p) + 3 * bj + q] * R[3 * jj + q];
        s += R[3 * ii + p] * t;
    }
    return s;
}

struct BeamArgs {
    int64_t E;
    const int64_t *cdof, *init_k;
    const double *R, *length, *ue;
    const double *props;
    int64_t nprops;
    const int32_t *pid;
    int64_t *Kr, *Kc;
    double *Kv;
    int64_t nk;
    int write_idx;
    int *err;
};

constexpr int BT = 32;       // elements per tile of the matrix kernel
constexpr int BSTR = 145;    // staged doubles per element (odd: banks spread)

// kind: 0 KC0, 1 KG, 2 M (mtype 0), 3 M (mtype 1)
template <int KIND>
__global__ void __launch_bounds__(BMT) beamc_matrix_kernel(BeamArgs a) {
    __shared__ double sK[BT * BSTR];
    __shared__ double sR[BT][9];
    __shared__ long long sk0[BT], sc[BT][2];
    __shared__ int sval[BT];
    constexpr int size = (KIND == 3) ? 36 : 144;
    const int tid = threadIdx.x;
    const int64_t ntiles = (a.E + BT - 1) / BT;
    for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int64_t e0 = tile * BT;
        __syncthreads();
        // all threads clear the local matrices; the closed forms then write
        // their non-zero terms only
        for (int i = tid; i < BT * BSTR; i += BMT) sK[i] = 0.;
        __syncthreads();
        if (tid < BT) {
            const int64_t e = e0 + tid;
            sval[tid] = 0;
            if (e < a.E) {
                const long long c1 = a.cdof[2 * e], c2 = a.cdof[2 * e + 1];
                const long long k0 = a.init_k[e];
                const int64_t p = a.pid ? (int64_t)a.pid[e] : e;
                if (c1 < 0 || c2 < 0 || k0 < 0 || k0 + size > a.nk || p < 0 || p >= a.nprops) {
                    raise_error(a.err, kErrBounds);
                } else {
                    const double *P = a.props + (int64_t)BP_STRIDE * p;
                    const double L = a.length[e];
                    double *K = sK + tid * BSTR;
                    if (KIND == 0) beam_kc0_local(L, P, K);
                    if (KIND == 1) beam_kg_local(L, P, a.ue + 12 * e, K);
                    if (KIND == 2) beam_m0_local(L, P, K);
                    if (KIND == 3) beam_m1_local(L, P, K);
#pragma unroll
                    for (int i = 0; i < 9; i++) sR[tid][i] = a.R[9 * e + i];
                    sk0[tid] = k0;
                    sc[tid][0] = c1;
                    sc[tid][1] = c2;
                    sval[tid] = 1;
                }
            }
        }
        __syncthreads();
        // the upper 3x3 blocks (bi <= bj; diagonal blocks only for the lumped
        // mass) turned to the global axes in place, R Kb R^T.  KC0 and KG
        // vanish on a rigid translation, and their closed forms hold that
        // exactly (the node-2 translation rows and columns are the node-1
        // ones negated), so only six blocks are turned and the other four
        // follow with a sign: T1T2 = -T1T1, T2T2 = T1T1, R1T2 = -(T1R1)^T,
        // T2R2 = -T1R2.
        constexpr int NB = (KIND == 3) ? 4 : (KIND == 2) ? 10 : 6;
        // block q of element el: the 32 lanes of a warp turn the same block
        // of 32 elements, so the structured forms below stay warp-uniform
        for (int w = tid; w < BT * NB; w += BMT) {
            const int q = w / BT, el = w - q * BT;
            if (!sval[el]) continue;
            int bi, bj;
            if (KIND == 3) {
                bi = bj = q;
            } else if (KIND == 2) {
                bi = q < 4 ? 0 : q < 7 ? 1 : q < 9 ? 2 : 3;
                bj = bi + q - (bi == 0 ? 0 : bi == 1 ? 4 : bi == 2 ? 7 : 9);
            } else {
                // (0,0) (0,1) (0,3) (1,1) (1,3) (3,3)
                bi = q < 3 ? 0 : q < 5 ? 1 : 3;
                bj = q == 0 ? 0 : q == 1 ? 1 : q == 2 ? 3 : q == 3 ? 1 : 3;
            }
            double *K = sK + el * BSTR;
            const double *R = sR[el];
            double kb[3][3], t[3][3], g[3][3];
#pragma unroll
            for (int i = 0; i < 3; i++)
#pragma unroll
                for (int j = 0; j < 3; j++) kb[i][j] = K[12 * (3 * bi + i) + 3 * bj + j];
            // t = Kb R^T.  KC0 and KG: T1T1 is [k00 0 0; 0 k11 k12; 0 k21 k22]
            // (the axial translation couples with itself only) and the first
            // entry of T1R1 and T1R2 is zero; the products with those exact
            // zeros are left out (they add nothing)
            if (KIND <= 1 && q == 0) {
#pragma unroll
                for (int j = 0; j < 3; j++) {
                    t[0][j] = kb[0][0] * R[3 * j + 0];
                    t[1][j] = kb[1][1] * R[3 * j + 1] + kb[1][2] * R[3 * j + 2];
                    t[2][j] = kb[2][1] * R[3 * j + 1] + kb[2][2] * R[3 * j + 2];
                }
            } else if (KIND <= 1 && (q == 1 || q == 2)) {
#pragma unroll
                for (int j = 0; j < 3; j++) {
                    t[0][j] = kb[0][1] * R[3 * j + 1] + kb[0][2] * R[3 * j + 2];
#pragma unroll
                    for (int p = 1; p < 3; p++)
                        t[p][j] = kb[p][0] * R[3 * j + 0] + kb[p][1] * R[3 * j + 1] + kb[p][2] * R[3 * j + 2];
                }
            } else {
#pragma unroll
                for (int p = 0; p < 3; p++)
#pragma unroll
                    for (int j = 0; j < 3; j++)
                        t[p][j] = kb[p][0] * R[3 * j + 0] + kb[p][1] * R[3 * j + 1] + kb[p][2] * R[3 * j + 2];
            }
            // G = R t; a diagonal block is symmetric: its upper triangle is
            // formed and mirrored
            if (bi == bj) {
#pragma unroll
                for (int i = 0; i < 3; i++)
#pragma unroll
                    for (int j = i; j < 3; j++) {
                        g[i][j] = R[3 * i + 0] * t[0][j] + R[3 * i + 1] * t[1][j] + R[3 * i + 2] * t[2][j];
                        g[j][i] = g[i][j];
                    }
            } else {
#pragma unroll
                for (int i = 0; i < 3; i++)
#pragma unroll
                    for (int j = 0; j < 3; j++)
                        g[i][j] = R[3 * i + 0] * t[0][j] + R[3 * i + 1] * t[1][j] + R[3 * i + 2] * t[2][j];
            }
#pragma unroll
            for (int i = 0; i < 3; i++)
#pragma unroll
                for (int j = 0; j < 3; j++) {
                    const double v = g[i][j];
                    const int r = 3 * bi + i, c = 3 * bj + j;
                    K[12 * r + c] = v;
                    if (bi != bj) K[12 * c + r] = v;
                    if (KIND <= 1) {
                        if (bi == 0 && bj == 0) {
                            K[12 * r + 6 + c] = -v;        // T1T2
                            K[12 * (6 + c) + r] = -v;      // T2T1
                            K[12 * (6 + r) + 6 + c] = v;   // T2T2
                        } else if (bi == 0 && bj == 1) {
                            K[12 * c + 6 + r] = -v;        // R1T2 = -(T1R1)^T
                            K[12 * (6 + r) + c] = -v;      // T2R1
                        } else if (bi == 0 && bj == 3) {
                            K[12 * (6 + r) + c] = -v;      // T2R2 = -T1R2
                            K[12 * c + 6 + r] = -v;        // R2T2
                        }
                    }
                }
        }
        __syncthreads();
        const int nel = (int)((a.E - e0) < BT ? (a.E - e0) : BT);
        // in batches of 8 slots per thread: the caller's values first (all
        // loads in flight), then the stores
        for (int i0 = tid; i0 < nel * size; i0 += 8 * BMT) {
            double old[8];
#pragma unroll
            for (int u = 0; u < 8; u++) {
                const int i = i0 + u * BMT;
                const int el = i / size;
                old[u] = (i < nel * size && sval[el]) ? a.Kv[sk0[el] + (i - el * size)] : 0.;
            }
#pragma unroll
            for (int u = 0; u < 8; u++) {
                const int i = i0 + u * BMT;
                if (i >= nel * size) break;
                const int el = i / size, j = i - el * size;
                if (!sval[el]) continue;
                const double *K = sK + el * BSTR;
                const long long k = sk0[el] + j;
                int row, col;
                if (KIND == 3) {
                    // 4 diagonal 3x3 blocks, row-major within each
                    const int blk = j / 9, r = j - 9 * blk;
                    row = 3 * blk + r / 3;
                    col = 3 * blk + r % 3;
                } else {
                    row = j / 12;
                    col = j - 12 * row;
                }
                a.Kv[k] = old[u] + K[12 * row + col];
                if (a.write_idx || KIND == 3) {
                    a.Kr[k] = sc[el][row / 6] + row % 6;
                    a.Kc[k] = sc[el][col / 6] + col % 6;
                }
            }
        }
    }
}

// BeamC.update_probe_finte / update_fint (beamc.pyx:352-486, 1354-1390):
// finte = KC0e ue in the element frame (the same local matrix as update_KC0)
// and fint[c + .] += R finte per node block.  finte (12 per element) and
// fint may each be NULL.  fint accumulates with FP64 atomics (elements that
// share a node add in any order).
__global__ void __launch_bounds__(BNT) beamc_fint_kernel(int64_t E, const int64_t *cdof, const double *R_in,
                                                         const double *length, const double *ue,
                                                         const double *props, int64_t nprops, const int32_t *pid,
                                                         double *fint, int64_t nf, double *finte, int *err) {
    const int64_t e = blockIdx.x * (int64_t)BNT + threadIdx.x;
    if (e >= E) return;
    const long long c1 = cdof[2 * e], c2 = cdof[2 * e + 1];
    const int64_t p = pid ? (int64_t)pid[e] : e;
    if (p < 0 || p >= nprops || (fint && (c1 < 0 || c2 < 0 || c1 + 6 > nf || c2 + 6 > nf))) {
        raise_error(err, kErrBounds);
        return;
    }
    double K[144] = {};
    beam_kc0_local(length[e], props + (int64_t)BP_STRIDE * p, K);
    double f[12];
    for (int i = 0; i < 12; i++) {
        double t = 0.;
        for (int j = 0; j < 12; j++) t += K[12 * i + j] * ue[12 * e + j];
        f[i] = t;
    }
    if (finte)
        for (int i = 0; i < 12; i++) finte[12 * e + i] = f[i];
    if (fint) {
        const double *R = R_in + 9 * e;
        const long long cc[2] = {c1, c2};
        for (int blk = 0; blk < 4; blk++)
            for (int i = 0; i < 3; i++)
                atomicAdd(fint + cc[blk / 2] + 3 * (blk % 2) + i,
                          R[3 * i] * f[3 * blk] + R[3 * i + 1] * f[3 * blk + 1] + R[3 * i + 2] * f[3 * blk + 2]);
    }
}

__global__ void beamc_frame_kernel(int64_t E, const int64_t *cdof, const double *x, int64_t nx,
                                   const double *vxy, int vxy_stride, double *Ro, double *xeo,
                                   double *Lo, int *err) {
    const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= E) return;
    const long long c1 = cdof[2 * e], c2 = cdof[2 * e + 1];
    if (c1 < 0 || c2 < 0 || c1 / 2 + 3 > nx || c2 / 2 + 3 > nx) {
        raise_error(err, kErrBounds);
        return;
    }
    const double *p1 = x + c1 / 2, *p2 = x + c2 / 2, *v = vxy + (int64_t)vxy_stride * e;
    double xa[3], z[3], y[3], t;
    for (int i = 0; i < 3; i++) xa[i] = p2[i] - p1[i];
    t = sqrt(xa[0] * xa[0] + xa[1] * xa[1] + xa[2] * xa[2]);
    xa[0] /= t; xa[1] /= t; xa[2] /= t;
    z[0] = xa[1] * v[2] - xa[2] * v[1];
    z[1] = -xa[0] * v[2] + xa[2] * v[0];
    z[2] = xa[0] * v[1] - xa[1] * v[0];
    t = sqrt(z[0] * z[0] + z[1] * z[1] + z[2] * z[2]);
    z[0] /= t; z[1] /= t; z[2] /= t;
    y[0] = -xa[1] * z[2] + xa[2] * z[1];
    y[1] = xa[0] * z[2] - xa[2] * z[0];
    y[2] = -xa[0] * z[1] + xa[1] * z[0];
    t = sqrt(y[0] * y[0] + y[1] * y[1] + y[2] * y[2]);
    y[0] /= t; y[1] /= t; y[2] /= t;
    double R[9];
    for (int i = 0; i < 3; i++) {
        R[3 * i] = xa[i];
        R[3 * i + 1] = y[i];
        R[3 * i + 2] = z[i];
    }
    if (Ro)
        for (int i = 0; i < 9; i++) Ro[9 * e + i] = R[i];
    double xe[6];
    const double *pp[2] = {p1, p2};
    for (int j = 0; j < 2; j++) {
        xe[3 * j + 0] = R[0] * pp[j][0] + R[3] * pp[j][1] + R[6] * pp[j][2];
        xe[3 * j + 1] = R[1] * pp[j][0] + R[4] * pp[j][1] + R[7] * pp[j][2];
        xe[3 * j + 2] = R[2] * pp[j][0] + R[5] * pp[j][1] + R[8] * pp[j][2];
    }
    if (xeo)
        for (int i = 0; i < 6; i++) xeo[6 * e + i] = xe[i];
    if (Lo) {
        const double dx = xe[3] - xe[0], dy = xe[4] - xe[1], dz = xe[5] - xe[2];
        Lo[e] = sqrt(dx * dx + dy * dy + dz * dz);
    }
}

// BeamC.update_probe_xe with the frame held by the element (beamc.pyx:287-349).
__global__ void beamc_probe_xe_kernel(int64_t E, const int64_t *cdof, const double *x, int64_t nx,
                                      const double *R, double *xeo, double *Lo, int *err) {
    const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= E) return;
    const double *r = R + 9 * e;
    double xe[6];
    for (int j = 0; j < 2; j++) {
        const long long c = cdof[2 * e + j];
        if (c < 0 || c / 2 + 3 > nx) {
            raise_error(err, kErrBounds);
            return;
        }
        const double *p = x + c / 2;
        xe[3 * j + 0] = r[0] * p[0] + r[3] * p[1] + r[6] * p[2];
        xe[3 * j + 1] = r[1] * p[0] + r[4] * p[1] + r[7] * p[2];
        xe[3 * j + 2] = r[2] * p[0] + r[5] * p[1] + r[8] * p[2];
    }
    if (xeo)
        for (int i = 0; i < 6; i++) xeo[6 * e + i] = xe[i];
    if (Lo) {
        const double dx = xe[3] - xe[0], dy = xe[4] - xe[1], dz = xe[5] - xe[2];
        Lo[e] = sqrt(dx * dx + dy * dy + dz * dz);
    }
}

__global__ void beamc_probe_ue_kernel(int64_t E, const int64_t *cdof, const double *u, int64_t nu,
                                      const double *R, double *ue, int *err) {
    const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= E) return;
    const double *r = R + 9 * e;
    for (int j = 0; j < 2; j++) {
        const long long c = cdof[2 * e + j];
        if (c < 0 || c + 6 > nu) {
            raise_error(err, kErrBounds);
            return;
        }
        for (int g = 0; g < 2; g++) {
            const double *p = u + c + 3 * g;
            double *q = ue + 12 * e + 6 * j + 3 * g;
            q[0] = r[0] * p[0] + r[3] * p[1] + r[6] * p[2];
            q[1] = r[1] * p[0] + r[4] * p[1] + r[7] * p[2];
            q[2] = r[2] * p[0] + r[5] * p[1] + r[8] * p[2];
        }
    }
}

inline unsigned beam_grid(int64_t E) { return (unsigned)((E + BNT - 1) / BNT); }
template <int KIND>
unsigned beam_mgrid(int64_t E) {
    static const int per_sm = resident_per_sm(beamc_matrix_kernel<KIND>, BMT, 0);
    const int64_t g = (E + BT - 1) / BT, cap = (int64_t)kSMs * per_sm;
    return (unsigned)(g < cap ? (g < 1 ? 1 : g) : cap);
}

}  // namespace
}  // namespace fe3d

using namespace fe3d;

extern "C" int fe3d_beamc_frame(int64_t E, const int64_t *cdof, const double *x, int64_t nx,
                                const double *vxy, int vxy_stride, double *R, double *xe,
                                double *length, int *err, void *stream) {
    if (E < 0 || (vxy_stride != 0 && vxy_stride != 3)) return FE3D_ERR_ARG;
    if (E == 0) return FE3D_OK;
    if (!cdof || !x || !vxy) return FE3D_ERR_ARG;
    beamc_frame_kernel<<<(unsigned)((E + 127) / 128), 128, 0, as_stream(stream)>>>(
        E, cdof, x, nx, vxy, vxy_stride, R, xe, length, err);
    FE3D_CHECK_LAUNCH();
    return FE3D_OK;
}

extern "C" int fe3d_beamc_probe_xe(int64_t E, const int64_t *cdof, const double *x, int64_t nx,
                                   const double *R, double *xe, double *length, int *err,
                                   void *stream) {
    if (E < 0) return FE3D_ERR_ARG;
    if (E == 0) return FE3D_OK;
    if (!cdof || !x || !R) return FE3D_ERR_ARG;
    beamc_probe_xe_kernel<<<(unsigned)((E + 127) / 128), 128, 0, as_stream(stream)>>>(E, cdof, x, nx,
                                                                                       R, xe, length, err);
    FE3D_CHECK_LAUNCH();
    return FE3D_OK;
}

extern "C" int fe3d_beamc_probe_ue(int64_t E, const int64_t *cdof, const double *u, int64_t nu,
                                   const double *R, double *ue, int *err, void *stream) {
    if (E < 0) return FE3D_ERR_ARG;
    if (E == 0) return FE3D_OK;
    if (!cdof || !u || !R || !ue) return FE3D_ERR_ARG;
    beamc_probe_ue_kernel<<<(unsigned)((E + 127) / 128), 128, 0, as_stream(stream)>>>(E, cdof, u, nu,
                                                                                       R, ue, err);
    FE3D_CHECK_LAUNCH();
    return FE3D_OK;
}

static int beam_common(int64_t E, const int64_t *cdof, const int64_t *init_k, const double *R,
                       const double *length, const double *props, int64_t nprops, double *Kv) {
    if (E < 0) return FE3D_ERR_ARG;
    if (E > 0 && (!cdof || !init_k || !R || !length || !props || !Kv || nprops <= 0))
        return FE3D_ERR_ARG;
    return FE3D_OK;
}

extern "C" int fe3d_beamc_kc0(int64_t E, const int64_t *cdof, const int64_t *init_k,
                              const double *R, const double *length, const double *props,
                              int64_t nprops, const int32_t *pid, int64_t *Kr, int64_t *Kc,
                              double *Kv, int64_t nk, int values_only, int *err, void *stream) {
    int rc = beam_common(E, cdof, init_k, R, length, props, nprops, Kv);
    if (rc) return rc;
    if (E == 0) return FE3D_OK;
    if (!values_only && (!Kr || !Kc)) return FE3D_ERR_ARG;
    BeamArgs a{E, cdof, init_k, R, length, nullptr, props, nprops, pid, Kr, Kc, Kv, nk,
               values_only == 0, err};
    beamc_matrix_kernel<0><<<beam_mgrid<0>(E), BMT, 0, as_stream(stream)>>>(a);
    FE3D_CHECK_LAUNCH();
    return FE3D_OK;
}

extern "C" int fe3d_beamc_kg(int64_t E, const int64_t *cdof, const int64_t *init_k,
                             const double *R, const double *length, const double *ue,
                             const double *props, int64_t nprops, const int32_t *pid, int64_t *Kr,
                             int64_t *Kc, double *Kv, int64_t nk, int values_only, int *err,
                             void *stream) {
    int rc = beam_common(E, cdof, init_k, R, length, props, nprops, Kv);
    if (rc) return rc;
    if (E == 0) return FE3D_OK;
    if (!ue || (!values_only && (!Kr || !Kc))) return FE3D_ERR_ARG;
    BeamArgs a{E, cdof, init_k, R, length, ue, props, nprops, pid, Kr, Kc, Kv, nk,
               values_only == 0, err};
    beamc_matrix_kernel<1><<<beam_mgrid<1>(E), BMT, 0, as_stream(stream)>>>(a);
    FE3D_CHECK_LAUNCH();
    return FE3D_OK;
}

extern "C" int fe3d_beamc_m(int64_t E, const int64_t *cdof, const int64_t *init_k,
                            const double *R, const double *length, const double *props,
                            int64_t nprops, const int32_t *pid, int64_t *Kr, int64_t *Kc,
                            double *Kv, int64_t nk, int mtype, int *err, void *stream) {
    int rc = beam_common(E, cdof, init_k, R, length, props, nprops, Kv);
    if (rc) return rc;
    if (mtype != 0 && mtype != 1) return FE3D_ERR_ARG;
    if (E == 0) return FE3D_OK;
    if (!Kr || !Kc) return FE3D_ERR_ARG;
    BeamArgs a{E, cdof, init_k, R, length, nullptr, props, nprops, pid, Kr, Kc, Kv, nk, 1, err};
    if (mtype == 0) beamc_matrix_kernel<2><<<beam_mgrid<2>(E), BMT, 0, as_stream(stream)>>>(a);
    else beamc_matrix_kernel<3><<<beam_mgrid<3>(E), BMT, 0, as_stream(stream)>>>(a);
    FE3D_CHECK_LAUNCH();
    return FE3D_OK;
}

extern "C" int fe3d_beamc_fint(int64_t E, const int64_t *cdof, const double *R, const double *length,
                               const double *ue, const double *props, int64_t nprops, const int32_t *pid,
                               double *fint, int64_t nf, double *finte, int *err, void *stream) {
    if (E < 0) return FE3D_ERR_ARG;
    if (E == 0) return FE3D_OK;
    if (!cdof || !length || !ue || !props || nprops <= 0 || (!fint && !finte) || (fint && !R))
        return FE3D_ERR_ARG;
    beamc_fint_kernel<<<beam_grid(E), BNT, 0, as_stream(stream)>>>(E, cdof, R, length, ue, props, nprops, pid,
                                                                   fint, nf, finte, err);
    FE3D_CHECK_LAUNCH();
    return FE3D_OK;
}

extern "C" int fe3d_version(void) { return 1; }

extern "C" const char *fe3d_error_string(int code) {
    switch (code) {
        case FE3D_OK: return "ok";
        case FE3D_ERR_ARG: return "invalid argument";
        case FE3D_ERR_LAUNCH: return "kernel launch failed";
        case FE3D_ERR_CUDA: return "CUDA runtime error";
        case FE3D_ERR_BOUNDS: return "offset outside the caller's buffers";
        case FE3D_ERR_NOMEM: return "device allocation failed";
        case FE3D_ERR_STATE: return "object used in the wrong state";
        case FE3D_ERR_TOO_LARGE: return "size above the allocation-free maximum (FE3D_NOALLOC_MAX_ROWS rows)";
        default: return "unknown error";
    }
}
