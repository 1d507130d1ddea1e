/*
 * fe3d_gb300.h -- C ABI of the GB300 (sm_103a) element-assembly-and-solve
 * library that stands behind the pyfe3d Quad4/BeamC element API.
 *
 * Conventions
 *  - Every pointer argument is a DEVICE pointer unless stated otherwise.
 *  - Index arrays are int64 (pyfe3d's INT on LP64 hosts), values are double.
 *  - `stream` is a cudaStream_t passed as void* (NULL = legacy default).
 *  - `err` is an optional device int: kernels OR bit 1 into it when an
 *    element's offsets fall outside the caller's buffers (that element is
 *    skipped).  Pass NULL to skip the checks' reporting.
 *  - Every entry point returns FE3D_OK (0) or a negative FE3D_ERR_* code;
 *    argument errors are detected before any launch.
 *  - Values are accumulated (+=) and indices overwritten, exactly like the
 *    reference's update_* methods; slots a method does not touch are left
 *    unchanged.
 *
 * Property records (row-major, one record per property id):
 *  shell, FE3D_SHELL_PROP_STRIDE doubles: A11 A12 A16 A22 A26 A66
 *     B11 B12 B16 B22 B26 B66 D11 D12 D16 D22 D26 D66 E44 E45 E55
 *     scf_k13 scf_k23 h intrho intrhoz intrhoz2 (pad)
 *     -- the ShellProp fields read by pyfe3d/quad4.pyx:826-843,903-905,3119-3121
 *  beam, FE3D_BEAM_PROP_STRIDE doubles: A E G Iyy Izz Iyz J Ay Az intrho
 *     intrhoy intrhoz intrhoy2 intrhoz2 intrhoyz (pad)
 *     -- the BeamProp fields of pyfe3d/beamprop.pxd:1-3
 */
#ifndef FE3D_GB300_H
#define FE3D_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FE3D_OK 0
#define FE3D_ERR_ARG (-1)      /* invalid argument (size, pointer, mode) */
#define FE3D_ERR_LAUNCH (-2)   /* kernel launch failed */
#define FE3D_ERR_CUDA (-3)     /* CUDA runtime call failed */
#define FE3D_ERR_BOUNDS (-4)   /* device detected an out-of-range offset */
#define FE3D_ERR_NOMEM (-5)    /* device allocation failed */
#define FE3D_ERR_STATE (-6)    /* object used in the wrong state */

#define FE3D_SHELL_PROP_STRIDE 28
#define FE3D_BEAM_PROP_STRIDE 16

#define FE3D_QUAD4_KC0_SIZE 576 /* Quad4Data.KC0_SPARSE_SIZE, quad4.pyx:175 */
#define FE3D_QUAD4_KG_SIZE 144  /* Quad4Data.KG_SPARSE_SIZE,  quad4.pyx:176 */
#define FE3D_QUAD4_M_SIZE 480   /* Quad4Data.M_SPARSE_SIZE,   quad4.pyx:177 */
#define FE3D_BEAMC_KC0_SIZE 144 /* BeamCData, beamc.pyx:44-46 */
#define FE3D_BEAMC_KG_SIZE 144
#define FE3D_BEAMC_M_SIZE 144

int fe3d_version(void);
const char *fe3d_error_string(int code);

/* ------------------------------------------------------------------ Quad4
 * Element e has the 4 DOF offsets cdof[4e..4e+3] (Quad4.c1..c4: 6 x node
 * position) and its coordinates at x[cdof/2 .. +2].
 */

/* Quad4.update_rotation_matrix + Quad4.update_probe_xe for E elements
 * (pyfe3d/quad4.pyx:491-624, 682-752).  xmat: NULL, one global vector
 * (xmat_stride 0) or one per element (xmat_stride 3).  m is in/out
 * (m11 m12 m21 m22), overwritten only where the material vector projects,
 * as in the reference.  R (9/element, row-major r11..r33), xe (12),
 * area (1) may each be NULL. */
int fe3d_quad4_frame(int64_t E, const int64_t *cdof, const double *x, int64_t nx,
                     const double *xmat, int xmat_stride, double *R, double *m,
                     double *xe, double *area, int *err, void *stream);

/* Quad4.update_probe_xe + update_area with the frame R the element holds
 * (pyfe3d/quad4.pyx:682-752): xe[12e..] = R^T x, area by the shoelace rule. */
int fe3d_quad4_probe_xe(int64_t E, const int64_t *cdof, const double *x, int64_t nx,
                        const double *R, double *xe, double *area, int *err, void *stream);

/* Quad4.update_probe_ue (pyfe3d/quad4.pyx:627-679): ue[24e..] = R^T u. */
int fe3d_quad4_probe_ue(int64_t E, const int64_t *cdof, const double *u, int64_t nu,
                        const double *R, double *ue, int *err, void *stream);

/* Quad4.update_KC0 (pyfe3d/quad4.pyx:1204-1313 with _update_probe_KC0ve
 * :755-1171).  Two input modes:
 *   fused  (x != NULL): the frame is computed on the fly from x (+xmat);
 *   probe  (x == NULL): R, m, xe, area per element are read (the state a
 *                       Quad4 object holds after its frame/probe updates).
 * props: nprops shell records; pid[e] selects element e's record (pid NULL:
 * record e).  Writes Kv[init_k[e] + 0..575] += values and, unless
 * values_only, Kr/Kc; nk is the length of Kr/Kc/Kv. */
int fe3d_quad4_kc0(int64_t E, const int64_t *cdof, const int64_t *init_k,
                   const double *x, int64_t nx, const double *xmat, int xmat_stride,
                   const double *R, const double *m, const double *xe, const double *area,
                   const double *props, int64_t nprops, const int32_t *pid,
                   int64_t *Kr, int64_t *Kc, double *Kv, int64_t nk, int values_only,
                   int *err, void *stream);

/* Quad4.update_KC0 (pyfe3d/quad4.pyx:1204-1313) with every array in HOST
 * memory (pinned for full overlap), the way the reference's callers hold
 * them: elements stream through the GPU in chunks (upload of offsets, ids
 * and the current values, the KC0 kernel, download of rows, columns and
 * values, on three streams, three staging sets), so transfers overlap the
 * compute.  Requires the reference's contiguous offsets init_k[e] =
 * init_k[0] + 576 e (else FE3D_ERR_ARG: use fe3d_quad4_kc0 on device
 * arrays); no material direction (xmat).  props: nprops records, pid[e]
 * selects element e's record (pid NULL: record e, nprops >= E).  chunk <= 0
 * picks 65536 elements.  err (host int, may be NULL) is OR-ed with the
 * device error bits.  Device staging is kept between calls.  Synchronises. */
int fe3d_quad4_kc0_host(int64_t E, const int64_t *cdof, const int64_t *init_k, const double *x, int64_t nx,
                        const double *props, int64_t nprops, const int32_t *pid, int64_t *Kr, int64_t *Kc,
                        double *Kv, int64_t nk, int values_only, int64_t chunk, int *err, void *stream);

/* Quad4.update_KG (pyfe3d/quad4.pyx:1365-2257).  Fused mode (x != NULL)
 * gathers ue from the global displacement u (length nu); probe mode reads
 * R, m, xe and ue (24/element).  Indices are written unless Kr and Kc are
 * both NULL (Quad4R.update_KG with update_KGv_only != 0; its matrix is the
 * Quad4 one, quad4r.pyx:4681-5572). */
int fe3d_quad4_kg(int64_t E, const int64_t *cdof, const int64_t *init_k,
                  const double *x, int64_t nx, const double *xmat, int xmat_stride,
                  const double *u, int64_t nu,
                  const double *R, const double *m, const double *xe, const double *ue,
                  const double *props, int64_t nprops, const int32_t *pid,
                  int64_t *Kr, int64_t *Kc, double *Kv, int64_t nk, int *err, void *stream);

/* Quad4.update_M (pyfe3d/quad4.pyx:3083-9489), mtype 0 (consistent),
 * 1 (reduced) or 2 (lumped; 288 of the 480 slots are written). */
int fe3d_quad4_m(int64_t E, const int64_t *cdof, const int64_t *init_k,
                 const double *x, int64_t nx,
                 const double *R, const double *xe, const double *area,
                 const double *props, int64_t nprops, const int32_t *pid,
                 int64_t *Kr, int64_t *Kc, double *Kv, int64_t nk, int mtype,
                 int *err, void *stream);

/* Quad4.update_fint (pyfe3d/quad4.pyx:1174-1201, 1316-1362):
 * fint[cdof + .] += R (KC0e ue) for every element (probe mode inputs). */
int fe3d_quad4_fint(int64_t E, const int64_t *cdof, const double *R, const double *m,
                    const double *xe, const double *area, const double *ue,
                    const double *props, int64_t nprops, const int32_t *pid,
                    double *fint, int64_t nf, int *err, void *stream);

/* Quad4.update_probe_finte (pyfe3d/quad4.pyx:1174-1201) for every element:
 * finte[24e..] = KC0e ue in the element frame; with fint also update_fint.
 * fint or finte may be NULL (not both). */
int fe3d_quad4_finte(int64_t E, const int64_t *cdof, const double *R, const double *m,
                     const double *xe, const double *area, const double *ue,
                     const double *props, int64_t nprops, const int32_t *pid,
                     double *fint, int64_t nf, double *finte, int *err, void *stream);

/* Quad4.update_KG_given_stress (pyfe3d/quad4.pyx:2259-3081): KG of a constant
 * stress state (Nxx, Nyy, Nxy) per element (nstress_stride 3) or shared by
 * all (nstress_stride 0), 2x2 Gauss points, 144 slots, indices written
 * unless Kr and Kc are both NULL (Quad4R.update_KG_given_stress with
 * update_KGv_only != 0, quad4r.pyx:5574-6396).
 * Fused mode (x != NULL, frame from x and xmat) or probe mode (R, xe). */
int fe3d_quad4_kg_given_stress(int64_t E, const int64_t *cdof, const int64_t *init_k,
                               const double *x, int64_t nx, const double *xmat, int xmat_stride,
                               const double *R, const double *xe, const double *nstress, int nstress_stride,
                               int64_t *Kr, int64_t *Kc, double *Kv, int64_t nk, int *err, void *stream);

/* ShellProp records of isotropic plates built on the device, one per entry
 * (shellprop_utils.isotropic_plate: shellprop.pyx:278-341, 485-549, 568-621):
 * records[28 i..] from h, E, nu, rho, offset (each an array with stride 1 or
 * a scalar with stride 0; rho and offset may be NULL for 0). */
int fe3d_isotropic_plate_records(int64_t n, const double *h, int h_stride, const double *E, int E_stride,
                                 const double *nu, int nu_stride, const double *rho, int rho_stride,
                                 const double *offset, int offset_stride, int calc_scf, double *records,
                                 void *stream);

/* ShellProp records of laminates built on the device, one per entry
 * (shellprop_utils.laminated_plate: the lamina constants of
 * shellprop_utils.py:13-93, Lamina.rebuild shellprop.pyx:278-341,
 * calc_constitutive_matrix :568-621, calc_scf :485-549): nply plies per
 * record; theta (degrees), plyt, rho hold nply values per record and lam
 * 6 per ply (E11 E22 nu12 G12 G13 G23); each array's record stride is 0 (one
 * stack for all records) or at least its per-record size; offset has stride
 * 0 or 1; rho and offset may be NULL for 0. */
int fe3d_laminate_records(int64_t n, int nply, const double *theta, int64_t theta_rs, const double *plyt,
                          int64_t plyt_rs, const double *lam, int64_t lam_rs, const double *rho, int64_t rho_rs,
                          const double *offset, int64_t offset_rs, int calc_scf, double *records, void *stream);

/* ------------------------------------------------------------------ Tria3R / Quad4R
 * Reduced-integration shells.  Tria3R element e has the 3 DOF offsets
 * cdof[3e..3e+2]; Quad4R uses the Quad4 layout.  Quad4R's frame, probes,
 * KG, KG of given stress and mass matrices are the Quad4 ones
 * (quad4r.pyx:286-548, 4681-12788 restate quad4.pyx:491-752, 1365-9489):
 * use the fe3d_quad4_* entry points for them.  k6rot (Tria3R/Quad4R.K6ROT)
 * is one value for all elements (k6rot_stride 0) or one per element (1).
 */

/* Tria3R.update_rotation_matrix + update_probe_xe + update_area for E
 * elements (pyfe3d/tria3r.pyx:294-547); arguments as fe3d_quad4_frame, xe
 * holds 9 doubles per element. */
int fe3d_tria3r_frame(int64_t E, const int64_t *cdof, const double *x, int64_t nx,
                      const double *xmat, int xmat_stride, double *R, double *m,
                      double *xe, double *area, int *err, void *stream);

/* Tria3R.update_probe_xe + update_area with the element's frame R
 * (pyfe3d/tria3r.pyx:480-547). */
int fe3d_tria3r_probe_xe(int64_t E, const int64_t *cdof, const double *x, int64_t nx,
                         const double *R, double *xe, double *area, int *err, void *stream);

/* Tria3R.update_probe_ue (pyfe3d/tria3r.pyx:426-477): ue[18e..] = R^T u. */
int fe3d_tria3r_probe_ue(int64_t E, const int64_t *cdof, const double *u, int64_t nu,
                         const double *R, double *ue, int *err, void *stream);

/* Tria3R.update_KC0 (pyfe3d/tria3r.pyx:950-2960): 324 slots per element,
 * row-major 18x18.  Fused (x != NULL) or probe mode (R, m, xe, area) as
 * fe3d_quad4_kc0.  alpha: alpha_shear_locking, alpha_stride 0 or 1.  As in
 * the reference, the drilling DOF rz enters KC0 only through its diagonal
 * rz_a - rz_a terms. */
int fe3d_tria3r_kc0(int64_t E, const int64_t *cdof, const int64_t *init_k,
                    const double *x, int64_t nx, const double *xmat, int xmat_stride,
                    const double *R, const double *m, const double *xe, const double *area,
                    const double *props, int64_t nprops, const int32_t *pid,
                    const double *k6rot, int k6rot_stride, const double *alpha, int alpha_stride,
                    int64_t *Kr, int64_t *Kc, double *Kv, int64_t nk, int values_only,
                    int *err, void *stream);

/* Quad4R.update_KC0 (pyfe3d/quad4r.pyx:1145-4618): 576 slots per element.
 * hgfactors: hgfactor_u, _v, _w, _rx, _ry, shared (hg_stride 0) or per
 * element (hg_stride 5); NULL means all 1. */
int fe3d_quad4r_kc0(int64_t E, const int64_t *cdof, const int64_t *init_k,
                    const double *x, int64_t nx, const double *xmat, int xmat_stride,
                    const double *R, const double *m, const double *xe, const double *area,
                    const double *props, int64_t nprops, const int32_t *pid,
                    const double *k6rot, int k6rot_stride, const double *hgfactors, int hg_stride,
                    int64_t *Kr, int64_t *Kc, double *Kv, int64_t nk, int values_only,
                    int *err, void *stream);

/* Tria3R.update_probe_finte / update_fint (pyfe3d/tria3r.pyx:549-947,
 * 2975-3017) in probe mode: finte[18e..] = KC0e ue (element frame, the whole
 * local matrix) and/or fint[c + .] += R finte (atomic; nf = length of fint).
 * Either output may be NULL. */
int fe3d_tria3r_finte(int64_t E, const int64_t *cdof, const double *R, const double *m,
                      const double *xe, const double *area, const double *ue,
                      const double *props, int64_t nprops, const int32_t *pid,
                      const double *k6rot, int k6rot_stride, const double *alpha, int alpha_stride,
                      double *fint, int64_t nf, double *finte, int *err, void *stream);

/* Quad4R.update_probe_finte / update_fint (pyfe3d/quad4r.pyx:549-1143,
 * 4620-4679), as fe3d_tria3r_finte with the hourglass factors. */
int fe3d_quad4r_finte(int64_t E, const int64_t *cdof, const double *R, const double *m,
                      const double *xe, const double *area, const double *ue,
                      const double *props, int64_t nprops, const int32_t *pid,
                      const double *k6rot, int k6rot_stride, const double *hgfactors, int hg_stride,
                      double *fint, int64_t nf, double *finte, int *err, void *stream);

/* Tria3R.update_KG (pyfe3d/tria3r.pyx:3020-3574): 81 slots row-major over
 * the translations of the 3 nodes.  Fused mode (x, u) or probe mode (R, m,
 * xe, area, ue).  Indices written unless values_only (update_KGv_only). */
int fe3d_tria3r_kg(int64_t E, const int64_t *cdof, const int64_t *init_k,
                   const double *x, int64_t nx, const double *xmat, int xmat_stride,
                   const double *u, int64_t nu, const double *R, const double *m,
                   const double *xe, const double *area, const double *ue,
                   const double *props, int64_t nprops, const int32_t *pid,
                   int64_t *Kr, int64_t *Kc, double *Kv, int64_t nk, int values_only,
                   int *err, void *stream);

/* Tria3R.update_KG_given_stress (pyfe3d/tria3r.pyx:3576-4061): nstress
 * (Nxx, Nyy, Nxy) per element (stride 3) or shared (stride 0); fused (x)
 * or probe mode (R, xe, area). */
int fe3d_tria3r_kg_given_stress(int64_t E, const int64_t *cdof, const int64_t *init_k,
                                const double *x, int64_t nx, const double *R, const double *xe,
                                const double *area, const double *nstress, int nstress_stride,
                                int64_t *Kr, int64_t *Kc, double *Kv, int64_t nk, int values_only,
                                int *err, void *stream);

/* Tria3R.update_M (pyfe3d/tria3r.pyx:4063-7723): mtype 0 (consistent) and
 * 1 (reduced) write 270 slots, 2 (lumped) 162.  Fused (x) or probe mode
 * (R, area). */
int fe3d_tria3r_m(int64_t E, const int64_t *cdof, const int64_t *init_k,
                  const double *x, int64_t nx, const double *R, const double *area,
                  const double *props, int64_t nprops, const int32_t *pid,
                  int64_t *Kr, int64_t *Kc, double *Kv, int64_t nk, int mtype,
                  int *err, void *stream);

/* ------------------------------------------------------------------ BeamC */

/* BeamC.update_rotation_matrix + update_probe_xe (pyfe3d/beamc.pyx:158-231,
 * 287-349).  vxy: 3 doubles per element (vxy_stride 3) or one vector
 * (vxy_stride 0).  R, xe (6/element), length may each be NULL. */
int fe3d_beamc_frame(int64_t E, const int64_t *cdof, const double *x, int64_t nx,
                     const double *vxy, int vxy_stride, double *R, double *xe,
                     double *length, int *err, void *stream);

/* BeamC.update_probe_xe + update_length with the frame R the element
 * holds (pyfe3d/beamc.pyx:287-349). */
int fe3d_beamc_probe_xe(int64_t E, const int64_t *cdof, const double *x, int64_t nx,
                        const double *R, double *xe, double *length, int *err, void *stream);

/* BeamC.update_probe_ue (pyfe3d/beamc.pyx:234-284). */
int fe3d_beamc_probe_ue(int64_t E, const int64_t *cdof, const double *u, int64_t nu,
                        const double *R, double *ue, int *err, void *stream);

/* BeamC.update_KC0 (pyfe3d/beamc.pyx:489-1352); probe inputs R, length. */
int fe3d_beamc_kc0(int64_t E, const int64_t *cdof, const int64_t *init_k,
                   const double *R, const double *length,
                   const double *props, int64_t nprops, const int32_t *pid,
                   int64_t *Kr, int64_t *Kc, double *Kv, int64_t nk, int values_only,
                   int *err, void *stream);

/* BeamC.update_KG (pyfe3d/beamc.pyx:1392-2179): indices are written when
 * values_only == 0 (the code's behaviour, beamc.pyx:1451). */
int fe3d_beamc_kg(int64_t E, const int64_t *cdof, const int64_t *init_k,
                  const double *R, const double *length, const double *ue,
                  const double *props, int64_t nprops, const int32_t *pid,
                  int64_t *Kr, int64_t *Kc, double *Kv, int64_t nk, int values_only,
                  int *err, void *stream);

/* BeamC.update_M (pyfe3d/beamc.pyx:2181-3152): mtype 0 consistent (144),
 * mtype 1 lumped (36 slots). */
int fe3d_beamc_m(int64_t E, const int64_t *cdof, const int64_t *init_k,
                 const double *R, const double *length,
                 const double *props, int64_t nprops, const int32_t *pid,
                 int64_t *Kr, int64_t *Kc, double *Kv, int64_t nk, int mtype,
                 int *err, void *stream);

/* BeamC.update_probe_finte / update_fint (pyfe3d/beamc.pyx:352-486,
 * 1354-1390): finte[12e..] = KC0e ue in the element frame (probe inputs R,
 * length, ue); fint[c + .] += R finte.  fint or finte may be NULL (not both). */
int fe3d_beamc_fint(int64_t E, const int64_t *cdof, const double *R, const double *length,
                    const double *ue, const double *props, int64_t nprops, const int32_t *pid,
                    double *fint, int64_t nf, double *finte, int *err, void *stream);

/* ------------------------------------------------------- assembly + BCs
 * Replaces the caller-side `coo_matrix((Kv, (Kr, Kc)), (N, N)).tocsc()` and
 * the boundary-condition slicing `K[bu, :][:, bu]` of the reference tests
 * (tests/test_quad4_static_point_load.py:80-99): the pattern is built once
 * from the COO indices, then every value update is assembled by a
 * deterministic segmented sum.
 */
typedef struct fe3d_pattern fe3d_pattern;

/* Build the reduced CSR pattern.  fixed: N bytes, non-zero for constrained
 * DOFs (bk of the reference tests), or NULL for no constraint.  COO slots
 * with a fixed row or column are dropped; duplicates are summed.  Requires
 * nnz_in < 2^31 and N < 2^31.  The pattern owns device memory (released by
 * fe3d_pattern_free). Synchronises `stream`. */
int fe3d_pattern_build(const int64_t *Kr, const int64_t *Kc, int64_t nnz_in, int64_t N,
                       const uint8_t *fixed, fe3d_pattern **out, int *err, void *stream);
int fe3d_pattern_free(fe3d_pattern *p);
/* Host: rows (free DOFs), CSR entries, COO slots of the pattern. */
int fe3d_pattern_info(const fe3d_pattern *p, int64_t *nrows, int64_t *nnz, int64_t *nnz_in);
/* Device arrays owned by the pattern: rowptr [nrows+1] (int64), colind [nnz]
 * (int32, sorted per row), dof_of_row [nrows] (reduced row -> full DOF),
 * row_of_dof [N] (full DOF -> reduced row or -1). Any output may be NULL. */
int fe3d_pattern_arrays(const fe3d_pattern *p, const int64_t **rowptr, const int32_t **colind,
                        const int64_t **dof_of_row, const int32_t **row_of_dof);
/* Copy the pattern's rowptr / colind / dof_of_row into caller device buffers
 * (any may be NULL). */
int fe3d_pattern_copy(const fe3d_pattern *p, int64_t *rowptr, int32_t *colind, int64_t *dof_of_row,
                      void *stream);
/* vals[nnz] = reduced CSR values of the COO values Kv[nnz_in]. */
int fe3d_assemble(const fe3d_pattern *p, const double *Kv, double *vals, void *stream);

/* ------------------------------------------- fused element -> CSR assembly
 * The same reduced CSR matrix as `coo_matrix(...).tocsc()` + `K[bu, :][:, bu]`
 * of the reference tests (tests/test_quad4_static_point_load.py:80-99), but
 * built from the element connectivity, with no COO triplets written: the
 * pattern comes from the elements' node pairs (every element couples all
 * DOFs of its nodes, as the KC0 triplets of Quad4, Quad4R, Tria3R and BeamC
 * do, pyfe3d/quad4.pyx:1204-1313, beamc.pyx:489-1352), and a scatter map
 * sends each element's 6x6 node-pair blocks straight to their CSR
 * positions.  Elements are coloured (no two elements of a colour share a
 * node) and each colour is one launch, so the blocks are read, added and
 * written without atomics, in a fixed order: the values are deterministic.
 */
typedef struct {
    int64_t E;            /* elements */
    int nn;               /* nodes per element: 2 (BeamC), 3 (Tria3R), 4 (Quad4, Quad4R) */
    const int64_t *cdof;  /* device [E, nn]: the elements' DOF offsets c1..c_nn (6 x node) */
} fe3d_elem_group;

#define FE3D_CSR_ADD 0     /* vals += every element block */
#define FE3D_CSR_ASSIGN 1  /* the first contributor of each node-pair block (first group of the map,
                              then lowest colour) stores, the others add: after every group of the
                              map has run in order, vals holds K whatever it held before */
#define FE3D_CSR_ATOMIC 2  /* vals += every element block in one launch with atomic additions
                              (no colour passes; the order of the additions, and so the last bits
                              of entries with three or more contributions, vary between runs) */

/* Reduced CSR pattern of the element groups (1..8 groups, together the mesh)
 * over N DOFs (N = 6 nodes), fixed as in fe3d_pattern_build.  Equal to the
 * pattern fe3d_pattern_build gives for the groups' KC0 triplets (same
 * rowptr and colind); its fe3d_assemble is unavailable (FE3D_ERR_STATE).
 * Synchronises `stream`. */
int fe3d_pattern_build_elements(const fe3d_elem_group *groups, int ngroups, int64_t N, const uint8_t *fixed,
                                fe3d_pattern **out, int *err, void *stream);

typedef struct fe3d_fmap fe3d_fmap;
/* Scatter map of the element groups on a pattern from
 * fe3d_pattern_build_elements (the groups of the build, same order): node
 * indices, block offsets, assign bits and the colouring (greedy, on the
 * host; elements with a repeated node are rejected).  Synchronises `stream`. */
int fe3d_fmap_build(const fe3d_pattern *p, const fe3d_elem_group *groups, int ngroups, fe3d_fmap **out,
                    int *err, void *stream);
int fe3d_fmap_free(fe3d_fmap *m);
/* Host: colours of group g and their element counts (counts may be NULL;
 * room for 64). */
int fe3d_fmap_info(const fe3d_fmap *m, int g, int *ncolors, int64_t *counts);

/* vals (+)= the element blocks of group g held as values-only element
 * matrices Kv[init_k[e] + (6 nn)^2) (row-major over the element's DOFs, the
 * layout of the reference's *_SPARSE_SIZE slots), e.g. from a values-only
 * update_KC0 into a zeroed buffer.  mode FE3D_CSR_ADD / FE3D_CSR_ASSIGN. */
int fe3d_csr_scatter(const fe3d_fmap *m, int g, const int64_t *init_k, const double *Kv, int64_t nk,
                     double *vals, int mode, int *err, void *stream);

/* Quad4.update_KC0 (pyfe3d/quad4.pyx:1204-1313) of group g (nn = 4) added
 * straight into the CSR values: the fe3d_quad4_kc0 kernel with the map's
 * scatter instead of the triplet write-out (no Kr/Kc/Kv).  x, xmat, props,
 * pid as in fe3d_quad4_kc0 (element order of the group).  Requires every
 * node's row length below 32768 (else FE3D_ERR_ARG). */
int fe3d_quad4_kc0_csr(const fe3d_fmap *m, int g, const double *x, int64_t nx, const double *xmat,
                       int xmat_stride, const double *props, int64_t nprops, const int32_t *pid,
                       double *vals, int mode, int *err, void *stream);

/* y = K x on the reduced system (FP64). */
int fe3d_spmv(const fe3d_pattern *p, const double *vals, const double *x, double *y, void *stream);

/* --------------------------------------------------------------- solver
 * Block-Jacobi preconditioned CG on the reduced system, standing in for
 * `spsolve(Kuu, fu)` (tests/test_beamc_static_point_load.py:109) and
 * `cg(Kuu, fu)` (tests/test_quad4_static_point_load.py:102).
 */
typedef struct fe3d_solver fe3d_solver;

typedef struct {
    double tol;          /* stop when ||f - K u|| <= tol ||f|| (FP64 residual) */
    int64_t maxiter;     /* iteration cap */
    int precision;       /* 0: FP64; 1: FP32 SpMV/preconditioner on the scaled system, FP64
                            reliable updates; 2: FP64 vectors and preconditioner with the
                            SpMV products on the FP32 pipe (values and direction split into
                            float pairs, float-float row sums, ~48-bit products); 3: nested
                            iterative refinement: inner FP32 PCG on the scaled system (FP32 SpMV,
                            block-Jacobi and accumulation) to inner_tol, outer FP64 residual
                            r = f - K u and update of the double-double iterate */
    int check_every;     /* iterations between host convergence checks */
    int replace_every;   /* precision 1: iterations between FP64 residual replacements */
    int flexible;        /* 1: flexible CG, beta = r1.(z1 - z0) / r0.z0 (for preconditioners
                            that are not exactly symmetric/fixed, e.g. learned blocks) */
    double inner_tol;    /* precision 3: an inner FP32 solve stops when its residual has dropped by
                            this factor (0: 1e-2); replace_every then caps its iterations */
} fe3d_solve_opts;

typedef struct {
    int status;          /* 0 converged, 1 iteration cap, 3 non-finite residual,
                            4 stagnated (precision 1 or 3: FP32 directions stopped reducing the
                            FP64 residual; continue with precision 0 from u) */
    int reserved;
    int64_t iterations;
    int64_t replacements;/* FP64 residual replacements performed */
    double relres;       /* final ||f - K u|| / ||f|| in FP64 */
} fe3d_solve_stats;

/* Solver bound to a pattern; block_size DOFs per node (6 for pyfe3d). */
int fe3d_solver_create(const fe3d_pattern *p, int block_size, fe3d_solver **out);
/* Factor the nodal diagonal blocks of vals (kept by reference, must stay
 * alive); mixed bit 0 also prepares the FP32 copies (precision 1), bit 1 the
 * split-FP32 values (precision 2); the SpMV lanes per row are timed on the
 * first setup of each precision.  nonpos_blocks (host,
 * may be NULL) receives the number of blocks that were not positive
 * definite (those fall back to scalar Jacobi). Synchronises `stream`. */
int fe3d_solver_setup(fe3d_solver *s, const double *vals, int mixed, int *nonpos_blocks,
                      void *stream);
/* Solve K u = f on the reduced system; u holds the initial guess on entry.
 * opts and stats are host pointers.  Synchronises `stream`. */
int fe3d_solver_solve(fe3d_solver *s, const double *f, double *u, const fe3d_solve_opts *opts,
                      fe3d_solve_stats *stats, void *stream);
/* No counterpart in the reference.  Replace the preconditioner blocks: blocks
 * (device, 36 doubles per node, row-major over the node's free DOFs in
 * increasing DOF order, zero padded) are factored like the diagonal blocks
 * in setup; a block that is not positive definite falls back to the
 * block-Jacobi inverse of that node's diagonal block.  fallback (device int8
 * per node, may be NULL) receives 1 for those nodes, nfallback (host, may be
 * NULL) their count.  Requires a prior setup; synchronises `stream`. */
int fe3d_solver_set_blocks(fe3d_solver *s, const double *blocks, int8_t *fallback, int *nfallback,
                           void *stream);
int fe3d_solver_free(fe3d_solver *s);

/* ------------------------------------------- learned block preconditioner
 * No counterpart in the reference.  A per-node MLP (FP32, FE3D_LPC_NFEAT
 * inputs -> 64 -> 64 -> 21, tanh) predicts a symmetric 6x6 correction C_j
 * of each node's diagonal block in the scaled coordinates
 * S^-1 D_j S^-1 (S = sqrt(diag K)); the preconditioner block is
 * B_j = D_j + out_scale * S C_j S, installed with fe3d_solver_set_blocks and
 * used inside flexible CG (fe3d_solve_opts.flexible).  Weights are packed
 * W1[64][35] b1[64] W2[64][64] b2[64] W3[21][64] b3[21]; outputs are the
 * upper triangle of C_j row-major.  All solver arguments need block size 6
 * and a prior fe3d_solver_setup.  Training: for residual samples r with
 * weight w = 1 / (e.r) (e = K^-1 r), z = B^-1 r (fe3d_lpc_apply), Kz
 * (fe3d_spmv), then fe3d_lpc_loss_grad accumulates the loss and dL/d(outputs)
 * into gout; fe3d_lpc_backward turns gout into weight gradients (added to
 * grad) and fe3d_lpc_adam takes an Adam step. */
#define FE3D_LPC_NFEAT 35
#define FE3D_LPC_NHID 64
#define FE3D_LPC_NOUT 21
#define FE3D_LPC_NWEIGHTS 7829
/* feat: float [nnodes][35]; sdiag: double [nrows] = sqrt(K_ii). */
int fe3d_lpc_features(const fe3d_solver *s, float *feat, double *sdiag, void *stream);
/* Feature set 0 is fe3d_lpc_features.  Set 1 (29 inputs; slots 29-34 are
 * zero, so their weights get no gradient): the 21 unique entries of the
 * node's diagonal block normalised by its diagonal, S^-1 D_j S^-1 (upper
 * triangle), then the 8 largest Frobenius norms of the normalised coupling
 * blocks S_j^-1 K_jk S_k^-1. */
int fe3d_lpc_features_set(const fe3d_solver *s, int set, float *feat, double *sdiag, void *stream);
/* out: float [nnodes][21]; act (may be NULL): float [nnodes][128] kept for
 * the backward pass. */
int fe3d_lpc_forward(int64_t nnodes, const float *feat, const float *weights, float *out, float *act,
                     void *stream);
/* blocks: double [nnodes][36] for fe3d_solver_set_blocks. */
int fe3d_lpc_blocks(const fe3d_solver *s, const double *sdiag, const float *out, float out_scale,
                    double *blocks, void *stream);
/* z = B^-1 r with the solver's current blocks (FP64). */
int fe3d_lpc_apply(const fe3d_solver *s, const double *r, double *z, void *stream);
/* One residual sample: inv_er = 1 / (e.r) (e = K^-1 r), factor = the
 * sample's share of the batch.  mode 0: L = factor (inv_er ||z - e||_K^2 - 1)
 * = factor inv_er (z.Kz - 2 z.r); mode 1: the error after the optimal step
 * along z, L = factor (1 - inv_er (z.r)^2 / (z.Kz)) (invariant to the scale
 * of the blocks, as CG is).  fallback: the per-node flags of
 * fe3d_solver_set_blocks (nodes that fell back get no gradient); acc: device
 * double[3], acc[0] accumulates L, acc[1..2] are scratch. */
int fe3d_lpc_loss_grad(const fe3d_solver *s, const double *sdiag, const double *r, const double *z,
                       const double *Kz, const int8_t *fallback, double inv_er, double factor,
                       float out_scale, int mode, float *gout, double *acc, void *stream);
/* delta: float scratch [nnodes][149]; grad: float [FE3D_LPC_NWEIGHTS], added to. */
int fe3d_lpc_backward(int64_t nnodes, const float *feat, const float *weights, const float *act,
                      const float *gout, float *delta, float *grad, void *stream);
int fe3d_lpc_adam(int64_t nw, float *w, const float *g, float *m, float *v, float lr, float beta1,
                  float beta2, float eps, int step, void *stream);

/* --------------------------------------------------------- eigensolver
 * Block kernels of the device LOBPCG (pyfe3d_gb300.eigen) that stands in
 * for the reference tests' eigsh calls (tests/test_quad4_natural_freq.py:117,
 * tests/test_quad4_linear_buckling_plate_rotated.py:129).
 * fe3d_spmm: Y = A X for row-major n x k blocks (1 <= k <= 16).
 * fe3d_solver_precond_multi: Z = Dinv R column by column with the solver's
 * nodal block inverses (requires setup). */
int fe3d_spmm(const fe3d_pattern *p, const double *vals, const double *X, double *Y, int k, void *stream);
int fe3d_solver_precond_multi(const fe3d_solver *s, const double *R, double *Z, int k, void *stream);
/* Rayleigh-Ritz projections of the LOBPCG (the dense products of the
 * reference tests' eigsh, tests/test_quad4_natural_freq.py:117-120):
 * G (k1 x k2, row-major) = X^T Y for row-major n x k1 and n x k2 blocks
 * (k1, k2 <= 64), summed in a fixed order over per-block partials held in the
 * caller's scratch of fe3d_dense_gram_scratch(k1, k2) doubles; and
 * Y (n x m) = beta Y + alpha X T for X n x k, T k x m (k, m <= 64; Y must not
 * overlap X or T). */
int64_t fe3d_dense_gram_scratch(int k1, int k2);
int fe3d_dense_gram(int64_t n, int k1, int k2, const double *X, const double *Y, double *G, double *scratch,
                    void *stream);
int fe3d_dense_gemm_tall(int64_t n, int k, int m, const double *X, const double *T, double alpha, double beta,
                         double *Y, void *stream);

/* ------------------------------------------------------- batched solver
 * Many independent systems (instances, e.g. one plate each) solved together,
 * replacing a loop of `spsolve(Kuu, fu)` calls
 * (tests/test_quad4_static_point_load.py:102), one per plate.  The pattern
 * holds the block-diagonal matrix of all instances; inst_of_row (int32
 * [nrows], host or device) gives each reduced row's instance in [0, ninst).
 * Every instance runs its own CG recurrence and convergence test.  Create
 * fails with FE3D_ERR_BOUNDS when an instance is out of range or a node's
 * rows span two instances, and with FE3D_ERR_ARG when the matrix couples two
 * instances.  Per-instance dot products use FP64 atomics: the last bits of
 * the iterates can differ from run to run. */
typedef struct fe3d_bsolver fe3d_bsolver;
int fe3d_bsolver_create(const fe3d_pattern *p, int block_size, int64_t ninst, const int32_t *inst_of_row,
                        fe3d_bsolver **out);
/* As fe3d_solver_setup; also times the SpMV lanes-per-row candidates
 * (4, 8, 16, 32) on this matrix and keeps the fastest per precision. */
int fe3d_bsolver_setup(fe3d_bsolver *b, const double *vals, int mixed, int *nonpos_blocks, void *stream);
/* Lanes per row chosen at setup (0 when that precision was not prepared). */
int fe3d_bsolver_info(const fe3d_bsolver *b, int *lanes_fp64, int *lanes_fp32);
/* Work split of precision-0 solves: instances whose reduced rows are
 * contiguous and at most max_rows in number are each solved by one thread
 * block of a block-resident FP64 PCG kernel (block-level reductions in a fixed
 * order, convergence confirmed on the FP64 residual; the search direction
 * and its product in shared memory), on a second stream
 * concurrently with the lockstep recurrence of the other instances; 0 (the
 * default) sends every instance to the lockstep recurrence.  eligible (host,
 * may be NULL) receives the number of instances the limit selects. */
int fe3d_bsolver_set_split(fe3d_bsolver *b, int64_t max_rows, int64_t *eligible);
/* Largest max_rows: the block keeps the instance's search direction and its
 * product in shared memory (2 x 8 bytes per row). */
#define FE3D_BSPLIT_MAX_ROWS 12288
/* Solve every instance; u holds the initial guess.  inst_status (0
 * converged, 1 iteration cap, 3 non-finite, 4 stagnated in precision 1),
 * inst_iters and inst_relres
 * (FP64 ||f - K u|| / ||f|| per instance) are host arrays of ninst, each may
 * be NULL; total gets the worst status and relative residual and the number
 * of lockstep iterations.  Synchronises `stream`. */
int fe3d_bsolver_solve(fe3d_bsolver *b, const double *f, double *u, const fe3d_solve_opts *opts,
                       int *inst_status, int64_t *inst_iters, double *inst_relres, fe3d_solve_stats *total,
                       void *stream);
int fe3d_bsolver_free(fe3d_bsolver *b);

/* ------------------------------------------------ allocation-free solve
 * No counterpart in the reference.  For callers that cannot allocate device
 * memory themselves (device memory owned by another runtime's pool, code
 * paths where cudaMalloc must not be called): a Jacobi-preconditioned CG on
 * the caller's reduced CSR matrix (rowptr int64 [n+1], colind int32, vals
 * double) and vectors (f, u; u holds the initial guess), using only a
 * library-owned file-scope device array of FE3D_NOALLOC_MAX_ROWS rows (about
 * 5.3 MB, held by every GPU that loads the library until exit).  It calls no
 * cudaMalloc, cudaFree or allocating library routine.  n above the maximum
 * is rejected with FE3D_ERR_TOO_LARGE before any device work.  All calls
 * share the array: calls that overlap on the GPU race and must be
 * serialised; each call initialises what it reads.  The first call on a
 * device looks up the array's address (cudaGetSymbolAddress), keeps it for
 * the life of the process and should come before any stream capture; the
 * entry point must not be used after a cudaDeviceReset.  Duplicate CSR
 * entries are summed (diagonal included).  opts/stats are host pointers
 * (opts.precision and opts.replace_every are ignored); synchronises
 * `stream`. */
#define FE3D_NOALLOC_MAX_ROWS 131072
#define FE3D_ERR_TOO_LARGE (-7) /* size above the allocation-free maximum */
int64_t fe3d_noalloc_max_rows(void);
int fe3d_jacobi_pcg_noalloc(int64_t n, const int64_t *rowptr, const int32_t *colind, const double *vals,
                            const double *f, double *u, const fe3d_solve_opts *opts,
                            fe3d_solve_stats *stats, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* FE3D_GB300_H */
