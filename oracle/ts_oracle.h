/*
 * CPU oracle for the staggered-grid (visco)elastic stepper: TEST
 * INFRASTRUCTURE ONLY.  It restates the reference's kernels on the CPU so
 * that the CUDA product path can be checked against it; nothing in the
 * product links or calls it.
 *
 * Three kernel families are restated, each following the reference line by
 * line, with the reference's operation order:
 *   - TS_ORC_TAICHI2D : sim_taichi_elastic.py:138-309 (2D isotropic elastic)
 *   - TS_ORC_WGSL2D   : shader_webgpu_viscoelastic.wgsl:829-1072 + 1118-1141
 *   - TS_ORC_WGSL3D   : shader_webgpu_3D_viscoelastic.wgsl:1341-1773 + 1824-1850
 * and the per-step order of their drivers (sim_taichi_elastic.py:311-335,
 * sim_webgpu_viscoelastic.py:469-537, sim_webgpu_3D_viscoelastic.py:628-695).
 *
 * Out-of-range reads return 0 and out-of-range writes are dropped, as the
 * WGSL accessors do (shader_webgpu_viscoelastic.wgsl:18-29, 92-96).
 *
 * Built twice from ts_oracle.c: ts_oracle_run_f32 computes in float (the
 * reference's precision) and ts_oracle_run_f64 in double (to measure the
 * float rounding error of either implementation).
 *
 * Pinning: the TAICHI2D family reproduces the reference's only known-answer
 * result (pedro/results/result_teste_aco.npy, relative L2 7.4e-6 over 10000
 * steps; tests/test_oracle_golden.py).  For the WGSL families parity is
 * unpinned: the reference ships no WGSL-produced result and its shaders
 * cannot run here (no graphics API), so they rest on line-by-line review and
 * the formulas they share with the pinned family.
 */
#ifndef TS_ORACLE_H
#define TS_ORACLE_H
#include <stdint.h>

#define TS_ORC_TAICHI2D 0
#define TS_ORC_WGSL2D 1
#define TS_ORC_WGSL3D 2

typedef struct {
    int32_t family;          /* TS_ORC_* */
    int32_t nx, ny, nz;      /* nz = 1 in 2D */
    int32_t n_steps;         /* steps to run */
    int32_t ord;             /* number of FD coefficients */
    const float *coefs;      /* [ord] */
    float dx, dy, dz, dt;
    float one_dx, one_dy;    /* Taichi multiplies by these */
    /* CPML tables, each of length n_axis - 2 (ord - 1) */
    const float *a_x, *b_x, *k_x, *a_xh, *b_xh, *k_xh;
    const float *a_y, *b_y, *k_y, *a_yh, *b_yh, *k_yh;
    const float *a_z, *b_z, *k_z, *a_zh, *b_zh, *k_zh;
    const float *rho, *cp, *cs;          /* grid, C order, last axis fastest */
    int32_t visco, n_sls;
    const float *tau;                    /* [4][n_sls] */
    const float *sum_alpha;              /* [2] */
    /* per-cell quality factor (extension): NULL = the reference's global taus */
    const float *g_p, *g_s;              /* grid */
    const float *zc, *zh, *zm;           /* [n_sls] */
    /* sources */
    const float *source_term;            /* flat, as the reference buffer */
    int32_t src_rows, src_cols;          /* 2D shape of source_term for Taichi */
    int32_t n_src_el;                    /* WGSL stride/bound (n_src) */
    const int32_t *pos_sources;          /* grid, -1 = none */
    /* receivers */
    int32_t n_rec, n_rec_pt;
    const int32_t *pos_sensors;          /* grid (Taichi) */
    const int32_t *info_rec_pt;          /* [n_rec_pt][3 or 4] (WGSL) */
    const int32_t *offset_sensors;       /* [n_rec] */
    const int32_t *delay_rec;            /* [n_rec] */
} ts_oracle_desc;

/* Runs n_steps steps from a zero state.  Outputs (grids of `real`): v[3] =
 * vx, vy, vz; s[6] = sxx, syy, szz, sxy, sxz, syz (2D uses vx, vy, sxx,
 * syy, sxy; unused entries may be NULL).  sens is [n_steps][n_rec] and
 * vmax2 [n_steps] (per-step max |v|^2), both of `real`.  Returns 0, or -1
 * when a scratch allocation fails. */
int ts_oracle_run_f32(const ts_oracle_desc *d, float **v, float **s, float *sens, float *vmax2);
int ts_oracle_run_f64(const ts_oracle_desc *d, double **v, double **s, double *sens, double *vmax2);

#endif
