/*
 * Body of the CPU oracle, included twice by ts_oracle.c with `real` = float
 * and = double.  TEST INFRASTRUCTURE ONLY (see ts_oracle.h).
 *
 * Every expression keeps the reference's association order; `(real)` casts
 * of the float tables are exact.  In float builds the compiler must not
 * contract a*b+c into fma (built with -ffp-contract=off).
 */

#define RD(a) ((real)(a))

/* ---- accessors with the reference's bounds semantics ------------------ */
typedef struct {
    const ts_oracle_desc *d;
    long nx, ny, nz;      /* nz = 1 in 2D */
    long ntab_x, ntab_y, ntab_z;
} FN(ctx);

static inline long FN(ix3)(const FN(ctx) *c, long x, long y, long z) {
    if (x < 0 || x >= c->nx || y < 0 || y >= c->ny || z < 0 || z >= c->nz) return -1;
    return (x * c->ny + y) * c->nz + z;
}

static inline real FN(get)(const FN(ctx) *c, const real *a, long x, long y, long z) {
    long i = FN(ix3)(c, x, y, z);
    return i < 0 ? RD(0) : a[i];
}

static inline real FN(getf)(const FN(ctx) *c, const float *a, long x, long y, long z) {
    long i = FN(ix3)(c, x, y, z);
    return i < 0 ? RD(0) : RD(a[i]);
}

/* CPML table value at table index n; zero outside [0, n_tab) (wgsl:92-96). */
static inline real FN(tab)(const float *t, long n, long ntab) {
    return (n >= 0 && n < ntab) ? RD(t[n]) : RD(0);
}

/* Zener constants of mechanism l, exactly as the shaders evaluate them
 * (shader_webgpu_viscoelastic.wgsl:881-894). */
typedef struct { real phi_p, phi_s, h_p, h_s, m_p, m_s; } FN(zener);

static FN(zener) FN(zener_global)(const ts_oracle_desc *d, int l) {
    FN(zener) z;
    const int L = d->n_sls;
    real dt = RD(d->dt);
    real inv_p = RD(1.0) / RD(d->tau[1 * L + l]);
    real inv_s = RD(1.0) / RD(d->tau[3 * L + l]);
    real a_p = RD(d->tau[0 * L + l]) / RD(d->tau[1 * L + l]);
    real a_s = RD(d->tau[2 * L + l]) / RD(d->tau[3 * L + l]);
    z.phi_p = dt * (RD(1.0) - a_p) * inv_p / RD(d->sum_alpha[0]);
    z.phi_s = dt * (RD(1.0) - a_s) * inv_s / RD(d->sum_alpha[1]);
    z.h_p = RD(0.5) * dt * inv_p;
    z.h_s = RD(0.5) * dt * inv_s;
    z.m_p = RD(1.0) / (RD(1.0) + z.h_p);
    z.m_s = RD(1.0) / (RD(1.0) + z.h_s);
    return z;
}

/* Per-cell Q (extension): phi = c_l * g(cell); h, m per mechanism. */
static FN(zener) FN(zener_cell)(const ts_oracle_desc *d, int l, long cell) {
    FN(zener) z;
    z.phi_p = RD(d->zc[l]) * RD(d->g_p[cell]);
    z.phi_s = RD(d->zc[l]) * RD(d->g_s[cell]);
    z.h_p = z.h_s = RD(d->zh[l]);
    z.m_p = z.m_s = RD(d->zm[l]);
    return z;
}

static inline FN(zener) FN(zener_at)(const ts_oracle_desc *d, int l, long cell) {
    return d->g_p ? FN(zener_cell)(d, l, cell) : FN(zener_global)(d, l);
}

/* offset_sensors[s] as the WGSL store kernel reads it (wgsl:797-799,
 * 1125): the array holds one entry per group of equal ids in info_rec_pt
 * (sim_support/simulator.py:289-294); past its end there is no point. */
static int FN(first_point)(const ts_oracle_desc *d, int sn, int cols) {
    if (d->n_rec_pt <= 0) return -1;
    int groups = 1;
    for (int pt = 1; pt < d->n_rec_pt; ++pt)
        if (d->info_rec_pt[pt * cols + cols - 1] != d->info_rec_pt[(pt - 1) * cols + cols - 1]) ++groups;
    return sn < groups ? d->offset_sensors[sn] : -1;
}

/* CPML convolution update of one derivative (b psi + a d; d/k + psi). */
static inline real FN(cpml)(real deriv, real *psi, real a, real b, real k) {
    real p = b * (*psi) + a * deriv;
    *psi = p;
    return deriv / k + p;
}

/* ===================================================================== */
/* Taichi 2D isotropic elastic (sim_taichi_elastic.py:138-309)             */
/* ===================================================================== */
static int FN(run_taichi2d)(const ts_oracle_desc *d, real **v, real **s, real *sens, real *vmax2) {
    FN(ctx) c = {d, d->nx, d->ny, 1, d->nx - 2 * (d->ord - 1), d->ny - 2 * (d->ord - 1), 0};
    const long nx = c.nx, ny = c.ny, n = nx * ny;
    const int ord = d->ord, off = ord - 1;
    real *vx = v[0], *vy = v[1], *sxx = s[0], *syy = s[1], *sxy = s[3];
    real *m[8];
    for (int i = 0; i < 8; ++i) {
        m[i] = (real *)calloc((size_t)n, sizeof(real));
        if (!m[i]) return -1;
    }
    real *m_dvx_dx = m[0], *m_dvy_dy = m[1], *m_dvy_dx = m[2], *m_dvx_dy = m[3];
    real *m_dsxx_dx = m[4], *m_dsxy_dy = m[5], *m_dsxy_dx = m[6], *m_dsyy_dy = m[7];
    const real dt = RD(d->dt), odx = RD(d->one_dx), ody = RD(d->one_dy);
    const long src_cols = d->src_cols;

    for (int step = 0; step < d->n_steps; ++step) {
        const int it = step + 1; /* the reference's loop index starts at 1 */
        /* ---- sigma_kernel (:138-229) ---- */
#pragma omp parallel for schedule(static)
        for (long x = 0; x < nx; ++x) {
            for (long y = 0; y < ny; ++y) {
                const long i = x * ny + y;
                if (x >= ord - 1 && x < nx - ord && y >= ord && y < ny - ord + 1) {
                    real ddx = RD(0), ddy = RD(0);
                    for (int k = 0; k < ord; ++k) {
                        ddx += RD(d->coefs[k]) * (vx[(x + k + 1) * ny + y] - vx[(x - k) * ny + y]) * odx;
                        ddy += RD(d->coefs[k]) * (vy[x * ny + y + k] - vy[x * ny + y - k - 1]) * ody;
                    }
                    ddx = FN(cpml)(ddx, &m_dvx_dx[i], RD(d->a_xh[x - off]), RD(d->b_xh[x - off]), RD(d->k_xh[x - off]));
                    ddy = FN(cpml)(ddy, &m_dvy_dy[i], RD(d->a_y[y - off]), RD(d->b_y[y - off]), RD(d->k_y[y - off]));
                    real div = ddx + ddy;
                    real rho_h = RD(0.5) * (RD(d->rho[i + ny]) + RD(d->rho[i]));
                    real cp_h = RD(0.5) * (RD(d->cp[i + ny]) + RD(d->cp[i]));
                    real cs_p1 = RD(d->cs[i + ny]), cs_m1 = RD(d->cs[i]);
                    real cs_l = RD(0.5) * (cs_p1 + cs_m1);
                    real cs_m = ((cs_p1 < cs_m1 ? cs_p1 : cs_m1) == RD(0)) ? RD(0) : cs_l;
                    real lam = rho_h * (cp_h * cp_h - RD(2.0) * cs_l * cs_l);
                    real mu = rho_h * (cs_m * cs_m);
                    real div_lam = lam * div;
                    sxx[i] += (div_lam + RD(2.0) * mu * ddx) * dt;
                    syy[i] += (div_lam + RD(2.0) * mu * ddy) * dt;
                }
                if (x >= ord && x < nx - ord + 1 && y >= ord - 1 && y < ny - ord) {
                    real dvy_dx = RD(0), dvx_dy = RD(0);
                    for (int k = 0; k < ord; ++k) {
                        dvy_dx += RD(d->coefs[k]) * (vy[(x + k) * ny + y] - vy[(x - k - 1) * ny + y]) * odx;
                        dvx_dy += RD(d->coefs[k]) * (vx[x * ny + y + k + 1] - vx[x * ny + y - k]) * ody;
                    }
                    dvy_dx = FN(cpml)(dvy_dx, &m_dvy_dx[i], RD(d->a_x[x - off]), RD(d->b_x[x - off]), RD(d->k_x[x - off]));
                    dvx_dy = FN(cpml)(dvx_dy, &m_dvx_dy[i], RD(d->a_yh[y - off]), RD(d->b_yh[y - off]), RD(d->k_yh[y - off]));
                    real rho_h = RD(0.5) * (RD(d->rho[i + 1]) + RD(d->rho[i]));
                    real cs_p1 = RD(d->cs[i + 1]), cs_m1 = RD(d->cs[i]);
                    real cs_h = ((cs_p1 < cs_m1 ? cs_p1 : cs_m1) == RD(0)) ? RD(0) : (RD(0.5) * (cs_p1 + cs_m1));
                    real mu = rho_h * (cs_h * cs_h);
                    sxy[i] += (dvx_dy + dvy_dx) * mu * dt;
                }
            }
        }
        /* receivers: sens[it-1, s] += syy inside the normal region (:188-190);
         * summed in grid order (the reference's atomic order is unspecified) */
        for (long x = ord - 1; x < nx - ord; ++x)
            for (long y = ord; y < ny - ord + 1; ++y) {
                int sn = d->pos_sensors[x * ny + y];
                if (sn != -1 && it >= d->delay_rec[sn]) sens[(long)(it - 1) * d->n_rec + sn] += syy[x * ny + y];
            }
        /* ---- velocity_kernel (:232-309) ---- */
        real vmax = RD(0);
#pragma omp parallel for schedule(static) reduction(max : vmax)
        for (long x = 0; x < nx; ++x) {
            for (long y = 0; y < ny; ++y) {
                const long i = x * ny + y;
                if (x >= ord && x < nx - ord + 1 && y >= ord && y < ny - ord + 1) {
                    real dsxx = RD(0), dsxy = RD(0);
                    for (int k = 0; k < ord; ++k) {
                        dsxx += RD(d->coefs[k]) * (sxx[(x + k) * ny + y] - sxx[(x - k - 1) * ny + y]) * odx;
                        dsxy += RD(d->coefs[k]) * (sxy[x * ny + y + k] - sxy[x * ny + y - k - 1]) * ody;
                    }
                    dsxx = FN(cpml)(dsxx, &m_dsxx_dx[i], RD(d->a_x[x - off]), RD(d->b_x[x - off]), RD(d->k_x[x - off]));
                    dsxy = FN(cpml)(dsxy, &m_dsxy_dy[i], RD(d->a_y[y - off]), RD(d->b_y[y - off]), RD(d->k_y[y - off]));
                    real rho = RD(d->rho[i]);
                    if (rho > RD(0)) vx[i] += (dsxx + dsxy) * dt / rho;
                } else {
                    vx[i] = RD(0);
                }
                if (x >= ord - 1 && x < nx - ord && y >= ord - 1 && y < ny - ord) {
                    real dsxy_dx = RD(0), dsyy = RD(0);
                    for (int k = 0; k < ord; ++k) {
                        dsxy_dx += RD(d->coefs[k]) * (sxy[(x + k + 1) * ny + y] - sxy[(x - k) * ny + y]) * odx;
                        dsyy += RD(d->coefs[k]) * (syy[x * ny + y + k + 1] - syy[x * ny + y - k]) * ody;
                    }
                    dsxy_dx = FN(cpml)(dsxy_dx, &m_dsxy_dx[i], RD(d->a_xh[x - off]), RD(d->b_xh[x - off]), RD(d->k_xh[x - off]));
                    dsyy = FN(cpml)(dsyy, &m_dsyy_dy[i], RD(d->a_yh[y - off]), RD(d->b_yh[y - off]), RD(d->k_yh[y - off]));
                    real rho = RD(0.25) * (RD(d->rho[i + 1]) + RD(d->rho[i]) + RD(d->rho[i + ny + 1]) + RD(d->rho[i + ny]));
                    if (rho > RD(0)) {
                        int isrc = d->pos_sources[i];
                        real val = RD(0);
                        if (isrc != -1) val = RD(d->source_term[(long)(it - 1) * src_cols + isrc]) * dt / rho;
                        vy[i] += val + (dsxy_dx + dsyy) * dt / rho;
                    }
                } else {
                    vy[i] = RD(0);
                }
                real v2 = vy[i] * vy[i] + vx[i] * vx[i];
                if (v2 > vmax || v2 != v2) vmax = v2;
            }
        }
        vmax2[step] = vmax;
    }
    for (int i = 0; i < 8; ++i) free(m[i]);
    return 0;
}

/* ===================================================================== */
/* WGSL 2D (visco)elastic (shader_webgpu_viscoelastic.wgsl:829-1141)       */
/* ===================================================================== */
static int FN(run_wgsl2d)(const ts_oracle_desc *d, real **v, real **s, real *sens, real *vmax2) {
    FN(ctx) c = {d, d->nx, d->ny, 1, d->nx - 2 * (d->ord - 1), d->ny - 2 * (d->ord - 1), 0};
    const long nx = c.nx, ny = c.ny, n = nx * ny;
    const int ord = d->ord, off = ord - 1, L = d->visco ? d->n_sls : 0;
    real *vx = v[0], *vy = v[1], *sxx = s[0], *syy = s[1], *sxy = s[3];
    real *m[8];
    for (int i = 0; i < 8; ++i) {
        m[i] = (real *)calloc((size_t)n, sizeof(real));
        if (!m[i]) return -1;
    }
    real *m_dvx_dx = m[0], *m_dvy_dy = m[1], *m_dvy_dx = m[2], *m_dvx_dy = m[3];
    real *m_dsxx_dx = m[4], *m_dsxy_dy = m[5], *m_dsxy_dx = m[6], *m_dsyy_dy = m[7];
    real *r_xx = NULL, *r_yy = NULL, *r_xy = NULL;
    if (L > 0) {
        r_xx = (real *)calloc((size_t)(n * L), sizeof(real));
        r_yy = (real *)calloc((size_t)(n * L), sizeof(real));
        r_xy = (real *)calloc((size_t)(n * L), sizeof(real));
        if (!r_xx || !r_yy || !r_xy) return -1;
    }
    const real dt = RD(d->dt), dx = RD(d->dx), dy = RD(d->dy);
    const long ntx = c.ntab_x, nty = c.ntab_y;

    for (int it = 0; it < d->n_steps; ++it) {
        /* ---- sigma_kernel (:829-984) ---- */
#pragma omp parallel for schedule(static)
        for (long x = 0; x < nx; ++x) {
            for (long y = 0; y < ny; ++y) {
                const long i = x * ny + y;
                if (x >= ord - 1 && x < nx - ord && y >= ord && y < ny - (ord - 1)) {
                    real ddx = RD(0), ddy = RD(0);
                    for (int k = 0; k < ord; ++k) {
                        ddx += RD(d->coefs[k]) * (FN(get)(&c, vx, x + k + 1, y, 0) - FN(get)(&c, vx, x - k, y, 0)) / dx;
                        ddy += RD(d->coefs[k]) * (FN(get)(&c, vy, x, y + k, 0) - FN(get)(&c, vy, x, y - k - 1, 0)) / dy;
                    }
                    ddx = FN(cpml)(ddx, &m_dvx_dx[i], FN(tab)(d->a_xh, x - off, ntx), FN(tab)(d->b_xh, x - off, ntx), FN(tab)(d->k_xh, x - off, ntx));
                    ddy = FN(cpml)(ddy, &m_dvy_dy[i], FN(tab)(d->a_y, y - off, nty), FN(tab)(d->b_y, y - off, nty), FN(tab)(d->k_y, y - off, nty));
                    real rho_h = RD(0.5) * (FN(getf)(&c, d->rho, x + 1, y, 0) + FN(getf)(&c, d->rho, x, y, 0));
                    real cp_h = RD(0.5) * (FN(getf)(&c, d->cp, x + 1, y, 0) + FN(getf)(&c, d->cp, x, y, 0));
                    real cs1 = FN(getf)(&c, d->cs, x + 1, y, 0), cs0 = FN(getf)(&c, d->cs, x, y, 0);
                    real cs_l = RD(0.5) * (cs1 + cs0);
                    real cs_m = ((cs1 < cs0 ? cs1 : cs0) == RD(0)) ? RD(0) : cs_l;
                    real lam = rho_h * (cp_h * cp_h - RD(2.0) * cs_l * cs_l);
                    real mu = rho_h * (cs_m * cs_m);
                    real l2m = lam + RD(2.0) * mu;
                    real lpm = lam + mu;
                    if (L > 0) {
                        real srxx = RD(0), sryy = RD(0);
                        for (int l = 0; l < L; ++l) {
                            FN(zener) z = FN(zener_at)(d, l, i);
                            real rxo = r_xx[i * L + l], ryo = r_yy[i * L + l];
                            real rxn = ((rxo + (ddx + ddy) * z.phi_p - rxo * z.h_p) * z.m_p);
                            real ryn = ((ryo + RD(0.5) * (ddx - ddy) * z.phi_s - ryo * z.h_s) * z.m_s);
                            srxx += rxo + rxn;
                            sryy += ryo + ryn;
                            r_xx[i * L + l] = rxn;
                            r_yy[i * L + l] = ryn;
                        }
                        sxx[i] = sxx[i] + (l2m * ddx + lam * ddy + RD(0.5) * lpm * srxx + mu * sryy) * dt;
                        syy[i] = syy[i] + (lam * ddx + l2m * ddy + RD(0.5) * lpm * srxx - mu * sryy) * dt;
                    } else {
                        sxx[i] = sxx[i] + (l2m * ddx + lam * ddy) * dt;
                        syy[i] = syy[i] + (lam * ddx + l2m * ddy) * dt;
                    }
                }
                if (x >= ord && x < nx - (ord - 1) && y >= ord - 1 && y < ny - ord) {
                    real dvy_dx = RD(0), dvx_dy = RD(0);
                    for (int k = 0; k < ord; ++k) {
                        dvy_dx += RD(d->coefs[k]) * (FN(get)(&c, vy, x + k, y, 0) - FN(get)(&c, vy, x - k - 1, y, 0)) / dx;
                        dvx_dy += RD(d->coefs[k]) * (FN(get)(&c, vx, x, y + k + 1, 0) - FN(get)(&c, vx, x, y - k, 0)) / dy;
                    }
                    dvy_dx = FN(cpml)(dvy_dx, &m_dvy_dx[i], FN(tab)(d->a_x, x - off, ntx), FN(tab)(d->b_x, x - off, ntx), FN(tab)(d->k_x, x - off, ntx));
                    dvx_dy = FN(cpml)(dvx_dy, &m_dvx_dy[i], FN(tab)(d->a_yh, y - off, nty), FN(tab)(d->b_yh, y - off, nty), FN(tab)(d->k_yh, y - off, nty));
                    real rho_h = RD(0.5) * (FN(getf)(&c, d->rho, x, y + 1, 0) + FN(getf)(&c, d->rho, x, y, 0));
                    real cs1 = FN(getf)(&c, d->cs, x, y + 1, 0), cs0 = FN(getf)(&c, d->cs, x, y, 0);
                    real cs_h = ((cs1 < cs0 ? cs1 : cs0) == RD(0)) ? RD(0) : (RD(0.5) * (cs1 + cs0));
                    real mu = rho_h * (cs_h * cs_h);
                    if (L > 0) {
                        real srxy = RD(0);
                        for (int l = 0; l < L; ++l) {
                            FN(zener) z = FN(zener_at)(d, l, i);
                            real ro = r_xy[i * L + l];
                            real rn = ((ro + (dvy_dx + dvx_dy) * z.phi_s - ro * z.h_s) * z.m_s);
                            srxy += ro + rn;
                            r_xy[i * L + l] = rn;
                        }
                        sxy[i] = sxy[i] + (mu * (dvy_dx + dvx_dy) + RD(0.5) * mu * srxy) * dt;
                    } else {
                        sxy[i] = sxy[i] + (dvx_dy + dvy_dx) * mu * dt;
                    }
                }
            }
        }
        /* ---- velocity_kernel (:987-1072) ---- */
        real vmax = RD(0);
#pragma omp parallel for schedule(static) reduction(max : vmax)
        for (long x = 0; x < nx; ++x) {
            for (long y = 0; y < ny; ++y) {
                const long i = x * ny + y;
                if (x >= ord && x < nx - (ord - 1) && y >= ord && y < ny - (ord - 1)) {
                    real dsxx = RD(0), dsxy = RD(0);
                    for (int k = 0; k < ord; ++k) {
                        dsxx += RD(d->coefs[k]) * (FN(get)(&c, sxx, x + k, y, 0) - FN(get)(&c, sxx, x - k - 1, y, 0)) / dx;
                        dsxy += RD(d->coefs[k]) * (FN(get)(&c, sxy, x, y + k, 0) - FN(get)(&c, sxy, x, y - k - 1, 0)) / dy;
                    }
                    dsxx = FN(cpml)(dsxx, &m_dsxx_dx[i], FN(tab)(d->a_x, x - off, ntx), FN(tab)(d->b_x, x - off, ntx), FN(tab)(d->k_x, x - off, ntx));
                    dsxy = FN(cpml)(dsxy, &m_dsxy_dy[i], FN(tab)(d->a_y, y - off, nty), FN(tab)(d->b_y, y - off, nty), FN(tab)(d->k_y, y - off, nty));
                    real rho = FN(getf)(&c, d->rho, x, y, 0);
                    if (rho > RD(0)) vx[i] = (dsxx + dsxy) * dt / rho + vx[i];
                }
                real rho4 = RD(0.25) * (FN(getf)(&c, d->rho, x, y, 0) + FN(getf)(&c, d->rho, x + 1, y, 0) +
                                        FN(getf)(&c, d->rho, x + 1, y + 1, 0) + FN(getf)(&c, d->rho, x, y + 1, 0));
                if (x >= ord - 1 && x < nx - ord && y >= ord - 1 && y < ny - ord) {
                    real dsxy_dx = RD(0), dsyy = RD(0);
                    for (int k = 0; k < ord; ++k) {
                        dsxy_dx += RD(d->coefs[k]) * (FN(get)(&c, sxy, x + k + 1, y, 0) - FN(get)(&c, sxy, x - k, y, 0)) / dx;
                        dsyy += RD(d->coefs[k]) * (FN(get)(&c, syy, x, y + k + 1, 0) - FN(get)(&c, syy, x, y - k, 0)) / dy;
                    }
                    dsxy_dx = FN(cpml)(dsxy_dx, &m_dsxy_dx[i], FN(tab)(d->a_xh, x - off, ntx), FN(tab)(d->b_xh, x - off, ntx), FN(tab)(d->k_xh, x - off, ntx));
                    dsyy = FN(cpml)(dsyy, &m_dsyy_dy[i], FN(tab)(d->a_yh, y - off, nty), FN(tab)(d->b_yh, y - off, nty), FN(tab)(d->k_yh, y - off, nty));
                    if (rho4 > RD(0)) vy[i] = (dsxy_dx + dsyy) * dt / rho4 + vy[i];
                } else {
                    vx[i] = RD(0);
                    vy[i] = RD(0);
                }
                int isrc = d->pos_sources[i];
                if (isrc != -1 && rho4 > RD(0)) {
                    real val = (it < d->n_steps && isrc < d->n_src_el && isrc >= 0)
                                   ? RD(d->source_term[(long)it * d->n_src_el + isrc]) : RD(0);
                    vy[i] = vy[i] + val * dt / rho4;
                }
                real v2 = vx[i] * vx[i] + vy[i] * vy[i];
                if (v2 > vmax || v2 != v2) vmax = v2;
            }
        }
        vmax2[it] = vmax;
        /* ---- store_sensors_kernel (:1118-1134) ---- */
        for (int sn = 0; sn < d->n_rec; ++sn) {
            int pt = FN(first_point)(d, sn, 3);
            while (pt >= 0 && pt < d->n_rec_pt && d->info_rec_pt[pt * 3 + 2] == sn) {
                if (it >= d->delay_rec[sn]) {
                    long x = d->info_rec_pt[pt * 3 + 0], y = d->info_rec_pt[pt * 3 + 1];
                    sens[(long)it * d->n_rec + sn] = sens[(long)it * d->n_rec + sn] + FN(get)(&c, syy, x, y, 0);
                }
                ++pt;
            }
        }
    }
    for (int i = 0; i < 8; ++i) free(m[i]);
    free(r_xx);
    free(r_yy);
    free(r_xy);
    return 0;
}

/* ===================================================================== */
/* WGSL 3D (visco)elastic (shader_webgpu_3D_viscoelastic.wgsl:1341-1850)   */
/* ===================================================================== */
#define G(a, X, Y, Z) FN(get)(&c, (a), (X), (Y), (Z))
#define GF(a, X, Y, Z) FN(getf)(&c, (a), (X), (Y), (Z))
#define T(t, n, nt) FN(tab)((t), (n), (nt))

static int FN(run_wgsl3d)(const ts_oracle_desc *d, real **v, real **s, real *sens, real *vmax2) {
    FN(ctx) c = {d, d->nx, d->ny, d->nz, d->nx - 2 * (d->ord - 1), d->ny - 2 * (d->ord - 1), d->nz - 2 * (d->ord - 1)};
    const long nx = c.nx, ny = c.ny, nz = c.nz, n = nx * ny * nz;
    const int ord = d->ord, off = ord - 1, L = d->visco ? d->n_sls : 0;
    const long ntx = c.ntab_x, nty = c.ntab_y, ntz = c.ntab_z;
    real *vx = v[0], *vy = v[1], *vz = v[2];
    real *sxx = s[0], *syy = s[1], *szz = s[2], *sxy = s[3], *sxz = s[4], *syz = s[5];
    real *m[18];
    for (int i = 0; i < 18; ++i) {
        m[i] = (real *)calloc((size_t)n, sizeof(real));
        if (!m[i]) return -1;
    }
    /* velocity-derivative memories (stress kernel) */
    real *m_dvx_dx = m[0], *m_dvy_dy = m[1], *m_dvz_dz = m[2], *m_dvy_dx = m[3], *m_dvx_dy = m[4];
    real *m_dvz_dx = m[5], *m_dvx_dz = m[6], *m_dvz_dy = m[7], *m_dvy_dz = m[8];
    /* stress-derivative memories (velocity kernel) */
    real *m_dsxx_dx = m[9], *m_dsxy_dy = m[10], *m_dsxz_dz = m[11], *m_dsxy_dx = m[12], *m_dsyy_dy = m[13];
    real *m_dsyz_dz = m[14], *m_dsxz_dx = m[15], *m_dsyz_dy = m[16], *m_dszz_dz = m[17];
    real *r[6] = {NULL, NULL, NULL, NULL, NULL, NULL};
    for (int i = 0; i < 6 && L > 0; ++i) {
        r[i] = (real *)calloc((size_t)(n * L), sizeof(real));
        if (!r[i]) return -1;
    }
    const real dt = RD(d->dt), dx = RD(d->dx), dy = RD(d->dy), dz = RD(d->dz);
    const real third = RD(3.0);

    for (int it = 0; it < d->n_steps; ++it) {
        /* ---- sigma_kernel (:1341-1631) ---- */
#pragma omp parallel for schedule(static) collapse(2)
        for (long x = 0; x < nx; ++x) {
            for (long y = 0; y < ny; ++y) {
                for (long z = 0; z < nz; ++z) {
                    const long i = (x * ny + y) * nz + z;
                    if (x >= ord - 1 && x < nx - ord && y >= ord && y < ny - (ord - 1) && z >= ord && z < nz - (ord - 1)) {
                        real ddx = RD(0), ddy = RD(0), ddz = RD(0);
                        for (int k = 0; k < ord; ++k) {
                            ddx += RD(d->coefs[k]) * (G(vx, x + k + 1, y, z) - G(vx, x - k, y, z)) / dx;
                            ddy += RD(d->coefs[k]) * (G(vy, x, y + k, z) - G(vy, x, y - k - 1, z)) / dy;
                            ddz += RD(d->coefs[k]) * (G(vz, x, y, z + k) - G(vz, x, y, z - k - 1)) / dz;
                        }
                        ddx = FN(cpml)(ddx, &m_dvx_dx[i], T(d->a_xh, x - off, ntx), T(d->b_xh, x - off, ntx), T(d->k_xh, x - off, ntx));
                        ddy = FN(cpml)(ddy, &m_dvy_dy[i], T(d->a_y, y - off, nty), T(d->b_y, y - off, nty), T(d->k_y, y - off, nty));
                        ddz = FN(cpml)(ddz, &m_dvz_dz[i], T(d->a_z, z - off, ntz), T(d->b_z, z - off, ntz), T(d->k_z, z - off, ntz));
                        real rho = GF(d->rho, x, y, z), cp = GF(d->cp, x, y, z), cs = GF(d->cs, x, y, z);
                        real lam = rho * (cp * cp - RD(2.0) * cs * cs);
                        real mu = rho * (cs * cs);
                        real l2m = lam + RD(2.0) * mu;
                        if (L > 0) {
                            real srxx = RD(0), sryy = RD(0), srzz = RD(0);
                            real div = ddx + ddy + ddz;
                            for (int l = 0; l < L; ++l) {
                                FN(zener) zz = FN(zener_at)(d, l, i);
                                real xo = r[0][i * L + l], yo = r[1][i * L + l], zo = r[2][i * L + l];
                                real xn = ((xo + div * zz.phi_p - xo * zz.h_p) * zz.m_p);
                                real yn = ((yo + (ddx - div / third) * zz.phi_s - yo * zz.h_s) * zz.m_s);
                                real zn = ((zo + (ddy - div / third) * zz.phi_s - zo * zz.h_s) * zz.m_s);
                                srxx += xo + xn;
                                sryy += yo + yn;
                                srzz += zo + zn;
                                r[0][i * L + l] = xn;
                                r[1][i * L + l] = yn;
                                r[2][i * L + l] = zn;
                            }
                            real l23 = lam + RD(2.0) * mu / third;
                            sxx[i] = sxx[i] + (l2m * ddx + lam * (ddy + ddz) + l23 * RD(0.5) * srxx + mu * sryy) * dt;
                            syy[i] = syy[i] + (lam * (ddx + ddz) + l2m * ddy + l23 * RD(0.5) * srxx + mu * srzz) * dt;
                            szz[i] = szz[i] + (lam * (ddx + ddy) + l2m * ddz + l2m * RD(0.5) * srxx - (mu / third) * (sryy + srzz)) * dt;
                        } else {
                            sxx[i] = sxx[i] + (l2m * ddx + lam * (ddy + ddz)) * dt;
                            syy[i] = syy[i] + (lam * (ddx + ddz) + l2m * ddy) * dt;
                            szz[i] = szz[i] + (lam * (ddx + ddy) + l2m * ddz) * dt;
                        }
                    }
                    /* sigma_xy (:1458-1516) and sigma_xz (:1519-1572) share their region */
                    if (x >= ord && x < nx - (ord - 1) && y >= ord - 1 && y < ny - ord && z >= ord - 1 && z < nz - ord) {
                        real a1 = RD(0), a2 = RD(0);
                        for (int k = 0; k < ord; ++k) {
                            a1 += RD(d->coefs[k]) * (G(vy, x + k, y, z) - G(vy, x - k - 1, y, z)) / dx;
                            a2 += RD(d->coefs[k]) * (G(vx, x, y + k + 1, z) - G(vx, x, y - k, z)) / dy;
                        }
                        a1 = FN(cpml)(a1, &m_dvy_dx[i], T(d->a_x, x - off, ntx), T(d->b_x, x - off, ntx), T(d->k_x, x - off, ntx));
                        a2 = FN(cpml)(a2, &m_dvx_dy[i], T(d->a_yh, y - off, nty), T(d->b_yh, y - off, nty), T(d->k_yh, y - off, nty));
                        real rho = RD(0.25) * (GF(d->rho, x + 1, y, z) + GF(d->rho, x, y, z) + GF(d->rho, x, y + 1, z) + GF(d->rho, x + 1, y + 1, z));
                        real cs = RD(0.25) * (GF(d->cs, x + 1, y, z) + GF(d->cs, x, y, z) + GF(d->cs, x, y + 1, z) + GF(d->cs, x + 1, y + 1, z));
                        real mu = rho * (cs * cs);
                        if (L > 0) {
                            real sr = RD(0);
                            for (int l = 0; l < L; ++l) {
                                FN(zener) zz = FN(zener_at)(d, l, i);
                                real o = r[3][i * L + l];
                                real nn = ((o + (a1 + a2) * zz.phi_s - o * zz.h_s) * zz.m_s);
                                sr += o + nn;
                                r[3][i * L + l] = nn;
                            }
                            sxy[i] = sxy[i] + (mu * (a1 + a2) + mu * RD(0.5) * sr) * dt;
                        } else {
                            sxy[i] = sxy[i] + (a2 + a1) * mu * dt;
                        }
                        real b1 = RD(0), b2 = RD(0);
                        for (int k = 0; k < ord; ++k) {
                            b1 += RD(d->coefs[k]) * (G(vz, x + k, y, z) - G(vz, x - k - 1, y, z)) / dx;
                            b2 += RD(d->coefs[k]) * (G(vx, x, y, z + k + 1) - G(vx, x, y, z - k)) / dz;
                        }
                        b1 = FN(cpml)(b1, &m_dvz_dx[i], T(d->a_x, x - off, ntx), T(d->b_x, x - off, ntx), T(d->k_x, x - off, ntx));
                        b2 = FN(cpml)(b2, &m_dvx_dz[i], T(d->a_zh, z - off, ntz), T(d->b_zh, z - off, ntz), T(d->k_zh, z - off, ntz));
                        rho = RD(0.25) * (GF(d->rho, x + 1, y, z) + GF(d->rho, x, y, z) + GF(d->rho, x, y, z + 1) + GF(d->rho, x + 1, y, z + 1));
                        cs = RD(0.25) * (GF(d->cs, x + 1, y, z) + GF(d->cs, x, y, z) + GF(d->cs, x, y, z + 1) + GF(d->cs, x + 1, y, z + 1));
                        mu = rho * (cs * cs);
                        if (L > 0) {
                            real sr = RD(0);
                            for (int l = 0; l < L; ++l) {
                                FN(zener) zz = FN(zener_at)(d, l, i);
                                real o = r[4][i * L + l];
                                real nn = (o + (b1 + b2) * zz.phi_s - o * zz.h_s) * zz.m_s;
                                sr += o + nn;
                                r[4][i * L + l] = nn;
                            }
                            sxz[i] = sxz[i] + (mu * (b2 + b1) + mu * RD(0.5) * sr) * dt;
                        } else {
                            sxz[i] = sxz[i] + (b2 + b1) * mu * dt;
                        }
                    }
                    /* sigma_yz (:1576-1629) */
                    if (x >= ord - 1 && x < nx - ord && y >= ord - 1 && y < ny - ord && z >= ord - 1 && z < nz - ord) {
                        real a1 = RD(0), a2 = RD(0);
                        for (int k = 0; k < ord; ++k) {
                            a1 += RD(d->coefs[k]) * (G(vz, x, y + k + 1, z) - G(vz, x, y - k, z)) / dy;
                            a2 += RD(d->coefs[k]) * (G(vy, x, y, z + k + 1) - G(vy, x, y, z - k)) / dz;
                        }
                        a1 = FN(cpml)(a1, &m_dvz_dy[i], T(d->a_yh, y - off, nty), T(d->b_yh, y - off, nty), T(d->k_yh, y - off, nty));
                        a2 = FN(cpml)(a2, &m_dvy_dz[i], T(d->a_zh, z - off, ntz), T(d->b_zh, z - off, ntz), T(d->k_zh, z - off, ntz));
                        real rho = RD(0.25) * (GF(d->rho, x, y + 1, z) + GF(d->rho, x, y, z) + GF(d->rho, x, y, z + 1) + GF(d->rho, x, y + 1, z + 1));
                        real cs = RD(0.25) * (GF(d->cs, x, y + 1, z) + GF(d->cs, x, y, z) + GF(d->cs, x, y, z + 1) + GF(d->cs, x, y + 1, z + 1));
                        real mu = rho * (cs * cs);
                        if (L > 0) {
                            real sr = RD(0);
                            for (int l = 0; l < L; ++l) {
                                FN(zener) zz = FN(zener_at)(d, l, i);
                                real o = r[5][i * L + l];
                                real nn = (o + (a2 + a1) * zz.phi_s - o * zz.h_s) * zz.m_s;
                                sr += o + nn;
                                r[5][i * L + l] = nn;
                            }
                            syz[i] = syz[i] + (mu * (a2 + a1) + mu * RD(0.5) * sr) * dt;
                        } else {
                            syz[i] = syz[i] + (a2 + a1) * mu * dt;
                        }
                    }
                }
            }
        }
        /* ---- velocity_kernel (:1634-1773) ---- */
        real vmax = RD(0);
#pragma omp parallel for schedule(static) collapse(2) reduction(max : vmax)
        for (long x = 0; x < nx; ++x) {
            for (long y = 0; y < ny; ++y) {
                for (long z = 0; z < nz; ++z) {
                    const long i = (x * ny + y) * nz + z;
                    if (x >= ord && x < nx - (ord - 1) && y >= ord && y < ny - (ord - 1) && z >= ord && z < nz - (ord - 1)) {
                        real a = RD(0), b = RD(0), e = RD(0);
                        for (int k = 0; k < ord; ++k) {
                            a += RD(d->coefs[k]) * (G(sxx, x + k, y, z) - G(sxx, x - k - 1, y, z)) / dx;
                            b += RD(d->coefs[k]) * (G(sxy, x, y + k, z) - G(sxy, x, y - k - 1, z)) / dy;
                            e += RD(d->coefs[k]) * (G(sxz, x, y, z + k) - G(sxz, x, y, z - k - 1)) / dz;
                        }
                        a = FN(cpml)(a, &m_dsxx_dx[i], T(d->a_x, x - off, ntx), T(d->b_x, x - off, ntx), T(d->k_x, x - off, ntx));
                        b = FN(cpml)(b, &m_dsxy_dy[i], T(d->a_y, y - off, nty), T(d->b_y, y - off, nty), T(d->k_y, y - off, nty));
                        e = FN(cpml)(e, &m_dsxz_dz[i], T(d->a_z, z - off, ntz), T(d->b_z, z - off, ntz), T(d->k_z, z - off, ntz));
                        real rho = RD(0.5) * (GF(d->rho, x + 1, y, z) + GF(d->rho, x, y, z));
                        if (rho > RD(0)) vx[i] = (a + b + e) * dt / rho + vx[i];
                    }
                    real rho_y = RD(0.5) * (GF(d->rho, x, y + 1, z) + GF(d->rho, x, y, z));
                    if (x >= ord - 1 && x < nx - ord && y >= ord - 1 && y < ny - ord && z >= ord && z < nz - (ord - 1)) {
                        real a = RD(0), b = RD(0), e = RD(0);
                        for (int k = 0; k < ord; ++k) {
                            a += RD(d->coefs[k]) * (G(sxy, x + k + 1, y, z) - G(sxy, x - k, y, z)) / dx;
                            b += RD(d->coefs[k]) * (G(syy, x, y + k + 1, z) - G(syy, x, y - k, z)) / dy;
                            e += RD(d->coefs[k]) * (G(syz, x, y, z + k) - G(syz, x, y, z - k - 1)) / dz;
                        }
                        a = FN(cpml)(a, &m_dsxy_dx[i], T(d->a_xh, x - off, ntx), T(d->b_xh, x - off, ntx), T(d->k_xh, x - off, ntx));
                        b = FN(cpml)(b, &m_dsyy_dy[i], T(d->a_yh, y - off, nty), T(d->b_yh, y - off, nty), T(d->k_yh, y - off, nty));
                        e = FN(cpml)(e, &m_dsyz_dz[i], T(d->a_z, z - off, ntz), T(d->b_z, z - off, ntz), T(d->k_z, z - off, ntz));
                        if (rho_y > RD(0)) vy[i] = (a + b + e) * dt / rho_y + vy[i];
                    }
                    if (x >= ord - 1 && x < nx - ord && y >= ord && y < ny - (ord - 1) && z >= ord - 1 && z < nz - ord) {
                        real a = RD(0), b = RD(0), e = RD(0);
                        for (int k = 0; k < ord; ++k) {
                            a += RD(d->coefs[k]) * (G(sxz, x + k + 1, y, z) - G(sxz, x - k, y, z)) / dx;
                            b += RD(d->coefs[k]) * (G(syz, x, y + k, z) - G(syz, x, y - k - 1, z)) / dy;
                            e += RD(d->coefs[k]) * (G(szz, x, y, z + k + 1) - G(szz, x, y, z - k)) / dz;
                        }
                        a = FN(cpml)(a, &m_dsxz_dx[i], T(d->a_xh, x - off, ntx), T(d->b_xh, x - off, ntx), T(d->k_xh, x - off, ntx));
                        b = FN(cpml)(b, &m_dsyz_dy[i], T(d->a_y, y - off, nty), T(d->b_y, y - off, nty), T(d->k_y, y - off, nty));
                        e = FN(cpml)(e, &m_dszz_dz[i], T(d->a_zh, z - off, ntz), T(d->b_zh, z - off, ntz), T(d->k_zh, z - off, ntz));
                        if (rho_y > RD(0)) vz[i] = (a + b + e) * dt / rho_y + vz[i];
                    } else {
                        vx[i] = RD(0);
                        vy[i] = RD(0);
                        vz[i] = RD(0);
                    }
                    int isrc = d->pos_sources[i];
                    if (isrc != -1 && rho_y > RD(0)) {
                        real val = (it < d->n_steps && isrc < d->n_src_el && isrc >= 0)
                                       ? RD(d->source_term[(long)it * d->n_src_el + isrc]) : RD(0);
                        vz[i] = vz[i] + val * dt / rho_y;
                    }
                    real v2 = vx[i] * vx[i] + vy[i] * vy[i] + vz[i] * vz[i];
                    if (v2 > vmax || v2 != v2) vmax = v2;
                }
            }
        }
        vmax2[it] = vmax;
        /* ---- store_sensors_kernel (:1824-1843) ---- */
        for (int sn = 0; sn < d->n_rec; ++sn) {
            int pt = FN(first_point)(d, sn, 4);
            while (pt >= 0 && pt < d->n_rec_pt && d->info_rec_pt[pt * 4 + 3] == sn) {
                if (it >= d->delay_rec[sn]) {
                    long x = d->info_rec_pt[pt * 4 + 0], y = d->info_rec_pt[pt * 4 + 1], z = d->info_rec_pt[pt * 4 + 2];
                    sens[(long)it * d->n_rec + sn] = sens[(long)it * d->n_rec + sn] + G(szz, x, y, z);
                }
                ++pt;
            }
        }
    }
    for (int i = 0; i < 18; ++i) free(m[i]);
    for (int i = 0; i < 6; ++i) free(r[i]);
    return 0;
}
#undef G
#undef GF
#undef T

int FN(ts_oracle_run)(const ts_oracle_desc *d, real **v, real **s, real *sens, real *vmax2) {
    switch (d->family) {
    case TS_ORC_TAICHI2D: return FN(run_taichi2d)(d, v, s, sens, vmax2);
    case TS_ORC_WGSL2D: return FN(run_wgsl2d)(d, v, s, sens, vmax2);
    case TS_ORC_WGSL3D: return FN(run_wgsl3d)(d, v, s, sens, vmax2);
    default: return -2;
    }
}
#undef RD
