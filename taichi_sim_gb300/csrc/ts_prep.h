// Host-side preparation shared by the single-simulation and batched entry
// points: CPML node tables and strips, per-node coefficients with the
// reference's averaging, Zener constants in update form.  Internal.
#pragma once
#include <algorithm>
#include <cstdint>
#include <vector>

#include "../../include/taichi_sim_gb300.h"
#include "ts_internal.cuh"

namespace ts {

struct Axis {
    std::vector<Cpml> full, half;
    Strip strip;
};

inline bool cpml_identity(const Cpml &c) { return c.a == 0.f && c.b == 1.f && c.ik == 1.f; }

// CPML tables of one axis re-indexed by grid node (table index = node - (ord-1));
// the strip is the prefix/suffix of nodes whose tables differ from the identity.
inline Axis make_axis(int n, int ord, const float *a, const float *b, const float *k, const float *ah,
                      const float *bh, const float *kh) {
    Axis ax;
    const int off = ord - 1, ntab = n - 2 * (ord - 1);
    ax.full.assign(n, Cpml{0.f, 1.f, 1.f, 1.f});
    ax.half.assign(n, Cpml{0.f, 1.f, 1.f, 1.f});
    std::vector<char> nonid(n, 0);
    for (int x = 0; x < n; ++x) {
        const int t = x - off;
        if (t < 0 || t >= ntab || !a) continue;
        ax.full[x] = Cpml{a[t], b[t], 1.f / k[t], k[t]};
        ax.half[x] = Cpml{ah[t], bh[t], 1.f / kh[t], kh[t]};
        nonid[x] = !cpml_identity(ax.full[x]) || !cpml_identity(ax.half[x]);
    }
    int lo = 0, hi = n;
    for (int x = 0; x < n / 2; ++x)
        if (nonid[x]) lo = x + 1;
    for (int x = n - 1; x >= n / 2; --x)
        if (nonid[x]) hi = x;
    ax.strip = Strip{lo, hi, lo + (n - hi)};
    return ax;
}

inline int round_up(int v, int m) { return (v + m - 1) / m * m; }

// First receiver point the WGSL kernels read for receiver r: offset_sensors
// has one entry per group of equal receiver ids in info_rec_pt
// (sim_support/simulator.py:289-294), which is fewer than n_rec when some
// receiving elements lie outside the ROI; an entry past its end reads as
// "no point" (-1) instead of past the array.
inline int receiver_groups(const ts_desc *d, int cols) {
    if (d->n_rec_pt <= 0) return 0;
    int groups = 1;
    for (int pt = 1; pt < d->n_rec_pt; ++pt)
        if (d->info_rec_pt[pt * cols + cols - 1] != d->info_rec_pt[(pt - 1) * cols + cols - 1]) ++groups;
    return groups;
}
// (groups: receiver_groups(d, cols), counted once per table, not per receiver)
inline int receiver_first_point(const ts_desc *d, int r, int groups) {
    return r < groups ? d->offset_sensors[r] : -1;
}

// Per-node coefficients of a 2D model (families TS_TAICHI2D / TS_WGSL2D),
// folded with dt, for node (x, y) of an nx x ny grid of the reference's
// tables (sim_taichi_elastic.py:171-178, 223-227, 263, 293;
// shader_webgpu_viscoelastic.wgsl:863-868, 948-950, 1020, 1032).
struct Coef2D {
    float lam, mu, mus, dtr_vx, dtr_vy, rho_vy;
    float lam_raw, mu_raw, mus_raw, rho_vx;   // the same before folding with dt
};

inline Coef2D coef_2d(const ts_desc *d, int x, int y) {
    const int nx = d->nx, ny = d->ny;
    auto g = [&](const float *a, int xx, int yy) -> float {
        return (xx < 0 || xx >= nx || yy < 0 || yy >= ny) ? 0.f : a[(int64_t)xx * ny + yy];
    };
    const float dt = d->dt;
    Coef2D c;
    const float rh = 0.5f * (g(d->rho, x + 1, y) + g(d->rho, x, y));
    const float cph = 0.5f * (g(d->cp, x + 1, y) + g(d->cp, x, y));
    const float c1 = g(d->cs, x + 1, y), c0 = g(d->cs, x, y);
    const float csl = 0.5f * (c1 + c0);
    const float csm = std::min(c1, c0) == 0.f ? 0.f : csl;
    c.lam_raw = rh * (cph * cph - 2.f * csl * csl);
    c.mu_raw = rh * (csm * csm);
    c.lam = c.lam_raw * dt;
    c.mu = c.mu_raw * dt;
    const float rhy = 0.5f * (g(d->rho, x, y + 1) + g(d->rho, x, y));
    const float s1 = g(d->cs, x, y + 1), s0 = g(d->cs, x, y);
    const float csh = std::min(s1, s0) == 0.f ? 0.f : 0.5f * (s1 + s0);
    c.mus_raw = rhy * (csh * csh);
    c.mus = c.mus_raw * dt;
    const float r = g(d->rho, x, y);
    c.rho_vx = r;
    c.dtr_vx = r > 0.f ? dt / r : 0.f;
    c.rho_vy = d->family == TS_TAICHI2D
                   ? 0.25f * (g(d->rho, x, y + 1) + g(d->rho, x, y) + g(d->rho, x + 1, y + 1) + g(d->rho, x + 1, y))
                   : 0.25f * (g(d->rho, x, y) + g(d->rho, x + 1, y) + g(d->rho, x + 1, y + 1) + g(d->rho, x, y + 1));
    c.dtr_vy = c.rho_vy > 0.f ? dt / c.rho_vy : 0.f;
    return c;
}

// Zener constants in update form r' = A r + B d (shader_webgpu_viscoelastic.wgsl:881-894
// for global taus; per-cell Q: phi = zc * g, relaxation zh, zm).
inline Zener zener_constants(const ts_desc *d) {
    Zener z{};
    if (!d->visco) return z;
    const int L = d->n_sls;
    const float dt = d->dt;
    z.n = L;
    for (int l = 0; l < L; ++l) {
        float hp, hs, mp, ms, bp, bs;
        if (!d->g_p) {
            const float inv_p = 1.f / d->tau[1 * L + l], inv_s = 1.f / d->tau[3 * L + l];
            const float ap = d->tau[0 * L + l] / d->tau[1 * L + l], as = d->tau[2 * L + l] / d->tau[3 * L + l];
            const float php = dt * (1.f - ap) * inv_p / d->sum_alpha[0];
            const float phs = dt * (1.f - as) * inv_s / d->sum_alpha[1];
            hp = 0.5f * dt * inv_p;
            hs = 0.5f * dt * inv_s;
            mp = 1.f / (1.f + hp);
            ms = 1.f / (1.f + hs);
            bp = php * mp;
            bs = phs * ms;
        } else {
            hp = hs = d->zh[l];
            mp = ms = d->zm[l];
            bp = bs = d->zc[l] * d->zm[l];
        }
        z.Ap[l] = (1.f - hp) * mp;
        z.As[l] = (1.f - hs) * ms;
        z.Bp[l] = bp;
        z.Bs[l] = bs;
    }
    return z;
}

}  // namespace ts
