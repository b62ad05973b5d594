"""Differentiable FP64 transcription of the WGSL 2D (visco)elastic time step
in torch: TEST INFRASTRUCTURE ONLY.

Only ``tests/`` use it, as the checker of the GPU adjoint: autograd through
this transcription gives the exact gradient of the same discrete forward, in
double precision, to compare the hand-written adjoint against.  It follows
shader_webgpu_viscoelastic.wgsl line by line, vectorised over the grid:

* sigma_kernel (:829-984): normal stresses on x in [ord-1, nx-ord),
  y in [ord, ny-ord+1); shear stress on x in [ord, nx-ord+1),
  y in [ord-1, ny-ord); material averaged per node (rho, cp over x+1 for
  the normal node, cs with the cs == 0 branch; rho, cs over y+1 for the
  shear node); L-mechanism Zener memory variables (:881-894, :906-940);
* velocity_kernel (:987-1072): vx on x in [ord, nx-ord+1),
  y in [ord, ny-ord+1) divided by rho; vy on x in [ord-1, nx-ord),
  y in [ord-1, ny-ord) divided by the 4-node rho average; both zero outside
  the vy region; source force source_term[it * n_src_el + idx] / rho4 at
  every node of the source map;
* store_sensors_kernel (:1118-1134): each receiver sums syy over its points
  from step delay_rec on.

CPML (:92-96, :850-860): psi' = b psi + a d, d~ = d / k + psi'.  The
per-cell Q extension uses phi = c_l * g(cell) with per-mechanism h, m.
The material is given per cell as (lambda, mu, rho); cp and cs are
recovered per cell, as the host model stores them.
"""
import numpy as np
import torch


def _sh(a, dx, dy):
    """out[x, y] = a[x + dx, y + dy], zero where that is outside the grid."""
    nx, ny = a.shape
    pad = max(abs(dx), abs(dy), 1)
    p = torch.nn.functional.pad(a, (pad, pad, pad, pad))
    return p[pad + dx:pad + dx + nx, pad + dy:pad + dy + ny]


def _mask(nx, ny, x0, x1, y0, y1, device):
    x = torch.arange(nx, device=device)[:, None]
    y = torch.arange(ny, device=device)[None, :]
    return (x >= x0) & (x < x1) & (y >= y0) & (y < y1)


class Wgsl2D:
    """The reference's 2D WGSL forward for one host model, differentiable in
    the per-cell material."""

    def __init__(self, sim, visco=None, dtype=torch.float64, device="cpu"):
        self.dtype, self.device = dtype, torch.device(device)
        self.nx, self.ny = sim.grid_shape()
        self.ord = int(sim._coefs.shape[0])
        self.coefs = [float(c) for c in np.asarray(sim._coefs, np.float32)]
        roi = sim._roi
        self.dx, self.dy = float(np.float32(roi.get_dx())), float(np.float32(roi.get_dz()))
        self.dt = float(np.float32(sim._dt))
        self.n_steps = int(sim._n_steps)
        if visco is None:
            visco = bool(sim._configs.get("simul_configs", {}).get("viscoelastic_attn", 0))
        self.visco = visco
        nx, ny, off = self.nx, self.ny, self.ord - 1
        T = lambda a: torch.as_tensor(np.asarray(a, np.float64), dtype=dtype, device=self.device)

        def table(name, n, along_x):
            t = np.asarray(getattr(sim, name), np.float64).reshape(-1)
            full = np.zeros(n) if not name.startswith("_k") else np.ones(n)
            full[off:off + t.size] = t[:max(0, min(t.size, n - off))]
            v = T(full)
            return v[:, None] if along_x else v[None, :]

        self.cx = {c: table(f"_{c}_x", nx, True) for c in "abk"}
        self.cxh = {c: table(f"_{c}_x_half", nx, True) for c in "abk"}
        self.cy = {c: table(f"_{c}_y", ny, False) for c in "abk"}
        self.cyh = {c: table(f"_{c}_y_half", ny, False) for c in "abk"}
        o = self.ord
        dev = self.device
        self.m_n = _mask(nx, ny, o - 1, nx - o, o, ny - o + 1, dev)
        self.m_s = _mask(nx, ny, o, nx - o + 1, o - 1, ny - o, dev)
        self.m_vx = _mask(nx, ny, o, nx - o + 1, o, ny - o + 1, dev)
        self.m_vy = _mask(nx, ny, o - 1, nx - o, o - 1, ny - o, dev)
        # Zener constants (phi, h, m) per mechanism, scalars or per-cell grids
        self.zener = []
        if visco:
            fit = getattr(sim, "_zener_fit", None)
            if fit is not None:
                c, h, m = (np.asarray(v, np.float64) for v in fit.mechanism_constants(sim._dt))
                gp = T(np.asarray(fit.cell_scale(sim._inv_qp_grid), np.float32))
                gs = T(np.asarray(fit.cell_scale(sim._inv_qs_grid), np.float32))
                for l in range(fit.n_sls):
                    cl = float(np.float32(c[l]))
                    hl, ml = float(np.float32(h[l])), float(np.float32(m[l]))
                    self.zener.append((cl * gp, cl * gs, hl, hl, ml, ml))
            else:
                from taichi_sim_gb300.sim_support.attenuation import AttenuationCoefficients
                att = AttenuationCoefficients()
                L = att._n_sls
                tau = np.asarray(att.tau_table(), np.float32).reshape(4, L).astype(np.float64)
                sa = np.asarray(att.sum_alpha(), np.float32).astype(np.float64)
                dt = self.dt
                for l in range(L):
                    inv_p, inv_s = 1.0 / tau[1, l], 1.0 / tau[3, l]
                    a_p, a_s = tau[0, l] / tau[1, l], tau[2, l] / tau[3, l]
                    hp, hs = 0.5 * dt * inv_p, 0.5 * dt * inv_s
                    self.zener.append((dt * (1 - a_p) * inv_p / sa[0], dt * (1 - a_s) * inv_s / sa[1],
                                       hp, hs, 1.0 / (1.0 + hp), 1.0 / (1.0 + hs)))
        # sources: nodes of the source map, value source_term.flat[it * n_src_el + idx]
        st = np.asarray(sim._source_term, np.float32)
        st = st[:, None] if st.ndim == 1 else st
        self.src_flat = T(st.reshape(-1))
        self.n_src_el = int(sim._n_src)
        pos = np.asarray(sim._pos_sources, np.int64).reshape(nx, ny)
        nodes = np.nonzero(pos.reshape(-1) != -1)[0]
        self.src_nodes = torch.as_tensor(nodes, device=dev)
        self.src_idx = torch.as_tensor(pos.reshape(-1)[nodes], device=dev)
        # receivers: points of receiver s from offset_sensors[s] while the id matches
        self.n_rec = int(sim._n_rec)
        info = np.asarray(sim._info_rec_pt, np.int64).reshape(-1, 3)
        offs = np.asarray(sim._offset_sensors, np.int64).reshape(-1)
        ids = info[:, 2]
        groups = 1 + int(np.count_nonzero(ids[1:] != ids[:-1])) if len(ids) else 0
        rec, cell = [], []
        for s in range(self.n_rec):
            pt = int(offs[s]) if s < groups else -1
            while 0 <= pt < len(info) and ids[pt] == s:
                rec.append(s)
                cell.append(int(info[pt, 0]) * ny + int(info[pt, 1]))
                pt += 1
        self.rec_ids = torch.as_tensor(np.asarray(rec, np.int64), device=dev)
        self.rec_cells = torch.as_tensor(np.asarray(cell, np.int64), device=dev)
        self.delay = torch.as_tensor(np.asarray(sim._delay_recv, np.int64).reshape(-1)[:self.n_rec], device=dev)

    def material(self, sim):
        T = lambda a: torch.as_tensor(np.asarray(a, np.float32).astype(np.float64), dtype=self.dtype,
                                      device=self.device)
        rho, cp, cs = T(sim._rho_grid_vx), T(sim._cp_grid_vx), T(sim._cs_grid_vx)
        mu = rho * cs * cs
        return rho * cp * cp - 2 * mu, mu, rho

    def _d(self, f, axis, lo, hi, step):
        """sum_k c_k (f[. + k + lo] - f[. - k + hi]) / step along `axis`."""
        acc = torch.zeros_like(f)
        for k, c in enumerate(self.coefs):
            if axis == 0:
                acc = acc + c * (_sh(f, k + lo, 0) - _sh(f, -k + hi, 0)) / step
            else:
                acc = acc + c * (_sh(f, 0, k + lo) - _sh(f, 0, -k + hi)) / step
        return acc

    @staticmethod
    def _cpml(d, psi, t, mask):
        p = torch.where(mask, t["b"] * psi + t["a"] * d, psi)
        return d / t["k"] + p, p

    def traces(self, lam, mu, rho, n_steps=None):
        """Receiver traces ``[n_steps][n_rec]`` from a zero state."""
        n_steps = self.n_steps if n_steps is None else int(n_steps)
        dt = self.dt
        z = lambda: torch.zeros((self.nx, self.ny), dtype=self.dtype, device=self.device)
        cs = torch.sqrt(mu / rho)
        cp = torch.sqrt((lam + 2 * mu) / rho)
        # material per node (sigma_kernel :863-868, :948-950; velocity_kernel :1020, :1032)
        rho_h = 0.5 * (_sh(rho, 1, 0) + rho)
        cp_h = 0.5 * (_sh(cp, 1, 0) + cp)
        cs1, cs0 = _sh(cs, 1, 0), cs
        cs_l = 0.5 * (cs1 + cs0)
        cs_m = torch.where(torch.minimum(cs1, cs0) == 0, torch.zeros_like(cs_l), cs_l)
        lam_n = rho_h * (cp_h * cp_h - 2.0 * cs_l * cs_l)
        mu_n = rho_h * (cs_m * cs_m)
        l2m, lpm = lam_n + 2.0 * mu_n, lam_n + mu_n
        rho_s = 0.5 * (_sh(rho, 0, 1) + rho)
        s1 = _sh(cs, 0, 1)
        cs_h = torch.where(torch.minimum(s1, cs0) == 0, torch.zeros_like(cs), 0.5 * (s1 + cs0))
        mu_s = rho_s * (cs_h * cs_h)
        rho4 = 0.25 * (rho + _sh(rho, 1, 0) + _sh(rho, 1, 1) + _sh(rho, 0, 1))
        one = torch.ones_like(rho)
        upd_vx = self.m_vx & (rho > 0)
        upd_vy = self.m_vy & (rho4 > 0)
        inv_rho = torch.where(rho > 0, 1.0 / torch.where(rho > 0, rho, one), torch.zeros_like(rho))
        inv_rho4 = torch.where(rho4 > 0, 1.0 / torch.where(rho4 > 0, rho4, one), torch.zeros_like(rho))
        src_scale = (dt * inv_rho4).reshape(-1)[self.src_nodes]
        src_ok = (self.src_idx >= 0) & (self.src_idx < self.n_src_el) & (rho4.reshape(-1)[self.src_nodes] > 0)

        vx, vy, sxx, syy, sxy = z(), z(), z(), z(), z()
        psi = [z() for _ in range(8)]
        L = len(self.zener)
        rxx, ryy, rxy = [z() for _ in range(L)], [z() for _ in range(L)], [z() for _ in range(L)]
        out = []
        for it in range(n_steps):
            # ---- sigma_kernel ----
            ddx = self._d(vx, 0, 1, 0, self.dx)
            ddy = self._d(vy, 1, 0, -1, self.dy)
            ddx, psi[0] = self._cpml(ddx, psi[0], self.cxh, self.m_n)
            ddy, psi[1] = self._cpml(ddy, psi[1], self.cy, self.m_n)
            ux = l2m * ddx + lam_n * ddy
            uy = lam_n * ddx + l2m * ddy
            if L:
                srxx, sryy = z(), z()
                for l, (php, phs, hp, hs, mp, ms) in enumerate(self.zener):
                    rxn = (rxx[l] + (ddx + ddy) * php - rxx[l] * hp) * mp
                    ryn = (ryy[l] + 0.5 * (ddx - ddy) * phs - ryy[l] * hs) * ms
                    srxx = srxx + rxx[l] + rxn
                    sryy = sryy + ryy[l] + ryn
                    rxx[l] = torch.where(self.m_n, rxn, rxx[l])
                    ryy[l] = torch.where(self.m_n, ryn, ryy[l])
                ux = ux + 0.5 * lpm * srxx + mu_n * sryy
                uy = uy + 0.5 * lpm * srxx - mu_n * sryy
            sxx = torch.where(self.m_n, sxx + ux * dt, sxx)
            syy = torch.where(self.m_n, syy + uy * dt, syy)
            dvy_dx = self._d(vy, 0, 0, -1, self.dx)
            dvx_dy = self._d(vx, 1, 1, 0, self.dy)
            dvy_dx, psi[2] = self._cpml(dvy_dx, psi[2], self.cx, self.m_s)
            dvx_dy, psi[3] = self._cpml(dvx_dy, psi[3], self.cyh, self.m_s)
            e = dvy_dx + dvx_dy
            us = mu_s * e
            if L:
                sr = z()
                for l, (php, phs, hp, hs, mp, ms) in enumerate(self.zener):
                    rn = (rxy[l] + e * phs - rxy[l] * hs) * ms
                    sr = sr + rxy[l] + rn
                    rxy[l] = torch.where(self.m_s, rn, rxy[l])
                us = us + 0.5 * mu_s * sr
            sxy = torch.where(self.m_s, sxy + us * dt, sxy)
            # ---- velocity_kernel ----
            dsxx = self._d(sxx, 0, 0, -1, self.dx)
            dsxy = self._d(sxy, 1, 0, -1, self.dy)
            dsxx, psi[4] = self._cpml(dsxx, psi[4], self.cx, self.m_vx)
            dsxy, psi[5] = self._cpml(dsxy, psi[5], self.cy, self.m_vx)
            vx = torch.where(upd_vx, vx + (dsxx + dsxy) * dt * inv_rho, vx)
            dsxy_dx = self._d(sxy, 0, 1, 0, self.dx)
            dsyy = self._d(syy, 1, 1, 0, self.dy)
            dsxy_dx, psi[6] = self._cpml(dsxy_dx, psi[6], self.cxh, self.m_vy)
            dsyy, psi[7] = self._cpml(dsyy, psi[7], self.cyh, self.m_vy)
            vy = torch.where(upd_vy, vy + (dsxy_dx + dsyy) * dt * inv_rho4, vy)
            vx = torch.where(self.m_vy, vx, torch.zeros_like(vx))
            vy = torch.where(self.m_vy, vy, torch.zeros_like(vy))
            if len(self.src_nodes):
                flat = it * self.n_src_el + self.src_idx
                ok = src_ok & (it < self.n_steps) & (flat < self.src_flat.numel())
                val = torch.where(ok, self.src_flat[torch.where(ok, flat, torch.zeros_like(flat))],
                                  torch.zeros_like(src_scale))
                vy = vy.reshape(-1).index_add(0, self.src_nodes, val * src_scale).reshape(self.nx, self.ny)
            # ---- store_sensors_kernel ----
            tr = torch.zeros(self.n_rec, dtype=self.dtype, device=self.device)
            if len(self.rec_cells):
                tr = tr.index_add(0, self.rec_ids, syy.reshape(-1)[self.rec_cells])
            out.append(torch.where(it >= self.delay, tr, torch.zeros_like(tr)))
        return torch.stack(out)
