"""FP64 CPU reference for the adjoint of the converged SSA solve (test infrastructure only).

The reference has no adjoint; this module differentiates the discrete fixed point that its
solve_SSA converges to (ice_dynamics_module.f90:408-694, restated in ufe_oracle_solve.c), by
assembling the Jacobian explicitly with scipy and solving with a direct sparse solver. It is
the checker of the GPU VJP and is itself checked against central finite differences of the
oracle's forward solve.

The discrete system at convergence, per AaAc row i (0-based here):

* interior rows (non-edge; what the SOR sweeps), with eta_i = eta(eps2_i(u)) (Glen, n = 3,
  SSA_effective_viscosity 695-726) and the friction factor fr_i = S_i / (max(0.1, H_i) eta_i)
  on grounded rows (is_floating, general_ice_model_data_module.f90:464-475):
      F_x,i = sum_c Cu_ic U_c + 3 sNxy_i V_i + (h_cu_i - fr_i) U_i - rho g hx_i / eta_i
      F_y,i = sum_c Cv_ic V_c + 3 sNxy_i U_i + (h_cv_i - fr_i) V_i - rho g hy_i / eta_i
  (Cu = 4 Nxx + Nyy, Cv = 4 Nyy + Nxx; the cross term uses the home value in every term,
  get_mesh_curvatures_vertex_AaAc, mesh_ArakawaC_module.f90:636-658);
* edge rows: u_e - mean(u over the non-edge neighbours) = 0; corners 1..4: u_c - mean(u over
  all neighbours) = 0 (apply_Neumann_boundary_AaAc, mesh_ArakawaC_module.f90:660-724).

Sliding: linear (S = beta^2, the library's extension) or the reference's Coulomb_regularised
law (SSA_sliding_term, ice_dynamics_module.f90:727-779), S = tau_c (dv^2 + U^2 + V^2)^e / u_t^q
with e = (q - 1)/2, q = 0.3, dv = 1e-3, u_t = 100, which depends on the row's own velocity: its
derivative adds a 2x2 block per grounded interior row, d(fr U)/dU = fr + 2 e fr U^2 / w,
d(fr U)/dV = 2 e fr U V / w (w = dv^2 + U^2 + V^2), and likewise for V. tau_c (basal_yield_stress,
780-844) is proportional to max(0.1, Hi), as is the denominator of fr, so under the Coulomb law the
friction term does not depend on the thickness.

Parameters: log(beta^2) on AaAc (linear sliding S = beta^2), and the ice thickness Hi on Aa,
which enters through Hi_AaAc (Aa rows and the Ac average, map_Aa_to_Ac) and the driving-
stress slopes hx, hy (get_mesh_derivatives on Aa, mesh_derivatives_module.f90:315-371,
get_mesh_derivatives_Ac, mesh_ArakawaC_module.f90:542-581, the shelf rule of
update_general_ice_model_data, general_ice_model_data_module.f90:70-87), with the masks
frozen. Misfit J = 1/2 sum over AaAc of (u - u_obs)^2 + (v - v_obs)^2.
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

RHO_I = 910.0
RHO_SW = 1028.0
GRAV = 9.81
N_FLOW = 3.0
EPS_SQ0 = 1e-12
Q_PLASTIC = 0.30
DELTA_V = 1e-3
U_THRESHOLD = 100.0


def _rows(m):
    """CSR-like neighbour structure of the AaAc mesh (0-based): (rows, cols, slot) of every
    neighbour entry, plus the home slot index per row."""
    nA = m.nVAaAc
    n = np.asarray(m.nCAaAc, dtype=np.int64)
    CA = np.asarray(m.CAaAc, dtype=np.int64) - 1
    ncm = CA.shape[1]
    slot = np.arange(ncm)[None, :]
    valid = slot < n[:, None]
    r = np.repeat(np.arange(nA), ncm).reshape(nA, ncm)[valid]
    c = CA[valid]
    k = np.broadcast_to(slot, (nA, ncm))[valid]
    return r, c, k, n


def is_edge_aaac(m):
    return np.concatenate([np.asarray(m.base.edge_index) > 0, np.asarray(m.edge_index_Ac) > 0])


def gather_fields(m, f):
    """AaAc gather of the solve inputs (ice_dynamics_module.f90:478-495)."""
    cat = lambda a, b: np.concatenate([np.asarray(f[a], dtype=np.float64), np.asarray(f[b], dtype=np.float64)])
    g = dict(Hi=cat("Hi", "Hi_Ac"), Hb=cat("Hb", "Hb_Ac"), SL=cat("SL", "SL_Ac"),
             hx=cat("dHs_dx_shelf", "dHs_dx_shelf_Ac"), hy=cat("dHs_dy_shelf", "dHs_dy_shelf_Ac"),
             Af=cat("A_flow_mean", "A_flow_mean_Ac"))
    beta = f.get("beta_sq_AaAc")
    g["beta"] = np.asarray(beta, dtype=np.float64) if beta is not None else np.full(m.nVAaAc, f.get("beta_sq_const", 1e3))
    return g


def derivative_ops(m):
    """Sparse d/dx and d/dy on AaAc (get_mesh_derivatives_AaAc, mesh_ArakawaC_module.f90:583-618)."""
    nA = m.nVAaAc
    r, c, k, n = _rows(m)
    Nx, Ny = np.asarray(m.Nx_AaAc), np.asarray(m.Ny_AaAc)
    home = np.arange(nA)
    rr = np.concatenate([r, home])
    cc = np.concatenate([c, home])
    Dx = sp.csr_matrix((np.concatenate([Nx[r, k], Nx[home, n]]), (rr, cc)), shape=(nA, nA))
    Dy = sp.csr_matrix((np.concatenate([Ny[r, k], Ny[home, n]]), (rr, cc)), shape=(nA, nA))
    return Dx, Dy


class Linearisation:
    """Everything the Jacobian needs at one velocity state (U, V on AaAc)."""

    def __init__(self, m, f, U, V, m_enh=1.0, tau_c=None):
        """tau_c (AaAc, the solve's basal yield stress) selects the Coulomb_regularised law;
        without it the sliding is linear with f's beta^2."""
        self.m = m
        self.tau_c = None if tau_c is None else np.asarray(tau_c, dtype=np.float64)
        nA = m.nVAaAc
        self.nA = nA
        self.g = gather_fields(m, f)
        self.U, self.V = np.asarray(U, dtype=np.float64), np.asarray(V, dtype=np.float64)
        self.edge = is_edge_aaac(m)
        self.corner = np.zeros(nA, dtype=bool)
        self.corner[:4] = True
        self.Dx, self.Dy = derivative_ops(m)
        r, c, k, n = _rows(m)
        self.r, self.c, self.k, self.n = r, c, k, n
        Nxx, Nyy, Nxy = np.asarray(m.Nxx_AaAc), np.asarray(m.Nyy_AaAc), np.asarray(m.Nxy_AaAc)
        home = np.arange(nA)
        self.Cu = 4.0 * Nxx[r, k] + Nyy[r, k]
        self.Cv = 4.0 * Nyy[r, k] + Nxx[r, k]
        self.hcu = 4.0 * Nxx[home, n] + Nyy[home, n]
        self.hcv = 4.0 * Nyy[home, n] + Nxx[home, n]
        self.sNxy = Nxy[home, n] + np.bincount(r, weights=Nxy[r, k], minlength=nA)
        g = self.g
        self.floating = g["Hi"] < ((g["SL"] - g["Hb"]) * RHO_SW) / RHO_I
        self.mH = np.maximum(0.1, g["Hi"])
        self.B = (m_enh * 0.5 * g["Af"]) ** (-1.0 / N_FLOW)
        self.p = (1.0 - N_FLOW) / (2.0 * N_FLOW)
        self.update(self.U, self.V)

    def update(self, U, V):
        self.U, self.V = U, V
        ux, uy = self.Dx @ U, self.Dy @ U
        vx, vy = self.Dx @ V, self.Dy @ V
        t = uy + vx
        self.eps2 = ux * ux + vy * vy + ux * vy + 0.25 * t * t + EPS_SQ0
        self.eta = self.B * self.eps2 ** self.p
        self.K1, self.K2, self.K3 = 2 * ux + vy, 0.5 * t, 2 * vy + ux
        if self.tau_c is None:
            S = self.g["beta"]
        else:
            self.w = DELTA_V ** 2 + U * U + V * V
            S = self.tau_c * self.w ** (0.5 * (Q_PLASTIC - 1.0)) / U_THRESHOLD ** Q_PLASTIC
        self.fr = np.where(self.floating, 0.0, S / (self.mH * self.eta))

    def residual(self):
        """F(u) on every row (interior momentum rows, boundary averaging rows)."""
        nA = self.nA
        U, V = self.U, self.V
        r, c = self.r, self.c
        sU = np.bincount(r, weights=self.Cu * U[c], minlength=nA)
        sV = np.bincount(r, weights=self.Cv * V[c], minlength=nA)
        Fx = sU + 3 * self.sNxy * V + (self.hcu - self.fr) * U - RHO_I * GRAV * self.g["hx"] / self.eta
        Fy = sV + 3 * self.sNxy * U + (self.hcv - self.fr) * V - RHO_I * GRAV * self.g["hy"] / self.eta
        Bm = self.boundary_matrix()
        bx, by = U - Bm @ U, V - Bm @ V
        Fx = np.where(self.edge, bx, Fx)
        Fy = np.where(self.edge, by, Fy)
        return np.concatenate([Fx, Fy])

    def boundary_matrix(self):
        """Averaging operator of the Neumann rows: edge rows over non-edge neighbours,
        corners over all neighbours."""
        r, c = self.r, self.c
        use = self.edge[r] & (self.corner[r] | ~self.edge[c])
        cnt = np.bincount(r[use], minlength=self.nA).astype(np.float64)
        w = 1.0 / cnt[r[use]]
        return sp.csr_matrix((w, (r[use], c[use])), shape=(self.nA, self.nA))

    def jacobian(self):
        """dF/du as a (2 nA, 2 nA) sparse matrix, unknowns ordered (U, V)."""
        nA = self.nA
        r, c, k = self.r, self.c, self.k
        U, V = self.U, self.V
        g = self.g
        interior = ~self.edge
        rg = RHO_I * GRAV
        # dF/deta on interior rows
        dFx_deta = (self.fr * U + rg * g["hx"] / self.eta) / self.eta
        dFy_deta = (self.fr * V + rg * g["hy"] / self.eta) / self.eta
        ax = dFx_deta * self.eta * self.p / self.eps2
        ay = dFy_deta * self.eta * self.p / self.eps2
        # d(eps2)/du_c coefficients, entries and home
        Nx, Ny = np.asarray(self.m.Nx_AaAc), np.asarray(self.m.Ny_AaAc)
        home = np.arange(nA)
        nxe, nye = Nx[r, k], Ny[r, k]
        nxh, nyh = Nx[home, self.n], Ny[home, self.n]
        kU_e = self.K1[r] * nxe + self.K2[r] * nye
        kV_e = self.K2[r] * nxe + self.K3[r] * nye
        kU_h = self.K1 * nxh + self.K2 * nyh
        kV_h = self.K2 * nxh + self.K3 * nyh
        ie = interior[r]
        rows, cols, vals = [], [], []

        def add(R, C, X):
            rows.append(R); cols.append(C); vals.append(X)
        # interior momentum rows: neighbours
        add(r[ie], c[ie], self.Cu[ie] + ax[r[ie]] * kU_e[ie])            # Fx / dU_c
        add(r[ie], nA + c[ie], ax[r[ie]] * kV_e[ie])                     # Fx / dV_c
        add(nA + r[ie], c[ie], ay[r[ie]] * kU_e[ie])                     # Fy / dU_c
        add(nA + r[ie], nA + c[ie], self.Cv[ie] + ay[r[ie]] * kV_e[ie])  # Fy / dV_c
        hi = home[interior]
        add(hi, hi, self.hcu[hi] - self.fr[hi] + ax[hi] * kU_h[hi])
        add(hi, nA + hi, 3 * self.sNxy[hi] + ax[hi] * kV_h[hi])
        add(nA + hi, hi, 3 * self.sNxy[hi] + ay[hi] * kU_h[hi])
        add(nA + hi, nA + hi, self.hcv[hi] - self.fr[hi] + ay[hi] * kV_h[hi])
        if self.tau_c is not None:
            # the Coulomb law's S'(u): local to the row
            cS = (Q_PLASTIC - 1.0) * self.fr[hi] / self.w[hi]
            Uh, Vh = U[hi], V[hi]
            add(hi, hi, -cS * Uh * Uh)
            add(hi, nA + hi, -cS * Uh * Vh)
            add(nA + hi, hi, -cS * Uh * Vh)
            add(nA + hi, nA + hi, -cS * Vh * Vh)
        # boundary rows
        Bm = self.boundary_matrix().tocoo()
        be = home[self.edge]
        add(be, be, np.ones(be.size))
        add(nA + be, nA + be, np.ones(be.size))
        add(Bm.row, Bm.col, -Bm.data)
        add(nA + Bm.row, nA + Bm.col, -Bm.data)
        R = np.concatenate(rows); C = np.concatenate(cols); X = np.concatenate(vals)
        return sp.csr_matrix((X, (R, C)), shape=(2 * nA, 2 * nA))

    # ------------------------------------------------------------ parameter derivatives
    def dF_dlogbeta(self):
        """dF/d(log S0) (diagonal per row): -fr U on interior grounded rows, where S0 is the
        law's coefficient field, S proportional to it: beta^2 (linear) or tau_c (Coulomb)."""
        interior = ~self.edge
        return np.where(interior, -self.fr * self.U, 0.0), np.where(interior, -self.fr * self.V, 0.0)

    def dF_dfields(self):
        """dF/d(hx), dF/d(hy), dF/d(Hi_AaAc) (diagonal per row)."""
        interior = ~self.edge
        rg = RHO_I * GRAV
        dhx = np.where(interior, -rg / self.eta, 0.0)
        dH = np.where(interior & (self.g["Hi"] > 0.1), self.fr / self.mH, 0.0)   # d(-fr u)/dH = fr u / H
        if self.tau_c is not None:
            dH = np.zeros_like(dH)     # tau_c / max(0.1, H) does not depend on H
        return dhx, dH * self.U, dH * self.V


def geometry_matrix(m, Hi, Hb, SL):
    """Linear map dHi (Aa, nV) -> (d hx, d hy, d Hi_AaAc) on AaAc rows, masks frozen."""
    base = m.base
    nV, nAc = base.nV, m.nAc
    nA = nV + nAc
    rr = RHO_I / RHO_SW
    Hi, Hb, SL = (np.asarray(a, dtype=np.float64) for a in (Hi, Hb, SL))
    ocean = Hi < ((SL - Hb) * RHO_SW) / RHO_I
    slope = np.where(ocean, 1.0 - rr, 1.0)           # dHs/dHi per Aa vertex
    Aci = np.asarray(m.Aci, dtype=np.int64) - 1
    vi, vj = Aci[:, 0], Aci[:, 1]
    Hi_Ac = (Hi[vi] + Hi[vj]) / 2.0
    Hb_Ac = (Hb[vi] + Hb[vj]) / 2.0
    SL_Ac = (SL[vi] + SL[vj]) / 2.0
    ocean_Ac = Hi_Ac < ((SL_Ac - Hb_Ac) * RHO_SW) / RHO_I
    # Aa rows: Aa neighbour functions (home in column nC)
    nC = np.asarray(base.nC, dtype=np.int64)
    C = np.asarray(base.C, dtype=np.int64) - 1
    Nx, Ny = np.asarray(m.Nx), np.asarray(m.Ny)
    ncm = C.shape[1]
    slot = np.arange(ncm)[None, :]
    valid = slot < nC[:, None]
    rA = np.repeat(np.arange(nV), ncm).reshape(nV, ncm)[valid]
    kA = np.broadcast_to(slot, (nV, ncm))[valid]
    cA = C[valid]
    rows = np.concatenate([rA, np.arange(nV)])
    cols = np.concatenate([cA, np.arange(nV)])
    wx = np.concatenate([Nx[rA, kA], Nx[np.arange(nV), nC]])
    wy = np.concatenate([Ny[rA, kA], Ny[np.arange(nV), nC]])
    fac = np.where(ocean[rows], 1.0 - rr, slope[cols])
    Gx_aa = sp.csr_matrix((wx * fac, (rows, cols)), shape=(nV, nV))
    Gy_aa = sp.csr_matrix((wy * fac, (rows, cols)), shape=(nV, nV))
    # Ac rows: 4-point stencil
    Nx_Ac, Ny_Ac = np.asarray(m.Nx_Ac), np.asarray(m.Ny_Ac)
    ra = np.repeat(np.arange(nAc), 4)
    ca = Aci.reshape(-1)
    facA = np.where(ocean_Ac[ra], 1.0 - rr, slope[ca])
    Gx_ac = sp.csr_matrix((Nx_Ac.reshape(-1) * facA, (ra, ca)), shape=(nAc, nV))
    Gy_ac = sp.csr_matrix((Ny_Ac.reshape(-1) * facA, (ra, ca)), shape=(nAc, nV))
    GH_ac = sp.csr_matrix((np.full(2 * nAc, 0.5), (np.repeat(np.arange(nAc), 2), np.stack([vi, vj], 1).reshape(-1))),
                          shape=(nAc, nV))
    Gx = sp.vstack([Gx_aa, Gx_ac]).tocsr()
    Gy = sp.vstack([Gy_aa, Gy_ac]).tocsr()
    GH = sp.vstack([sp.identity(nV, format="csr"), GH_ac]).tocsr()
    return Gx, Gy, GH


def dlogtau_dHb(Hb, SL, Hi=None):
    """d log(tau_c) / d Hb per row of basal_yield_stress (ice_dynamics_module.f90:780-844):
    tau_c = tan(phi pi / 180) rho g max(0.1, Hi) (1 - 0.96 lambda_p), with
    phi = clamp(5 + 15 (1 + Hb / 1000), 5, 20) and lambda_p = clamp(1 - (Hb - SL) / 1000, 0, 1);
    a clamped branch contributes nothing."""
    Hb = np.asarray(Hb, dtype=np.float64)
    SL = np.asarray(SL, dtype=np.float64)
    phi_raw = 5.0 + 15.0 * (1.0 + Hb / 1000.0)
    phi = np.clip(phi_raw, 5.0, 20.0)
    dphi = np.where((phi_raw > 5.0) & (phi_raw < 20.0), 15.0 / 1000.0, 0.0)
    lam_raw = 1.0 - (Hb - SL) / 1000.0
    lam = np.clip(lam_raw, 0.0, 1.0)
    dlam = np.where((lam_raw > 0.0) & (lam_raw < 1.0), -1.0 / 1000.0, 0.0)
    r = np.pi / 180.0
    return r * dphi / (np.sin(r * phi) * np.cos(r * phi)) + (-0.96 * dlam) / (1.0 - 0.96 * lam)


def bed_matrix(m, Hi, Hb, SL):
    """Linear map dHb (Aa, nV) -> (d hx, d hy, d Hb_AaAc) on AaAc rows, masks frozen: the
    surface Hs = Hi + max(SL - rho_i/rho_sw Hi, Hb) moves with the bed on grounded vertices
    only, and floating rows take their slope from Hi (the shelf rule), not from Hs."""
    base = m.base
    nV, nAc = base.nV, m.nAc
    Hi, Hb, SL = (np.asarray(a, dtype=np.float64) for a in (Hi, Hb, SL))
    ocean = Hi < ((SL - Hb) * RHO_SW) / RHO_I
    slope = np.where(ocean, 0.0, 1.0)                # dHs/dHb per Aa vertex
    Aci = np.asarray(m.Aci, dtype=np.int64) - 1
    vi, vj = Aci[:, 0], Aci[:, 1]
    Hi_Ac, Hb_Ac, SL_Ac = (Hi[vi] + Hi[vj]) / 2.0, (Hb[vi] + Hb[vj]) / 2.0, (SL[vi] + SL[vj]) / 2.0
    ocean_Ac = Hi_Ac < ((SL_Ac - Hb_Ac) * RHO_SW) / RHO_I
    nC = np.asarray(base.nC, dtype=np.int64)
    C = np.asarray(base.C, dtype=np.int64) - 1
    Nx, Ny = np.asarray(m.Nx), np.asarray(m.Ny)
    ncm = C.shape[1]
    slot = np.arange(ncm)[None, :]
    valid = slot < nC[:, None]
    rA = np.repeat(np.arange(nV), ncm).reshape(nV, ncm)[valid]
    kA = np.broadcast_to(slot, (nV, ncm))[valid]
    cA = C[valid]
    rows = np.concatenate([rA, np.arange(nV)])
    cols = np.concatenate([cA, np.arange(nV)])
    wx = np.concatenate([Nx[rA, kA], Nx[np.arange(nV), nC]])
    wy = np.concatenate([Ny[rA, kA], Ny[np.arange(nV), nC]])
    fac = np.where(ocean[rows], 0.0, slope[cols])
    Gx_aa = sp.csr_matrix((wx * fac, (rows, cols)), shape=(nV, nV))
    Gy_aa = sp.csr_matrix((wy * fac, (rows, cols)), shape=(nV, nV))
    Nx_Ac, Ny_Ac = np.asarray(m.Nx_Ac), np.asarray(m.Ny_Ac)
    ra = np.repeat(np.arange(nAc), 4)
    ca = Aci.reshape(-1)
    facA = np.where(ocean_Ac[ra], 0.0, slope[ca])
    Gx_ac = sp.csr_matrix((Nx_Ac.reshape(-1) * facA, (ra, ca)), shape=(nAc, nV))
    Gy_ac = sp.csr_matrix((Ny_Ac.reshape(-1) * facA, (ra, ca)), shape=(nAc, nV))
    GB_ac = sp.csr_matrix((np.full(2 * nAc, 0.5), (np.repeat(np.arange(nAc), 2), np.stack([vi, vj], 1).reshape(-1))),
                          shape=(nAc, nV))
    return (sp.vstack([Gx_aa, Gx_ac]).tocsr(), sp.vstack([Gy_aa, Gy_ac]).tocsr(),
            sp.vstack([sp.identity(nV, format="csr"), GB_ac]).tocsr())


def coulomb_bed_gradient(m, f, d_logtau, s_hx, s_hy):
    """dJ/dHb on Aa under the Coulomb law from the adjoint's dJ/dlog(tau_c) and driving-stress
    sensitivities (AaAc rows): through tau_c's bed dependence and through the surface slope."""
    g = gather_fields(m, f)
    Gx, Gy, GB = bed_matrix(m, f["Hi"], f["Hb"], f["SL"])
    return GB.T @ (np.asarray(d_logtau) * dlogtau_dHb(g["Hb"], g["SL"])) + Gx.T @ s_hx + Gy.T @ s_hy


def adjoint_gradient(lin: Linearisation, gU, gV, G=None):
    """Solve (dF/du)^T mu = dJ/du and return (mu_U, mu_V, dJ/dlog(beta^2) (dJ/dlog(tau_c)
    under the Coulomb law), dJ/dHi or None, field sensitivities dict)."""
    nA = lin.nA
    K = lin.jacobian()
    mu = spla.spsolve(K.T.tocsc(), np.concatenate([gU, gV]))
    mx, my = mu[:nA], mu[nA:]
    bx, by = lin.dF_dlogbeta()        # log(beta^2) (linear law) or log(tau_c) (Coulomb law)
    d_logbeta = -(mx * bx + my * by)
    dhx, dHx, dHy = lin.dF_dfields()
    s_hx = -mx * dhx
    s_hy = -my * dhx
    s_H = -(mx * dHx + my * dHy)
    dHi = None
    if G is not None:
        Gx, Gy, GH = G
        dHi = Gx.T @ s_hx + Gy.T @ s_hy + GH.T @ s_H
    return mx, my, d_logbeta, dHi, dict(hx=s_hx, hy=s_hy, Hi=s_H)


def tangent_linear(lin: Linearisation, d_logbeta=None, d_Hi=None, G=None):
    """du for a parameter perturbation: solve (dF/du) du = -(dF/dp) dp."""
    nA = lin.nA
    rhs = np.zeros(2 * nA)
    if d_logbeta is not None:
        bx, by = lin.dF_dlogbeta()
        rhs[:nA] -= bx * d_logbeta
        rhs[nA:] -= by * d_logbeta
    if d_Hi is not None:
        Gx, Gy, GH = G
        dhx, dHx, dHy = lin.dF_dfields()
        rhs[:nA] -= dhx * (Gx @ d_Hi) + dHx * (GH @ d_Hi)
        rhs[nA:] -= dhx * (Gy @ d_Hi) + dHy * (GH @ d_Hi)
    du = spla.spsolve(lin.jacobian().tocsc(), rhs)
    return du[:nA], du[nA:]


def aaac_velocity(out):
    """U, V on AaAc from a solve's outputs (Aa then Ac)."""
    return (np.concatenate([out["U_SSA"], out["Ux_SSA_Ac"]]), np.concatenate([out["V_SSA"], out["Uy_SSA_Ac"]]))


def misfit(U, V, Uo, Vo):
    return 0.5 * float(np.sum((U - Uo) ** 2 + (V - Vo) ** 2))
