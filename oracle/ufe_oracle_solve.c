/*
 * CPU oracle, solver part -- TEST INFRASTRUCTURE ONLY (see ufe_oracle.h).
 *
 * Literal FP64 restatements of
 *   ice_dynamics_module.f90:240-314   solve_SIA
 *   ice_dynamics_module.f90:408-557   solve_SSA
 *   ice_dynamics_module.f90:558-694   solve_SSA_linearised
 *   ice_dynamics_module.f90:695-726   SSA_effective_viscosity
 *   ice_dynamics_module.f90:727-779   SSA_sliding_term (+ the linear law S = beta^2)
 *   ice_dynamics_module.f90:780-844   basal_yield_stress
 *   ice_dynamics_module.f90:848-949   calculate_GL_flux (Coulomb_regularised / Tsai et al.)
 *   mesh_ArakawaC_module.f90:583-618  get_mesh_derivatives_AaAc
 *   mesh_ArakawaC_module.f90:636-658  get_mesh_curvatures_vertex_AaAc (home value d(ai) in
 *                                     every neighbour term, as coded)
 *   mesh_ArakawaC_module.f90:660-724  apply_Neumann_boundary_AaAc
 *   mesh_ArakawaC_module.f90:726-791  map_Aa_to_Ac / map_Ac_to_Aa
 *   mesh_ArakawaC_module.f90:815-844  rotate_xy_to_po
 *   mesh_ArakawaC_module.f90:542-581  get_mesh_derivatives_Ac
 *   mesh_derivatives_module.f90:315-371 get_mesh_derivatives (Aa)
 *   zeta_module.f90:33-85             vertical_average / vertical_integrate
 *   general_ice_model_data_module.f90:23-96, 97-297, 464-475  (geometry part)
 * Constants: parameters_module.f90:9-21. n_flow = 3 is a PARAMETER in the reference.
 */
#include "ufe_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define A1(p, i) ((p)[(size_t)(i) - 1])
#define A2(p, ld, i, j) ((p)[(size_t)((i) - 1) + (size_t)((j) - 1) * (size_t)(ld)])

static const double pi = 3.141592653589793;
static const double grav = 9.81;
static const double n_flow = 3.0;
static const double ice_density = 910.0;
static const double seawater_density = 1028.0;

static inline double fmax_f(double a, double b) { return a > b ? a : b; } /* Fortran MAX */
static inline double fmin_f(double a, double b) { return a < b ? a : b; } /* Fortran MIN */

/* gfortran's inline NORM2: the scaled one-pass sum of squares. */
static double norm2_2(double a, double b) {
  double scale = 0.0, ssq = 1.0, v[2] = {a, b};
  for (int i = 0; i < 2; i++) {
    if (v[i] != 0.0) {
      const double absx = fabs(v[i]);
      if (scale < absx) {
        const double r = scale / absx;
        ssq = 1.0 + (ssq * r) * r;
        scale = absx;
      } else {
        const double r = absx / scale;
        ssq = ssq + r * r;
      }
    }
  }
  return scale * sqrt(ssq);
}

static int is_floating(double Hi, double Hb, double SL) {
  return Hi < ((SL - Hb) * seawater_density) / ice_density;
}

void or_map_Aa_to_Ac(const or_aaac *m, int nV, const double *d_Aa, double *d_Ac) {
  (void)nV;
  for (int aci = 1; aci <= m->nAc; aci++) {
    const int vi = A2(m->Aci, m->nAc, aci, 1), vj = A2(m->Aci, m->nAc, aci, 2);
    A1(d_Ac, aci) = (A1(d_Aa, vi) + A1(d_Aa, vj)) / 2.0;
  }
}

void or_map_Ac_to_Aa(const or_base *b, const or_aaac *m, const double *d_Ac, double *d_Aa) {
  const int nV = b->nV;
  for (int vi = 1; vi <= nV; vi++) A1(d_Aa, vi) = 0.0;
  for (int vi = 1; vi <= nV; vi++) {
    for (int ci = 1; ci <= A1(b->nC, vi); ci++) {
      const int aci = A2(m->iAci, nV, vi, ci);
      A1(d_Aa, vi) = A1(d_Aa, vi) + A1(d_Ac, aci) / (double)A1(b->nC, vi);
    }
  }
}

/* get_mesh_derivatives (Aa), mesh_derivatives_module.f90:315-371 */
static void ddx_ddy_Aa(const or_base *b, const or_aaac *m, const double *d, double *ddx, double *ddy) {
  const int nV = b->nV;
  for (int vi = 1; vi <= nV; vi++) {
    const int n = A1(b->nC, vi);
    double dx = A2(m->Nx, nV, vi, n + 1) * A1(d, vi);
    double dy = A2(m->Ny, nV, vi, n + 1) * A1(d, vi);
    for (int ci = 1; ci <= n; ci++) {
      dx = dx + A2(m->Nx, nV, vi, ci) * A1(d, A2(b->C, nV, vi, ci));
      dy = dy + A2(m->Ny, nV, vi, ci) * A1(d, A2(b->C, nV, vi, ci));
    }
    A1(ddx, vi) = dx;
    A1(ddy, vi) = dy;
  }
}

/* get_mesh_derivatives_Ac, mesh_ArakawaC_module.f90:542-581 */
static void derivs_Ac(const or_aaac *m, const double *d_Aa, double *ddx, double *ddy, double *ddp,
                      double *ddo) {
  const int nAc = m->nAc;
  for (int aci = 1; aci <= nAc; aci++) {
    double dx = 0.0, dy = 0.0, dp = 0.0, d_o = 0.0;
    for (int n = 1; n <= 4; n++) {
      const double dv = A1(d_Aa, A2(m->Aci, nAc, aci, n));
      dx = dx + A2(m->Nx_Ac, nAc, aci, n) * dv;
      dy = dy + A2(m->Ny_Ac, nAc, aci, n) * dv;
      d_o = d_o + A2(m->No_Ac, nAc, aci, n) * dv;
    }
    dp = A1(m->Np_Ac, aci) * (A1(d_Aa, A2(m->Aci, nAc, aci, 2)) - A1(d_Aa, A2(m->Aci, nAc, aci, 1)));
    A1(ddx, aci) = dx; A1(ddy, aci) = dy; A1(ddp, aci) = dp; A1(ddo, aci) = d_o;
  }
}

int or_update_geometry(const or_base *b, const or_aaac *m, or_geom *g) {
  const int nV = b->nV, nAc = m->nAc;
  const double rr = ice_density / seawater_density;
  or_map_Aa_to_Ac(m, nV, g->Hi, g->Hi_Ac);
  or_map_Aa_to_Ac(m, nV, g->Hb, g->Hb_Ac);
  or_map_Aa_to_Ac(m, nV, g->SL, g->SL_Ac);
  for (int vi = 1; vi <= nV; vi++)
    A1(g->Hs, vi) = A1(g->Hi, vi) + fmax_f(A1(g->SL, vi) - rr * A1(g->Hi, vi), A1(g->Hb, vi));
  for (int aci = 1; aci <= nAc; aci++)
    A1(g->Hs_Ac, aci) = A1(g->Hi_Ac, aci) + fmax_f(A1(g->SL_Ac, aci) - rr * A1(g->Hi_Ac, aci), A1(g->Hb_Ac, aci));
  /* determine_masks: ocean / ice / sheet / shelf on Aa and Ac, grounding line on Ac */
  for (int vi = 1; vi <= nV; vi++) {
    const int ocean = is_floating(A1(g->Hi, vi), A1(g->Hb, vi), A1(g->SL, vi));
    const int ice = A1(g->Hi, vi) > 0.0;
    A1(g->mask_ocean, vi) = ocean;
    A1(g->mask_ice, vi) = ice;
    A1(g->mask_sheet, vi) = ice && !ocean;
    A1(g->mask_shelf, vi) = ice && ocean;
  }
  for (int aci = 1; aci <= nAc; aci++) {
    const int ocean = is_floating(A1(g->Hi_Ac, aci), A1(g->Hb_Ac, aci), A1(g->SL_Ac, aci));
    const int ice = A1(g->Hi_Ac, aci) > 0.0;
    A1(g->mask_ocean_Ac, aci) = ocean;
    A1(g->mask_ice_Ac, aci) = ice;
    A1(g->mask_sheet_Ac, aci) = ice && !ocean;
    A1(g->mask_shelf_Ac, aci) = ice && ocean;
    const int vi = A2(m->Aci, nAc, aci, 1), vj = A2(m->Aci, nAc, aci, 2);
    A1(g->mask_gl_Ac, aci) = (A1(g->mask_sheet, vi) == 1 && A1(g->mask_shelf, vj) == 1) ||
                             (A1(g->mask_sheet, vj) == 1 && A1(g->mask_shelf, vi) == 1);
  }
  ddx_ddy_Aa(b, m, g->Hi, g->dHi_dx, g->dHi_dy);
  ddx_ddy_Aa(b, m, g->Hs, g->dHs_dx, g->dHs_dy);
  derivs_Ac(m, g->Hi, g->dHi_dx_Ac, g->dHi_dy_Ac, g->dHi_dp_Ac, g->dHi_do_Ac);
  derivs_Ac(m, g->Hb, g->dHb_dx_Ac, g->dHb_dy_Ac, g->dHb_dp_Ac, g->dHb_do_Ac);
  derivs_Ac(m, g->Hs, g->dHs_dx_Ac, g->dHs_dy_Ac, g->dHs_dp_Ac, g->dHs_do_Ac);
  derivs_Ac(m, g->SL, g->dSL_dx_Ac, g->dSL_dy_Ac, g->dSL_dp_Ac, g->dSL_do_Ac);
  for (int vi = 1; vi <= nV; vi++) {
    if (A1(g->mask_ocean, vi) == 0) {
      A1(g->dHs_dx_shelf, vi) = A1(g->dHs_dx, vi);
      A1(g->dHs_dy_shelf, vi) = A1(g->dHs_dy, vi);
    } else {
      A1(g->dHs_dx_shelf, vi) = (1.0 - rr) * A1(g->dHi_dx, vi);
      A1(g->dHs_dy_shelf, vi) = (1.0 - rr) * A1(g->dHi_dy, vi);
    }
  }
  for (int aci = 1; aci <= nAc; aci++) {
    if (A1(g->mask_ocean_Ac, aci) == 0) {
      A1(g->dHs_dx_shelf_Ac, aci) = A1(g->dHs_dx_Ac, aci);
      A1(g->dHs_dy_shelf_Ac, aci) = A1(g->dHs_dy_Ac, aci);
    } else {
      A1(g->dHs_dx_shelf_Ac, aci) = (1.0 - rr) * A1(g->dHi_dx_Ac, aci);
      A1(g->dHs_dy_shelf_Ac, aci) = (1.0 - rr) * A1(g->dHi_dy_Ac, aci);
    }
  }
  return OR_OK;
}

/* ================================== SIA ================================== */

int or_solve_SIA(const or_base *b, const or_aaac *m, const or_params *p, or_sia_fields *f) {
  const int nAc = m->nAc, nZ = p->nZ;
  const double *zeta = p->zeta;
  const double D_uv_3D_cutoff = -1e5;
  double D_def[64], fz[64], prof[64];
  if (nZ < 2 || nZ > 64) return OR_ERR_BAD_ARG;
  for (int aci = 1; aci <= nAc; aci++) {
    for (int k = 1; k <= nZ; k++) A2(f->D_SIA_3D_Ac, nAc, aci, k) = 0.0;
    A1(f->D_SIA_Ac, aci) = 0.0; A1(f->Ux_SIA_Ac, aci) = 0.0; A1(f->Uy_SIA_Ac, aci) = 0.0;
    A1(f->Up_SIA_Ac, aci) = 0.0; A1(f->Uo_SIA_Ac, aci) = 0.0;
  }
  for (int aci = 1; aci <= nAc; aci++) {
    if (A1(f->mask_sheet_Ac, aci) == 1) {
      const double H = A1(f->Hi_Ac, aci);
      const double sp = A1(f->dHs_dp_Ac, aci), so = A1(f->dHs_do_Ac, aci);
      const double D_0 = pow(ice_density * grav * H, n_flow) * pow(sp * sp + so * so, (n_flow - 1.0) / 2.0);
      /* vertical_integrate( m_enh_sia * A_flow_Ac(aci,:) * zeta**n_flow ) */
      for (int k = 1; k <= nZ; k++) fz[k - 1] = (p->m_enh_sia * A2(f->A_flow_Ac, nAc, aci, k)) * pow(zeta[k - 1], n_flow);
      D_def[nZ - 1] = 0.0;
      for (int k = nZ - 1; k >= 1; k--)
        D_def[k - 1] = D_def[k] - (0.5 * (fz[k] + fz[k - 1])) * (zeta[k] - zeta[k - 1]);
      for (int k = 1; k <= nZ; k++) D_def[k - 1] = (2.0 * H) * D_def[k - 1];
      for (int k = 1; k <= nZ; k++) A2(f->D_SIA_3D_Ac, nAc, aci, k) = D_0 * D_def[k - 1];
    }
    for (int k = 1; k <= nZ; k++)
      if (A2(f->D_SIA_3D_Ac, nAc, aci, k) < D_uv_3D_cutoff) A2(f->D_SIA_3D_Ac, nAc, aci, k) = D_uv_3D_cutoff;
  }
  for (int aci = 1; aci <= nAc; aci++) {
    if (A1(f->mask_sheet_Ac, aci) == 1) {
      double D_uv_2D = 0.0;
      for (int k = 1; k <= nZ; k++) prof[k - 1] = A2(f->D_SIA_3D_Ac, nAc, aci, k);
      for (int k = 1; k <= nZ - 1; k++)
        D_uv_2D = D_uv_2D + (0.5 * (prof[k] + prof[k - 1])) * (zeta[k] - zeta[k - 1]);
      A1(f->D_SIA_Ac, aci) = A1(f->Hi_Ac, aci) * D_uv_2D;
      A1(f->Ux_SIA_Ac, aci) = D_uv_2D * A1(f->dHs_dx_Ac, aci);
      A1(f->Uy_SIA_Ac, aci) = D_uv_2D * A1(f->dHs_dy_Ac, aci);
      A1(f->Up_SIA_Ac, aci) = D_uv_2D * A1(f->dHs_dp_Ac, aci);
      A1(f->Uo_SIA_Ac, aci) = D_uv_2D * A1(f->dHs_do_Ac, aci);
    }
  }
  or_map_Ac_to_Aa(b, m, f->Ux_SIA_Ac, f->U_SIA);
  or_map_Ac_to_Aa(b, m, f->Uy_SIA_Ac, f->V_SIA);
  or_map_Ac_to_Aa(b, m, f->D_SIA_Ac, f->D_SIA);
  return OR_OK;
}

/* ================================== SSA ================================== */

/* get_mesh_derivatives_AaAc, mesh_ArakawaC_module.f90:583-618 */
void or_ddx_ddy_AaAc(const or_aaac *m, int nC_mem, const double *d, double *ddx, double *ddy) {
  const int nA = m->nVAaAc;
  (void)nC_mem;
  for (int ai = 1; ai <= nA; ai++) {
    const int n = A1(m->nCAaAc, ai);
    double dx = A2(m->Nx_AaAc, nA, ai, n + 1) * A1(d, ai);
    double dy = A2(m->Ny_AaAc, nA, ai, n + 1) * A1(d, ai);
    for (int ci = 1; ci <= n; ci++) {
      dx = dx + A2(m->Nx_AaAc, nA, ai, ci) * A1(d, A2(m->CAaAc, nA, ai, ci));
      dy = dy + A2(m->Ny_AaAc, nA, ai, ci) * A1(d, A2(m->CAaAc, nA, ai, ci));
    }
    A1(ddx, ai) = dx;
    A1(ddy, ai) = dy;
  }
}

static int is_edge_AaAc(const or_base *b, const or_aaac *m, int ai) {
  if (ai <= b->nV) return A1(b->edge_index, ai) > 0;
  return A1(m->edge_index_Ac, ai - b->nV) > 0;
}

/* apply_Neumann_boundary_AaAc, mesh_ArakawaC_module.f90:660-724 */
void or_neumann_AaAc(const or_base *b, const or_aaac *m, double *d) {
  const int nA = m->nVAaAc;
  for (int ai = 5; ai <= nA; ai++) {
    double vals[64];
    int nvals = 0;
    if (!is_edge_AaAc(b, m, ai)) continue;
    for (int ci = 1; ci <= A1(m->nCAaAc, ai); ci++) {
      const int ac = A2(m->CAaAc, nA, ai, ci);
      if (is_edge_AaAc(b, m, ac)) continue;
      nvals = nvals + 1;
      vals[nvals - 1] = A1(d, ac);
    }
    /* SUM(vals) runs over all nC_mem entries; the unused ones are +0. */
    double s = 0.0;
    for (int k = 0; k < b->nC_mem; k++) s = s + (k < nvals ? vals[k] : 0.0);
    A1(d, ai) = s / (double)nvals;
  }
  for (int ai = 1; ai <= 4; ai++) {
    double vals[64];
    int nvals = 0;
    for (int ci = 1; ci <= A1(m->nCAaAc, ai); ci++) {
      const int ac = A2(m->CAaAc, nA, ai, ci);
      nvals = nvals + 1;
      vals[nvals - 1] = A1(d, ac);
    }
    double s = 0.0;
    for (int k = 0; k < b->nC_mem; k++) s = s + (k < nvals ? vals[k] : 0.0);
    A1(d, ai) = s / (double)nvals;
  }
}

/* SOR loop of solve_SSA_linearised (ice_dynamics_module.f90:597-691), given the right-hand
 * sides and centre coefficients. Returns the number of sweeps; *did_reset as the reference;
 * n_fixed > 0 forces exactly that many sweeps (replay). */
static int sor_loop(const or_base *b, const or_aaac *m, const or_params *p,
                    const int32_t *mask_gl_Ac, const double *RHSx, const double *RHSy,
                    const double *eu, const double *ev, double *U, double *V, int *did_reset,
                    int *not_converged, double *max_res_out, int n_fixed, int64_t sweeps_before) {
  const int nA = m->nVAaAc, nV = b->nV;
  const double omega = p->SSA_SOR_omega;
  int has_converged = 0, inner_loop_i = 0;
  double max_residual_UV = 0.0;
  *did_reset = 0;
  *not_converged = 0;
  const int max_inner = n_fixed > 0 ? n_fixed : p->SSA_max_inner_loops;
  while (!has_converged && inner_loop_i < max_inner) {
    inner_loop_i = inner_loop_i + 1;
    max_residual_UV = 0.0;
    for (int fci = 1; fci <= 5; fci++) {
      const int n_c = A1(m->colour_nV, fci);
      double cmax = 0.0;
#pragma omp parallel for num_threads(p->n_threads > 0 ? p->n_threads : 1) reduction(max : cmax) schedule(static)
      for (int fcvi = 1; fcvi <= n_c; fcvi++) {
        const int ai = A2(m->colour_vi, nA, fcvi, fci);
        if (is_edge_AaAc(b, m, ai)) continue;
        if (p->use_analytical_GL_flux && ai > nV && A1(mask_gl_Ac, ai - nV) == 1) continue;
        const int n = A1(m->nCAaAc, ai);
        /* get_mesh_curvatures_vertex_AaAc for U and V (only the xy term is used) */
        const double Uai = A1(U, ai), Vai = A1(V, ai);
        double Uxyi = Uai * A2(m->Nxy_AaAc, nA, ai, n + 1);
        double Vxyi = Vai * A2(m->Nxy_AaAc, nA, ai, n + 1);
        for (int ci = 1; ci <= n; ci++) {
          Uxyi = Uxyi + Uai * A2(m->Nxy_AaAc, nA, ai, ci);
          Vxyi = Vxyi + Vai * A2(m->Nxy_AaAc, nA, ai, ci);
        }
        double sumUc = 0.0, sumVc = 0.0;
        for (int ci = 1; ci <= n; ci++) {
          const int ac = A2(m->CAaAc, nA, ai, ci);
          const double nxx = A2(m->Nxx_AaAc, nA, ai, ci), nyy = A2(m->Nyy_AaAc, nA, ai, ci);
          sumUc = sumUc + A1(U, ac) * (4.0 * nxx + nyy);
          sumVc = sumVc + A1(V, ac) * (4.0 * nyy + nxx);
        }
        const double LHSx = (sumUc + (3.0 * Vxyi)) + (A1(eu, ai) * Uai);
        const double LHSy = (sumVc + (3.0 * Uxyi)) + (A1(ev, ai) * Vai);
        const double resU = (LHSx - A1(RHSx, ai)) / A1(eu, ai);
        const double resV = (LHSy - A1(RHSy, ai)) / A1(ev, ai);
        cmax = fmax_f(cmax, fabs(resU));
        cmax = fmax_f(cmax, fabs(resV));
        A1(U, ai) = Uai - omega * resU;
        A1(V, ai) = Vai - omega * resV;
      }
      max_residual_UV = fmax_f(max_residual_UV, cmax);
    }
    or_neumann_AaAc(b, m, U);
    or_neumann_AaAc(b, m, V);
    if (p->progress) *p->progress = sweeps_before + inner_loop_i;
    if (n_fixed > 0) continue;
    if (max_residual_UV < p->SSA_max_residual_UV) {
      *did_reset = 0;
      has_converged = 1;
    } else if (max_residual_UV > 1e6) {
      for (int ai = 1; ai <= nA; ai++) { A1(U, ai) = 0.0; A1(V, ai) = 0.0; }
      *did_reset = 1;
      has_converged = 1;
    } else if (inner_loop_i == p->SSA_max_inner_loops) {
      *not_converged = 1; /* reference: WRITE(0,*) ' WARNING - SSA SOR solver doesnt converge!' */
    }
  }
  if (max_res_out) *max_res_out = max_residual_UV;
  return inner_loop_i;
}

/* RHS and centre coefficients (ice_dynamics_module.f90:580-595) */
static void rhs_and_centre(const or_aaac *m, const double *Hi, const double *Hb, const double *SL,
                           const double *hx, const double *hy, const double *eta, const double *S,
                           double *RHSx, double *RHSy, double *eu, double *ev) {
  const int nA = m->nVAaAc;
  for (int ai = 1; ai <= nA; ai++) {
    A1(RHSx, ai) = ((ice_density * grav) * A1(hx, ai)) / A1(eta, ai);
    A1(RHSy, ai) = ((ice_density * grav) * A1(hy, ai)) / A1(eta, ai);
  }
  for (int ai = 1; ai <= nA; ai++) {
    const int h = A1(m->nCAaAc, ai) + 1;
    const double nxx = A2(m->Nxx_AaAc, nA, ai, h), nyy = A2(m->Nyy_AaAc, nA, ai, h);
    if (!is_floating(A1(Hi, ai), A1(Hb, ai), A1(SL, ai))) {
      A1(eu, ai) = (4.0 * nxx + nyy) - A1(S, ai) / (fmax_f(0.1, A1(Hi, ai)) * A1(eta, ai));
      A1(ev, ai) = (4.0 * nyy + nxx) - A1(S, ai) / (fmax_f(0.1, A1(Hi, ai)) * A1(eta, ai));
    } else {
      A1(eu, ai) = (4.0 * nxx + nyy);
      A1(ev, ai) = (4.0 * nyy + nxx);
    }
  }
}

int or_solve_SSA_linearised(const or_base *b, const or_aaac *m, const or_params *p,
                            const double *Hi, const double *Hb, const double *SL,
                            const double *hx, const double *hy, const double *eta,
                            const double *S, const int32_t *mask_gl_Ac,
                            double *U, double *V, int32_t *sweeps, double *max_res) {
  const int nA = m->nVAaAc;
  double *w = (double *)malloc(sizeof(double) * (size_t)nA * 4);
  int did_reset, not_conv;
  if (!w) return OR_ERR_BAD_ARG;
  double *RHSx = w, *RHSy = w + nA, *eu = w + 2 * (size_t)nA, *ev = w + 3 * (size_t)nA;
  rhs_and_centre(m, Hi, Hb, SL, hx, hy, eta, S, RHSx, RHSy, eu, ev);
  const int ns = sor_loop(b, m, p, mask_gl_Ac, RHSx, RHSy, eu, ev, U, V, &did_reset, &not_conv, max_res, 0, 0);
  if (sweeps) *sweeps = ns;
  free(w);
  if (did_reset) return OR_RESET_ONCE;
  return not_conv ? OR_NOT_CONVERGED : OR_OK;
}

/* basal_yield_stress, ice_dynamics_module.f90:780-844 */
static void basal_yield_stress(const or_base *b, const or_aaac *m, const or_ssa_fields *f, double *phi,
                               double *tau) {
  const int nV = b->nV, nAc = m->nAc;
  const double pf1 = -1000.0, pf2 = 0.0, p_min = 5.0, p_max = 20.0;
  for (int vi = 1; vi <= nV; vi++) {
    const int ai = vi;
    const double lambda_p = fmax_f(0.0, fmin_f(1.0, (1.0 - (A1(f->Hb, vi) - A1(f->SL, vi)) / 1000.0)));
    const double pwp = ((0.96 * ice_density) * grav) * fmax_f(0.1, A1(f->Hi, vi)) * lambda_p;
    A1(phi, ai) = fmax_f(p_min, fmin_f(p_max, (p_min + (p_max - p_min) * (1.0 + (A1(f->Hb, vi) - pf2) / (pf2 - pf1)))));
    A1(tau, ai) = tan((pi / 180.0) * A1(phi, ai)) * (((ice_density * grav) * fmax_f(0.1, A1(f->Hi, vi))) - pwp);
  }
  for (int aci = 1; aci <= nAc; aci++) {
    const int ai = aci + nV;
    const double lambda_p = fmax_f(0.0, fmin_f(1.0, (1.0 - (A1(f->Hb_Ac, aci) - A1(f->SL_Ac, aci)) / 1000.0)));
    const double pwp = ((0.96 * ice_density) * grav) * fmax_f(0.1, A1(f->Hi_Ac, aci)) * lambda_p;
    A1(phi, ai) = fmax_f(p_min, fmin_f(p_max, (p_min + (p_max - p_min) * (1.0 + (A1(f->Hb_Ac, aci) - pf2) / (pf2 - pf1)))));
    A1(tau, ai) = tan((pi / 180.0) * A1(phi, ai)) * (((ice_density * grav) * fmax_f(0.1, A1(f->Hi_Ac, aci))) - pwp);
  }
}

/* calculate_GL_flux, ice_dynamics_module.f90:848-949 (Coulomb_regularised / Tsai et al. 2015) */
static int gl_flux(const or_base *b, const or_aaac *m, const or_params *p, or_ssa_fields *f,
                   const double *phi_fric_AaAc) {
  const int nAc = m->nAc;
  const double Q0 = 0.61;
  if (p->sliding_law != 0) return OR_ERR_BAD_ARG; /* reference: only Coulomb_regularised */
  for (int aci = 1; aci <= nAc; aci++) {
    if (A1(f->mask_gl_Ac, aci) == 0) continue;
    const int vi = A2(m->Aci, nAc, aci, 1), vj = A2(m->Aci, nAc, aci, 2);
    const double TAFi = A1(f->Hi, vi) - ((A1(f->SL, vi) - A1(f->Hb, vi)) * (seawater_density / ice_density));
    const double TAFj = A1(f->Hi, vj) - ((A1(f->SL, vj) - A1(f->Hb, vj)) * (seawater_density / ice_density));
    const double lambda_GL = TAFi / (TAFi - TAFj);
    const double Hi_GL = (A1(f->Hi, vi) * (1.0 - lambda_GL)) + (A1(f->Hi, vj) * lambda_GL);
    double phi_GL, A_GL;
    if (A1(f->mask_sheet, vi) == 1) { phi_GL = A1(phi_fric_AaAc, vi); A_GL = A1(f->A_flow_mean, vi); }
    else { phi_GL = A1(phi_fric_AaAc, vj); A_GL = A1(f->A_flow_mean, vj); }
    const double rg = ice_density * grav;
    const double one_m = 1.0 - (ice_density / seawater_density);
    const double factor_Tsai = ((((8.0 * Q0) * A_GL) * pow(rg, n_flow)) * (one_m * one_m)) / pow(4.0, n_flow);
    const double Qabs = (factor_Tsai * pow(Hi_GL, n_flow + 2.0)) / tan(phi_GL * (pi / 180.0));
    double Fx = -(A1(f->dHi_dx_Ac, aci) - ((A1(f->dSL_dx_Ac, aci) - A1(f->dHb_dx_Ac, aci)) * (seawater_density / ice_density)));
    double Fy = -(A1(f->dHi_dy_Ac, aci) - ((A1(f->dSL_dy_Ac, aci) - A1(f->dHb_dy_Ac, aci)) * (seawater_density / ice_density)));
    const double F = norm2_2(Fx, Fy);
    Fx = Fx / F;
    Fy = Fy / F;
    A1(f->Ux_SSA_Ac, aci) = (Qabs * Fx) / Hi_GL;
    A1(f->Uy_SSA_Ac, aci) = (Qabs * Fy) / Hi_GL;
  }
  return OR_OK;
}

int or_solve_SSA(const or_base *b, const or_aaac *m, const or_params *p, or_ssa_fields *f,
                 or_ssa_stats *st) {
  const int nV = b->nV, nAc = m->nAc, nA = m->nVAaAc;
  const double epsilon_sq_0 = 1e-12;
  const double delta_v = 1e-3, q_plastic = 0.30, u_threshold = 100.0;
  int set_zero = p->zero_velocities != 0;
  int rc = OR_OK;
  int did_reset_before = 0;
  memset(st, 0, sizeof(*st));

  long sum_sheet = 0;
  for (int vi = 1; vi <= nV; vi++) sum_sheet += A1(f->mask_sheet, vi);
  if (sum_sheet == 0) set_zero = 1;
  if (set_zero) {
    for (int vi = 1; vi <= nV; vi++) { A1(f->U_SSA, vi) = 0.0; A1(f->V_SSA, vi) = 0.0; }
    for (int aci = 1; aci <= nAc; aci++) {
      A1(f->Ux_SSA_Ac, aci) = 0.0; A1(f->Uy_SSA_Ac, aci) = 0.0;
      if (f->Up_SSA_Ac) A1(f->Up_SSA_Ac, aci) = 0.0;
      if (f->Uo_SSA_Ac) A1(f->Uo_SSA_Ac, aci) = 0.0;
    }
    return OR_OK;
  }

  const size_t nAz = (size_t)nA;
  double *w = (double *)calloc(nAz * 22, sizeof(double));
  if (!w) return OR_ERR_BAD_ARG;
  double *Hi = w, *Hb = w + nAz, *SL = w + 2 * nAz, *hx = w + 3 * nAz, *hy = w + 4 * nAz,
         *Af = w + 5 * nAz, *U = w + 6 * nAz, *V = w + 7 * nAz, *eta = w + 8 * nAz,
         *N = w + 9 * nAz, *Nprev = w + 10 * nAz, *S = w + 11 * nAz, *tau = w + 12 * nAz,
         *phi = w + 13 * nAz, *dUdx = w + 14 * nAz, *dUdy = w + 15 * nAz, *dVdx = w + 16 * nAz,
         *dVdy = w + 17 * nAz, *RHSx = w + 18 * nAz, *RHSy = w + 19 * nAz, *eu = w + 20 * nAz,
         *ev = w + 21 * nAz;

  /* N_AaAc persists in the ice model between calls */
  if (f->N_AaAc) memcpy(N, f->N_AaAc, sizeof(double) * nAz);

  basal_yield_stress(b, m, f, phi, tau);
  if (p->use_analytical_GL_flux) {
    rc = gl_flux(b, m, p, f, phi);
    if (rc != OR_OK) { free(w); return rc; }
  }

  /* Gather Aa and Ac fields into AaAc (ice_dynamics_module.f90:478-495) */
  for (int vi = 1; vi <= nV; vi++) {
    A1(Hi, vi) = A1(f->Hi, vi); A1(Hb, vi) = A1(f->Hb, vi); A1(SL, vi) = A1(f->SL, vi);
    A1(hx, vi) = A1(f->dHs_dx_shelf, vi); A1(hy, vi) = A1(f->dHs_dy_shelf, vi);
    A1(Af, vi) = A1(f->A_flow_mean, vi);
    A1(U, vi) = A1(f->U_SSA, vi); A1(V, vi) = A1(f->V_SSA, vi);
  }
  for (int aci = 1; aci <= nAc; aci++) {
    const int ai = nV + aci;
    A1(Hi, ai) = A1(f->Hi_Ac, aci); A1(Hb, ai) = A1(f->Hb_Ac, aci); A1(SL, ai) = A1(f->SL_Ac, aci);
    A1(hx, ai) = A1(f->dHs_dx_shelf_Ac, aci); A1(hy, ai) = A1(f->dHs_dy_shelf_Ac, aci);
    A1(Af, ai) = A1(f->A_flow_mean_Ac, aci);
    A1(U, ai) = A1(f->Ux_SSA_Ac, aci); A1(V, ai) = A1(f->Uy_SSA_Ac, aci);
  }
  if (f->S_AaAc) memcpy(S, f->S_AaAc, sizeof(double) * nAz);

  int has_converged = 0, it = 0;
  const int max_outer = p->replay_picard > 0 ? p->replay_picard : p->SSA_max_outer_loops;
  while (!has_converged && it < max_outer) {
    it = it + 1;
    st->picard_iterations = it;
    memcpy(Nprev, N, sizeof(double) * nAz);
    /* SSA_effective_viscosity */
    or_ddx_ddy_AaAc(m, b->nC_mem, U, dUdx, dUdy);
    or_ddx_ddy_AaAc(m, b->nC_mem, V, dVdx, dVdy);
    for (int ai = 1; ai <= nA; ai++) {
      const double ux = A1(dUdx, ai), uy = A1(dUdy, ai), vx = A1(dVdx, ai), vy = A1(dVdy, ai);
      const double t = uy + vx;
      const double e2 = (((ux * ux + vy * vy) + ux * vy) + 0.25 * (t * t)) + epsilon_sq_0;
      A1(eta, ai) = pow((p->m_enh_ssa * 0.5) * A1(Af, ai), -1.0 / n_flow) *
                    pow(e2, (1.0 - n_flow) / (2.0 * n_flow));
      A1(N, ai) = A1(eta, ai) * fmax_f(0.1, A1(Hi, ai));
    }
    double sum_DN_sq = 0.0, sum_N_sq = 0.0;
    for (int ai = 1; ai <= nA; ai++) {
      const double d = A1(N, ai) - A1(Nprev, ai);
      sum_DN_sq = sum_DN_sq + d * d;
    }
    for (int ai = 1; ai <= nA; ai++) sum_N_sq = sum_N_sq + A1(N, ai) * A1(N, ai);
    const double RN = sqrt(sum_DN_sq / sum_N_sq);
    st->last_RN = RN;
    if (p->replay_picard <= 0 && RN < p->SSA_RN_tol) { has_converged = 1; break; }
    if (p->replay_picard > 0 && it == p->replay_picard) break;
    /* SSA_sliding_term */
    if (p->sliding_law == 0) {
      const double expo = 0.5 * (q_plastic - 1.0);
      const double uq = pow(u_threshold, q_plastic);
      for (int ai = 1; ai <= nA; ai++)
        A1(S, ai) = (A1(tau, ai) * pow((delta_v * delta_v + A1(U, ai) * A1(U, ai)) + A1(V, ai) * A1(V, ai), expo)) / uq;
    } else {
      for (int ai = 1; ai <= nA; ai++) A1(S, ai) = f->beta_sq_AaAc ? A1(f->beta_sq_AaAc, ai) : f->beta_sq_const;
    }
    /* solve_SSA_linearised */
    rhs_and_centre(m, Hi, Hb, SL, hx, hy, eta, S, RHSx, RHSy, eu, ev);
    int did_reset_now = 0, not_conv = 0;
    const int n_fixed = (p->replay_picard > 0 && p->replay_sweeps) ? p->replay_sweeps[it - 1] : 0;
    const int ns = sor_loop(b, m, p, f->mask_gl_Ac, RHSx, RHSy, eu, ev, U, V, &did_reset_now,
                            &not_conv, &st->last_max_residual, n_fixed, st->total_sweeps);
    if (st->linear_solves < 64) st->sweeps[st->linear_solves] = ns;
    st->linear_solves++;
    st->total_sweeps += ns;
    st->not_converged += not_conv;
    if (did_reset_now) {
      st->resets++;
      if (!did_reset_before) did_reset_before = 1;
      else { rc = OR_ERR_DIVERGED; break; }
    }
  }

  /* Scatter back (ice_dynamics_module.f90:548-552) and rotate (555) */
  for (int vi = 1; vi <= nV; vi++) { A1(f->U_SSA, vi) = A1(U, vi); A1(f->V_SSA, vi) = A1(V, vi); }
  for (int aci = 1; aci <= nAc; aci++) {
    A1(f->Ux_SSA_Ac, aci) = A1(U, nV + aci);
    A1(f->Uy_SSA_Ac, aci) = A1(V, nV + aci);
  }
  if (f->Up_SSA_Ac && f->Uo_SSA_Ac) {
    for (int ci = 1; ci <= nAc; ci++) {
      const int vi = A2(m->Aci, nAc, ci, 1), vj = A2(m->Aci, nAc, ci, 2);
      const double Dx = A2(b->V, nV, vj, 1) - A2(b->V, nV, vi, 1);
      const double Dy = A2(b->V, nV, vj, 2) - A2(b->V, nV, vi, 2);
      const double D = sqrt(Dx * Dx + Dy * Dy);
      A1(f->Up_SSA_Ac, ci) = (A1(f->Ux_SSA_Ac, ci) * Dx) / D + (A1(f->Uy_SSA_Ac, ci) * Dy) / D;
      A1(f->Uo_SSA_Ac, ci) = (A1(f->Uy_SSA_Ac, ci) * Dx) / D - (A1(f->Ux_SSA_Ac, ci) * Dy) / D;
    }
  }
  if (f->N_AaAc) memcpy(f->N_AaAc, N, sizeof(double) * nAz);
  if (f->eta_AaAc) memcpy(f->eta_AaAc, eta, sizeof(double) * nAz);
  if (f->S_AaAc) memcpy(f->S_AaAc, S, sizeof(double) * nAz);
  if (f->tau_c_AaAc) memcpy(f->tau_c_AaAc, tau, sizeof(double) * nAz);
  if (f->phi_fric_AaAc) memcpy(f->phi_fric_AaAc, phi, sizeof(double) * nAz);
  free(w);
  if (rc == OR_OK && st->resets == 1) rc = OR_RESET_ONCE;
  if (rc == OR_OK && st->not_converged > 0) rc = OR_NOT_CONVERGED;
  return rc;
}
