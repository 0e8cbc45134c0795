/*
 * CPU oracle, ice thickness update -- TEST INFRASTRUCTURE ONLY (see ufe_oracle.h).
 *
 * Literal FP64 restatement of calculate_ice_thickness_change, ice_dynamics_module.f90:31-237:
 * upwind ice volume fluxes across every Aa connection from the Ac parallel velocities
 * (66-106), the outflux rescale against the available ice plus SMB/BMB (108-169, a
 * sequential loop over the vertices as the reference runs it on one rank), dHi/dt
 * (171-181), the zero-time-step rule (183-185), the thickness update (187-190), the domain-
 * edge rule (192-230) and the no-ice mask (232-236); and bottom_frictional_heating,
 * thermodynamics_module.f90:281-311.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "ufe_oracle.h"

#define A1(p, i) ((p)[(size_t)(i) - 1])
#define A2(p, ld, i, j) ((p)[(size_t)((i) - 1) + (size_t)((j) - 1) * (size_t)(ld)])

int or_thickness_change(const or_base *b, const or_aaac *m, const double *A, const double *Cw,
                        const double *Up_SIA_Ac, const double *Up_SSA_Ac, const double *SMB_year,
                        const double *BMB, const int32_t *mask_noice, double dt, int zero_edges,
                        double *Hi, double *Hi_prev, double *dHi_dt, double *dVi_in) {
  const int nV = b->nV, nAc = m->nAc, ncm = b->nC_mem;
  double *Vi_SMB = (double *)calloc((size_t)nV, sizeof(double));
  if (!Vi_SMB) return OR_ERR_BAD_ARG;
  memset(dVi_in, 0, sizeof(double) * (size_t)nV * (size_t)ncm);
  for (int aci = 1; aci <= nAc; aci++) {
    const int vi = A2(m->Aci, nAc, aci, 1), vj = A2(m->Aci, nAc, aci, 2);
    int ci = 0, cj = 0;
    for (int cii = 1; cii <= A1(b->nC, vi); cii++)
      if (A2(b->C, nV, vi, cii) == vj) { ci = cii; break; }
    for (int cji = 1; cji <= A1(b->nC, vj); cji++)
      if (A2(b->C, nV, vj, cji) == vi) { cj = cji; break; }
    const double Upar = A1(Up_SIA_Ac, aci) + A1(Up_SSA_Ac, aci);
    double dVi;
    if (Upar > 0.0) dVi = ((A1(Hi, vi) * Upar) * A2(Cw, nV, vi, ci)) * dt;
    else dVi = ((A1(Hi, vj) * Upar) * A2(Cw, nV, vi, ci)) * dt;
    A2(dVi_in, nV, vi, ci) = -dVi;
    A2(dVi_in, nV, vj, cj) = dVi;
  }
  for (int vi = 1; vi <= nV; vi++)
    A1(Vi_SMB, vi) = ((A1(SMB_year, vi) + A1(BMB, vi)) * A1(A, vi)) * dt;
  for (int vi = 1; vi <= nV; vi++) {
    const double Vi_available = A1(A, vi) * A1(Hi, vi);
    double Vi_out = 0.0;
    for (int ci = 1; ci <= A1(b->nC, vi); ci++) {
      if (!(A2(dVi_in, nV, vi, ci) > 0.0)) Vi_out = Vi_out - A2(dVi_in, nV, vi, ci);
    }
    double rescale_factor = 1.0;
    if (-A1(Vi_SMB, vi) >= Vi_available) {
      A1(Vi_SMB, vi) = -Vi_available;
      rescale_factor = 0.0;
    }
    if (Vi_out > Vi_available + A1(Vi_SMB, vi)) rescale_factor = (Vi_available + A1(Vi_SMB, vi)) / Vi_out;
    if (rescale_factor < 1.0) {
      for (int ci = 1; ci <= A1(b->nC, vi); ci++) {
        const int vj = A2(b->C, nV, vi, ci);
        if (A2(dVi_in, nV, vi, ci) < 0.0) {
          A2(dVi_in, nV, vi, ci) = A2(dVi_in, nV, vi, ci) * rescale_factor;
          for (int cji = 1; cji <= A1(b->nC, vj); cji++) {
            if (A2(b->C, nV, vj, cji) == vi) { A2(dVi_in, nV, vj, cji) = -A2(dVi_in, nV, vi, ci); break; }
          }
        }
      }
    }
  }
  for (int vi = 1; vi <= nV; vi++) {
    double dVi = 0.0;
    for (int ci = 1; ci <= ncm; ci++) dVi = dVi + A2(dVi_in, nV, vi, ci);   /* SUM over the whole row */
    A1(dHi_dt, vi) = (dVi + A1(Vi_SMB, vi)) / (A1(A, vi) * dt);
  }
  if (dt == 0.0)
    for (int vi = 1; vi <= nV; vi++) A1(dHi_dt, vi) = 0.0;
  for (int vi = 1; vi <= nV; vi++) {
    A1(Hi_prev, vi) = A1(Hi, vi);
    A1(Hi, vi) = A1(Hi, vi) + (A1(dHi_dt, vi) * dt);
  }
  if (zero_edges)
    for (int vi = 1; vi <= nV; vi++)
      if (A1(b->edge_index, vi) > 0) A1(Hi, vi) = 0.0;
  if (mask_noice)
    for (int vi = 1; vi <= nV; vi++)
      if (A1(mask_noice, vi) == 1) A1(Hi, vi) = 0.0;
  free(Vi_SMB);
  return OR_OK;
}

/* bottom_frictional_heating, thermodynamics_module.f90:281-311: on grounded-ice vertices,
 * beta_base = tau_c * (delta_v^2 + U^2 + V^2)^(0.5 (q - 1)) / u_threshold^q and the heating
 * beta_base * (U^2 + V^2); zero elsewhere. */
void or_frictional_heating(int nV, const int32_t *mask_sheet, const double *tau_c_AaAc, const double *U,
                           const double *V, double *heating) {
  const double delta_v = 1e-3, q_plastic = 0.30, u_threshold = 100.0;
  for (int vi = 1; vi <= nV; vi++) {
    A1(heating, vi) = 0.0;
    if (A1(mask_sheet, vi) == 1) {
      const double u = A1(U, vi), v = A1(V, vi);
      const double beta_base = (A1(tau_c_AaAc, vi) * pow((delta_v * delta_v + u * u) + v * v, 0.5 * (q_plastic - 1.0))) /
                               pow(u_threshold, q_plastic);
      A1(heating, vi) = beta_base * (u * u + v * v);
    }
  }
}
