/*
 * CPU oracle, 3-D SIA velocities -- TEST INFRASTRUCTURE ONLY (see ufe_oracle.h).
 *
 * Literal FP64 restatement of solve_SIA_3D, ice_dynamics_module.f90:317-405, with
 * apply_Neumann_boundary_3D (mesh_derivatives_module.f90:541-597, edge vertices from their
 * non-edge neighbours, then the four corners from all neighbours), get_mesh_derivatives_vertex_3D
 * (372-391, home term first) and vertical_integrate (zeta_module.f90:58-85).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "ufe_oracle.h"

#define A1(p, i) ((p)[(size_t)(i) - 1])
#define A2(p, ld, i, j) ((p)[(size_t)((i) - 1) + (size_t)((j) - 1) * (size_t)(ld)])

static void neumann_3d(const or_base *b, double *d, int nz) {
  const int nV = b->nV;
  for (int vi = 5; vi <= nV; vi++) {
    if (A1(b->edge_index, vi) == 0) continue;
    for (int k = 1; k <= nz; k++) {
      double s = 0.0;
      int nvals = 0;
      for (int ci = 1; ci <= A1(b->nC, vi); ci++) {
        const int vc = A2(b->C, nV, vi, ci);
        if (A1(b->edge_index, vc) > 0) continue;
        nvals = nvals + 1;
        s = s + A2(d, nV, vc, k);
      }
      if (nvals < b->nC_mem) s = s + 0.0;   /* SUM over the unused +0 slots */
      A2(d, nV, vi, k) = s / (double)nvals;
    }
  }
  for (int vi = 1; vi <= 4; vi++) {
    for (int k = 1; k <= nz; k++) {
      double s = 0.0;
      int nvals = 0;
      for (int ci = 1; ci <= A1(b->nC, vi); ci++) {
        const int vc = A2(b->C, nV, vi, ci);
        nvals = nvals + 1;
        s = s + A2(d, nV, vc, k);
      }
      if (nvals < b->nC_mem) s = s + 0.0;
      A2(d, nV, vi, k) = s / (double)nvals;
    }
  }
}

static void ddxy_3d(const or_base *b, const or_aaac *m, const double *d, int vi, int k, double *ddx, double *ddy) {
  const int nV = b->nV, n = A1(b->nC, vi);
  double dx = A2(m->Nx, nV, vi, n + 1) * A2(d, nV, vi, k);
  double dy = A2(m->Ny, nV, vi, n + 1) * A2(d, nV, vi, k);
  for (int ci = 1; ci <= n; ci++) {
    const int vc = A2(b->C, nV, vi, ci);
    dx = dx + A2(m->Nx, nV, vi, ci) * A2(d, nV, vc, k);
    dy = dy + A2(m->Ny, nV, vi, ci) * A2(d, nV, vc, k);
  }
  *ddx = dx;
  *ddy = dy;
}

int or_solve_SIA_3D(const or_base *b, const or_aaac *m, const double *zeta, int nZ, double m_enh_sia,
                    const double *Hi, const int32_t *mask_shelf, const int32_t *mask_sheet, const double *dHs_dx,
                    const double *dHs_dy, const double *dHi_dx, const double *dHi_dy, const double *A_flow,
                    const double *dHb_dt, const double *U_SSA, const double *V_SSA, double *U_3D, double *V_3D,
                    double *W_3D) {
  const int nV = b->nV;
  const double n_flow = 3.0, rho_g = 910.0 * 9.81, cutoff = -1e5;
  double fz[64], D_def[64];
  if (nZ < 2 || nZ > 64) return OR_ERR_BAD_ARG;
  for (int vi = 1; vi <= nV; vi++)
    for (int k = 1; k <= nZ; k++) { A2(U_3D, nV, vi, k) = 0.0; A2(V_3D, nV, vi, k) = 0.0; A2(W_3D, nV, vi, k) = 0.0; }
  for (int vi = 1; vi <= nV; vi++) {
    for (int k = 1; k <= nZ; k++) { A2(U_3D, nV, vi, k) = A1(U_SSA, vi); A2(V_3D, nV, vi, k) = A1(V_SSA, vi); }
    if (A1(mask_shelf, vi) == 1) continue;
    if (A1(Hi, vi) == 0.0) continue;
    const double sx = A1(dHs_dx, vi), sy = A1(dHs_dy, vi);
    const double D_0 = pow(rho_g * A1(Hi, vi), n_flow) * pow(sx * sx + sy * sy, (n_flow - 1.0) / 2.0);
    for (int k = 1; k <= nZ; k++) fz[k - 1] = (m_enh_sia * A2(A_flow, nV, vi, k)) * pow(zeta[k - 1], n_flow);
    D_def[nZ - 1] = 0.0;
    for (int k = nZ - 1; k >= 1; k--) D_def[k - 1] = D_def[k] - (0.5 * (fz[k] + fz[k - 1])) * (zeta[k] - zeta[k - 1]);
    for (int k = 1; k <= nZ; k++) {
      double D = D_0 * ((2.0 * A1(Hi, vi)) * D_def[k - 1]);
      if (D < cutoff) D = cutoff;
      A2(U_3D, nV, vi, k) = D * sx + A1(U_SSA, vi);
      A2(V_3D, nV, vi, k) = D * sy + A1(V_SSA, vi);
    }
  }
  neumann_3d(b, U_3D, nZ);
  neumann_3d(b, V_3D, nZ);
  for (int vi = 1; vi <= nV; vi++) {
    if (A1(b->edge_index, vi) > 0) continue;
    if (A1(mask_sheet, vi) == 0) continue;
    const double dHb_dx = A1(dHs_dx, vi) - A1(dHi_dx, vi);
    const double dHb_dy = A1(dHs_dy, vi) - A1(dHi_dy, vi);
    A2(W_3D, nV, vi, nZ) = (A1(dHb_dt, vi) + A2(U_3D, nV, vi, nZ) * dHb_dx) + A2(V_3D, nV, vi, nZ) * dHb_dy;
    const double mH = A1(Hi, vi) > 0.1 ? A1(Hi, vi) : 0.1;
    for (int k = nZ - 1; k >= 1; k--) {
      double dUdx_k, dUdy_k, dUdx_kp1, dUdy_kp1, dVdx_k, dVdy_k, dVdx_kp1, dVdy_kp1;
      ddxy_3d(b, m, U_3D, vi, k, &dUdx_k, &dUdy_k);
      ddxy_3d(b, m, U_3D, vi, k + 1, &dUdx_kp1, &dUdy_kp1);
      ddxy_3d(b, m, V_3D, vi, k, &dVdx_k, &dVdy_k);
      ddxy_3d(b, m, V_3D, vi, k + 1, &dVdx_kp1, &dVdy_kp1);
      const double w1 = (dUdx_k + dUdx_kp1) / 2.0;
      const double w2 = (dVdy_k + dVdy_kp1) / 2.0;
      const double dz = zeta[k] - zeta[k - 1];
      const double zm = 0.5 * (zeta[k] + zeta[k - 1]);
      const double w3 = ((A1(dHs_dx, vi) - zm * A1(dHi_dx, vi)) / mH) * ((A2(U_3D, nV, vi, k + 1) - A2(U_3D, nV, vi, k)) / dz);
      const double w4 = ((A1(dHs_dy, vi) - zm * A1(dHi_dy, vi)) / mH) * ((A2(V_3D, nV, vi, k + 1) - A2(V_3D, nV, vi, k)) / dz);
      A2(W_3D, nV, vi, k) = A2(W_3D, nV, vi, k + 1) - (A1(Hi, vi) * (((w1 + w2) + w3) + w4)) * dz;
    }
  }
  neumann_3d(b, W_3D, nZ);
  return OR_OK;
}
