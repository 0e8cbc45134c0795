/*
 * CPU oracle, ice physical properties -- TEST INFRASTRUCTURE ONLY (see ufe_oracle.h).
 *
 * Literal FP64 restatement of ice_physical_properties, general_ice_model_data_module.f90:298-462
 * (the benchmark branches 324-368, the Arrhenius law and the Pounder / Ritz parameterisations
 * 370-459), with map_Aa_to_Ac_3D (mesh_ArakawaC_module.f90:748-769) for Ti_Ac and
 * vertical_average (zeta_module.f90:33-57). Constants T0, CC, SMT, sec_per_year from
 * parameters_module.f90:10-21; the Arrhenius constants are the routine's own (318-322).
 */
#include <math.h>
#include <stddef.h>

#include "ufe_oracle.h"

#define A1(p, i) ((p)[(size_t)(i) - 1])
#define A2(p, ld, i, j) ((p)[(size_t)((i) - 1) + (size_t)((j) - 1) * (size_t)(ld)])

static const double kT0 = 273.16, kCC = 8.7E-04, kSMT = 271.15, kSecPerYear = 31556943.36;
static const double kALow = 1.14E-05, kAHigh = 5.47E+10, kQLow = 6.0E+04, kQHigh = 13.9E+04, kRGas = 8.314;

static double arrhenius(double T) {
  if (T < 263.15) return kALow * exp(-kQLow / (kRGas * T));
  return kAHigh * exp(-kQHigh / (kRGas * T));
}

/* zeta_module.f90:33-57: trapezoid sum from the base upwards. The profile is f(k) = p[(k-1)*ld]. */
static double vertical_average(const double *zeta, int nZ, const double *p, size_t ld) {
  double s = 0.0;
  for (int k = 1; k <= nZ - 1; k++) s = s + 0.5 * (p[(size_t)k * ld] + p[(size_t)(k - 1) * ld]) * (zeta[k] - zeta[k - 1]);
  return s;
}

int or_ice_physical_properties(int nV, int nAc, int nZ, const double *zeta, const int32_t *Aci, int flow_law,
                               double time, const double *Hi, const int32_t *mask_sheet,
                               const int32_t *mask_sheet_Ac, const double *Ti, double *A_flow, double *A_flow_Ac,
                               double *A_flow_mean, double *A_flow_mean_Ac, double *Ti_pmp, double *Cpi, double *Ki,
                               double *Ti_Ac) {
  if (nV < 1 || nAc < 1 || nZ < 2 || !zeta || !Aci || !Hi || !mask_sheet || !mask_sheet_Ac || !A_flow ||
      !A_flow_Ac || !A_flow_mean || !A_flow_mean_Ac || !Ti_pmp || !Cpi || !Ki || !Ti_Ac)
    return OR_ERR_BAD_ARG;
  if (flow_law == 1) {          /* EISMINT_1..6, Halfar, Bueler, mesh_generation_test (326-351) */
    for (int vi = 1; vi <= nV; vi++)
      for (int k = 1; k <= nZ; k++) {
        A2(A_flow, nV, vi, k) = 1.0E-16;
        A2(Ki, nV, vi, k) = 2.1 * kSecPerYear;
        A2(Cpi, nV, vi, k) = 2009.0;
      }
    for (int ci = 1; ci <= nAc; ci++)
      for (int k = 1; k <= nZ; k++) A2(A_flow_Ac, nAc, ci, k) = 1.0E-16;
    for (int vi = 1; vi <= nV; vi++) A1(A_flow_mean, vi) = 1.0E-16;
    for (int ci = 1; ci <= nAc; ci++) A1(A_flow_mean_Ac, ci) = 1.0E-16;
    for (int vi = 1; vi <= nV; vi++)
      for (int k = 1; k <= nZ; k++) A2(Ti_pmp, nV, vi, k) = kT0 - (zeta[k - 1] * A1(Hi, vi) * 8.7E-04);
    return OR_OK;
  }
  if (flow_law == 2) {          /* MISMIP_mod (353-368) */
    double A = 1.0E-16;
    if (time < 25000.0) A = 1.0E-16;
    else if (time < 50000.0) A = 1.0E-17;
    else if (time < 75000.0) A = 1.0E-16;
    for (int vi = 1; vi <= nV; vi++)
      for (int k = 1; k <= nZ; k++) A2(A_flow, nV, vi, k) = A;
    for (int ci = 1; ci <= nAc; ci++)
      for (int k = 1; k <= nZ; k++) A2(A_flow_Ac, nAc, ci, k) = A;
    for (int vi = 1; vi <= nV; vi++) A1(A_flow_mean, vi) = A;
    for (int ci = 1; ci <= nAc; ci++) A1(A_flow_mean_Ac, ci) = A;
    return OR_OK;
  }
  if (flow_law != 0 || !Ti) return OR_ERR_BAD_ARG;
  /* update_general_ice_model_data maps Ti to Ac before the masks and properties (43) */
  for (int aci = 1; aci <= nAc; aci++) {
    const int vi = A2(Aci, nAc, aci, 1), vj = A2(Aci, nAc, aci, 2);
    for (int k = 1; k <= nZ; k++) A2(Ti_Ac, nAc, aci, k) = (A2(Ti, nV, vi, k) + A2(Ti, nV, vj, k)) / 2.0;
  }
  /* Aa (386-421) */
  for (int vi = 1; vi <= nV; vi++) {
    for (int k = 1; k <= nZ; k++) A2(Ti_pmp, nV, vi, k) = kT0 - kCC * A1(Hi, vi) * zeta[k - 1];
    for (int k = 1; k <= nZ; k++) {
      const double T = A2(Ti, nV, vi, k);
      A2(A_flow, nV, vi, k) = arrhenius(T);
      A2(Cpi, nV, vi, k) = 2115.3 + 7.79293 * (T - kT0);
      A2(Ki, nV, vi, k) = 3.101E+08 * exp(-0.0057 * T);
    }
    if (A1(mask_sheet, vi) == 1) {
      A1(A_flow_mean, vi) = vertical_average(zeta, nZ, &A2(A_flow, nV, vi, 1), (size_t)nV);
    } else {
      const double Ti_mean = (A2(Ti, nV, vi, 1) + kSMT) / 2.0;
      A1(A_flow_mean, vi) = arrhenius(Ti_mean);
    }
  }
  /* Ac (426-459) */
  for (int ci = 1; ci <= nAc; ci++) {
    for (int k = 1; k <= nZ; k++) A2(A_flow_Ac, nAc, ci, k) = arrhenius(A2(Ti_Ac, nAc, ci, k));
    if (A1(mask_sheet_Ac, ci) == 1) {
      A1(A_flow_mean_Ac, ci) = vertical_average(zeta, nZ, &A2(A_flow_Ac, nAc, ci, 1), (size_t)nAc);
    } else {
      const double Ti_mean = (A2(Ti_Ac, nAc, ci, 1) + kSMT) / 2.0;
      A1(A_flow_mean_Ac, ci) = arrhenius(Ti_mean);
    }
  }
  return OR_OK;
}
