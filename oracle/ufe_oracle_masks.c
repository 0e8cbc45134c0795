/*
 * CPU oracle, the full mask set -- TEST INFRASTRUCTURE ONLY (see ufe_oracle.h).
 *
 * Literal restatement of determine_masks, general_ice_model_data_module.f90:97-297: land,
 * ocean, lake, ice, sheet, shelf, coast, margin, grounding-line and calving-front masks on the Aa
 * vertices and the Ac edges, and the combined type mask, whose value is the last type the
 * routine assigns (in its order: ocean, sheet, shelf, then coast, margin, grounding line,
 * calving front). is_floating follows general_ice_model_data_module.f90:464-475.
 */
#include <stddef.h>

#include "ufe_oracle.h"

#define A1(p, i) ((p)[(size_t)(i) - 1])
#define A2(p, ld, i, j) ((p)[(size_t)((i) - 1) + (size_t)((j) - 1) * (size_t)(ld)])

enum { T_LAND = 0, T_OCEAN = 1, T_LAKE = 2, T_SHEET = 3, T_SHELF = 4, T_COAST = 5, T_MARGIN = 6, T_GL = 7, T_CF = 8 };

static int floating(double Hi, double Hb, double SL) {
  return Hi < ((SL - Hb) * 1028.0) / 910.0;
}

/* Column k of the (n, OR_MASK_COUNT) array of masks. */
#define MK(p, n, i, k) A2(p, n, i, (k) + 1)

void or_determine_masks(const or_base *b, const or_aaac *m, const double *Hi, const double *Hb, const double *SL,
                        const double *Hi_Ac, const double *Hb_Ac, const double *SL_Ac, int32_t *aa, int32_t *ac) {
  const int nV = b->nV, nAc = m->nAc;
  for (int vi = 1; vi <= nV; vi++) {
    for (int k = 0; k < OR_MASK_COUNT; k++) MK(aa, nV, vi, k) = 0;
    MK(aa, nV, vi, OR_MASK_LAND) = 1;
    MK(aa, nV, vi, OR_MASK_TYPE) = T_LAND;
  }
  for (int aci = 1; aci <= nAc; aci++) {
    for (int k = 0; k < OR_MASK_COUNT; k++) MK(ac, nAc, aci, k) = 0;
    MK(ac, nAc, aci, OR_MASK_LAND) = 1;
    MK(ac, nAc, aci, OR_MASK_TYPE) = T_LAND;
  }
  /* Aa: ocean, ice, sheet, shelf (146-167) */
  for (int vi = 1; vi <= nV; vi++) {
    if (floating(A1(Hi, vi), A1(Hb, vi), A1(SL, vi))) {
      MK(aa, nV, vi, OR_MASK_OCEAN) = 1;
      MK(aa, nV, vi, OR_MASK_LAND) = 0;
      MK(aa, nV, vi, OR_MASK_TYPE) = T_OCEAN;
    }
    if (A1(Hi, vi) > 0.0) MK(aa, nV, vi, OR_MASK_ICE) = 1;
    if (MK(aa, nV, vi, OR_MASK_ICE) == 1 && MK(aa, nV, vi, OR_MASK_LAND) == 1) {
      MK(aa, nV, vi, OR_MASK_SHEET) = 1;
      MK(aa, nV, vi, OR_MASK_TYPE) = T_SHEET;
    }
    if (MK(aa, nV, vi, OR_MASK_ICE) == 1 && MK(aa, nV, vi, OR_MASK_OCEAN) == 1) {
      MK(aa, nV, vi, OR_MASK_SHELF) = 1;
      MK(aa, nV, vi, OR_MASK_TYPE) = T_SHELF;
    }
  }
  /* Aa: coast, margin, grounding line, calving front from the neighbours (171-225) */
  for (int vi = 1; vi <= nV; vi++) {
    const int n = A1(b->nC, vi);
    if (MK(aa, nV, vi, OR_MASK_LAND) == 1)
      for (int ci = 1; ci <= n; ci++)
        if (MK(aa, nV, A2(b->C, nV, vi, ci), OR_MASK_OCEAN) == 1) {
          MK(aa, nV, vi, OR_MASK_TYPE) = T_COAST;
          MK(aa, nV, vi, OR_MASK_COAST) = 1;
        }
    if (MK(aa, nV, vi, OR_MASK_ICE) == 1)
      for (int ci = 1; ci <= n; ci++)
        if (MK(aa, nV, A2(b->C, nV, vi, ci), OR_MASK_ICE) == 0) {
          MK(aa, nV, vi, OR_MASK_TYPE) = T_MARGIN;
          MK(aa, nV, vi, OR_MASK_MARGIN) = 1;
        }
    if (MK(aa, nV, vi, OR_MASK_SHEET) == 1)
      for (int ci = 1; ci <= n; ci++)
        if (MK(aa, nV, A2(b->C, nV, vi, ci), OR_MASK_SHELF) == 1) {
          MK(aa, nV, vi, OR_MASK_TYPE) = T_GL;
          MK(aa, nV, vi, OR_MASK_GL) = 1;
        }
    if (MK(aa, nV, vi, OR_MASK_ICE) == 1)
      for (int ci = 1; ci <= n; ci++)
        if (MK(aa, nV, A2(b->C, nV, vi, ci), OR_MASK_OCEAN) == 1) {
          MK(aa, nV, vi, OR_MASK_TYPE) = T_CF;
          MK(aa, nV, vi, OR_MASK_CF) = 1;
        }
  }
  /* Ac: ocean, ice, sheet, shelf (230-256) */
  for (int aci = 1; aci <= nAc; aci++) {
    if (floating(A1(Hi_Ac, aci), A1(Hb_Ac, aci), A1(SL_Ac, aci))) {
      MK(ac, nAc, aci, OR_MASK_OCEAN) = 1;
      MK(ac, nAc, aci, OR_MASK_LAND) = 0;
      MK(ac, nAc, aci, OR_MASK_TYPE) = T_OCEAN;
    }
    if (A1(Hi_Ac, aci) > 0.0) MK(ac, nAc, aci, OR_MASK_ICE) = 1;
    if (MK(ac, nAc, aci, OR_MASK_ICE) == 1 && MK(ac, nAc, aci, OR_MASK_LAND) == 1) {
      MK(ac, nAc, aci, OR_MASK_SHEET) = 1;
      MK(ac, nAc, aci, OR_MASK_TYPE) = T_SHEET;
    }
    if (MK(ac, nAc, aci, OR_MASK_ICE) == 1 && MK(ac, nAc, aci, OR_MASK_OCEAN) == 1) {
      MK(ac, nAc, aci, OR_MASK_SHELF) = 1;
      MK(ac, nAc, aci, OR_MASK_TYPE) = T_SHELF;
    }
  }
  /* Ac: coast, margin, grounding line, calving front from the edge's two vertices (260-294) */
  for (int aci = 1; aci <= nAc; aci++) {
    const int vi = A2(m->Aci, nAc, aci, 1), vj = A2(m->Aci, nAc, aci, 2);
#define AA(v, k) MK(aa, nV, v, k)
    if ((AA(vi, OR_MASK_LAND) == 1 && AA(vj, OR_MASK_OCEAN) == 1) ||
        (AA(vj, OR_MASK_LAND) == 1 && AA(vi, OR_MASK_OCEAN) == 1)) {
      MK(ac, nAc, aci, OR_MASK_TYPE) = T_COAST;
      MK(ac, nAc, aci, OR_MASK_COAST) = 1;
    }
    if ((AA(vi, OR_MASK_ICE) == 1 && AA(vj, OR_MASK_ICE) == 0) ||
        (AA(vj, OR_MASK_ICE) == 1 && AA(vi, OR_MASK_ICE) == 0)) {
      MK(ac, nAc, aci, OR_MASK_TYPE) = T_MARGIN;
      MK(ac, nAc, aci, OR_MASK_MARGIN) = 1;
    }
    if ((AA(vi, OR_MASK_SHEET) == 1 && AA(vj, OR_MASK_SHELF) == 1) ||
        (AA(vj, OR_MASK_SHEET) == 1 && AA(vi, OR_MASK_SHELF) == 1)) {
      MK(ac, nAc, aci, OR_MASK_TYPE) = T_GL;
      MK(ac, nAc, aci, OR_MASK_GL) = 1;
    }
    if ((AA(vi, OR_MASK_ICE) == 1 && AA(vj, OR_MASK_SHELF) == 0 && AA(vj, OR_MASK_OCEAN) == 1) ||
        (AA(vj, OR_MASK_ICE) == 1 && AA(vi, OR_MASK_SHELF) == 0 && AA(vi, OR_MASK_OCEAN) == 1)) {
      MK(ac, nAc, aci, OR_MASK_TYPE) = T_CF;
      MK(ac, nAc, aci, OR_MASK_CF) = 1;
    }
#undef AA
  }
}
