/*
 * CPU oracle, mesh part -- TEST INFRASTRUCTURE ONLY (see ufe_oracle.h).
 *
 * Literal restatements of
 *   mesh_help_functions_module.f90:673-747   is_boundary_segment
 *   mesh_ArakawaC_module.f90:24-241           make_Ac_mesh
 *   mesh_ArakawaC_module.f90:242-285          find_Ac_edge_indices
 *   mesh_ArakawaC_module.f90:286-540          make_combined_AaAc_mesh (TriAaAc omitted: plotting only)
 *   mesh_derivatives_module.f90:14-75         get_neighbour_functions (vertex part)
 *   mesh_derivatives_module.f90:76-313        get_neighbour_functions_vertex_gr
 *   mesh_five_colour_module.f90:18-735        calculate_five_colouring_AaAc and its queue routines
 * with one process (partition_list with n = 1 gives the full index range,
 * mesh_help_functions_module.f90:1475-1495).
 */
#include "ufe_oracle.h"

#include <math.h>
#include <setjmp.h>
#include <stdlib.h>
#include <string.h>

/* 1-based, column-major access, as in the Fortran source. */
#define A1(p, i) ((p)[(size_t)(i) - 1])
#define A2(p, ld, i, j) ((p)[(size_t)((i) - 1) + (size_t)((j) - 1) * (size_t)(ld)])

static int is_boundary_segment(const or_base *b, int v1, int v2) {
  const int e1 = A1(b->edge_index, v1), e2 = A1(b->edge_index, v2);
  if (e1 == 0 || e2 == 0) return 0;
  switch (e1) {
    case 1: return e2 == 8 || e2 == 1 || e2 == 2;
    case 2: return e2 == 8 || e2 == 1 || e2 == 2 || e2 == 3 || e2 == 4;
    case 3: return e2 == 2 || e2 == 3 || e2 == 4;
    case 4: return e2 == 2 || e2 == 3 || e2 == 4 || e2 == 5 || e2 == 6;
    case 5: return e2 == 4 || e2 == 5 || e2 == 6;
    case 6: return e2 == 4 || e2 == 5 || e2 == 6 || e2 == 7 || e2 == 8;
    case 7: return e2 == 6 || e2 == 7 || e2 == 8;
    case 8: return e2 == 6 || e2 == 7 || e2 == 8 || e2 == 1 || e2 == 2;
  }
  return 0;
}

/* get_neighbour_functions_vertex_gr, mesh_derivatives_module.f90:76-313.
 * Nx..Nyy have nC_mem+1 entries in the caller; here indexed 1..n+1. */
void or_neighbour_functions_vertex(const double *V_vi, int n, const double *V_vc, int ld_vc,
                                   int is_edge, double *Nx, double *Ny, double *Nxx,
                                   double *Nxy, double *Nyy) {
#define VC(i, j) A2(V_vc, ld_vc, i, j)
  double NxTri[64][3], NyTri[64][3], NxSub[64][3], NySub[64][3];
  int nTri, nSub, ti, tip1s, si, sip1s, sip2s, ci, cim1s, sim1s, sim2s;
  double xi, yi, xt, yt, xtp1s, ytp1s, nzt;
  double xs, ys, xsp1s, ysp1s, xsp2s, ysp2s, nzs;
  double Axxis, Bxxis, Cxxis, Axyis, Bxyis, Cxyis, Ayyis, Byyis, Cyyis;
  double s;

  /* Nx = 0 ... (the caller's whole row is zeroed) */
  for (ci = 1; ci <= n + 1; ci++) {
    A1(Nx, ci) = 0.0; A1(Ny, ci) = 0.0; A1(Nxx, ci) = 0.0; A1(Nxy, ci) = 0.0; A1(Nyy, ci) = 0.0;
  }
  if (is_edge) { nTri = n - 1; nSub = n - 2; }
  else { nTri = n; nSub = n; }

  for (ti = 1; ti <= nTri; ti++) {
    tip1s = ti + 1;
    if (tip1s > n) tip1s = tip1s - n;
    xi = V_vi[0]; yi = V_vi[1];
    xt = VC(ti, 1); yt = VC(ti, 2);
    xtp1s = VC(tip1s, 1); ytp1s = VC(tip1s, 2);
    nzt = ((xt - xi) * (ytp1s - yi)) - ((yt - yi) * (xtp1s - xi)); /* Eq. A1 */
    NxTri[ti - 1][0] = (yt - ytp1s) / nzt;                           /* Eq. A3a */
    NxTri[ti - 1][1] = (ytp1s - yi) / nzt;
    NxTri[ti - 1][2] = (yi - yt) / nzt;
    NyTri[ti - 1][0] = (xtp1s - xt) / nzt;                           /* Eq. A3b */
    NyTri[ti - 1][1] = (xi - xtp1s) / nzt;
    NyTri[ti - 1][2] = (xt - xi) / nzt;
  }

  for (si = 1; si <= nSub; si++) {
    sip1s = si + 1;
    if (sip1s > n) sip1s = sip1s - n;
    sip2s = sip1s + 1;
    if (sip2s > n) sip2s = sip2s - n;
    xi = V_vi[0]; yi = V_vi[1];
    xs = VC(si, 1); ys = VC(si, 2);
    xsp1s = VC(sip1s, 1); ysp1s = VC(sip1s, 2);
    xsp2s = VC(sip2s, 1); ysp2s = VC(sip2s, 2);
    /* Eq. A11: 1._dp/3._dp * (a) * (b) evaluates as ((1/3)*a)*b; 2*xi is 2.0*xi. */
    nzs = (((1.0 / 3.0) * ((xs + xsp1s) - 2.0 * xi)) * ((ysp1s + ysp2s) - 2.0 * yi)) -
          (((1.0 / 3.0) * ((ys + ysp1s) - 2.0 * yi)) * ((xsp1s + xsp2s) - 2.0 * xi));
    NxSub[si - 1][0] = (ys - ysp2s) / nzs;                                   /* Eq. A13a */
    NxSub[si - 1][1] = ((ysp1s + ysp2s) - 2.0 * yi) / nzs;
    NxSub[si - 1][2] = ((2.0 * yi - ys) - ysp1s) / nzs;
    NySub[si - 1][0] = (xsp2s - xs) / nzs;                                   /* Eq. A13b */
    NySub[si - 1][1] = ((2.0 * xi - xsp1s) - xsp2s) / nzs;
    NySub[si - 1][2] = ((xs + xsp1s) - 2.0 * xi) / nzs;
  }

  /* First-order neighbour functions on the vertex */
  if (!is_edge) {
    s = 0.0;
    for (ti = 1; ti <= n; ti++) s = s + NxTri[ti - 1][0];
    A1(Nx, n + 1) = (1.0 / (double)n) * s;                                  /* Eq. A7a */
    s = 0.0;
    for (ti = 1; ti <= n; ti++) s = s + NyTri[ti - 1][0];
    A1(Ny, n + 1) = (1.0 / (double)n) * s;
    for (ci = 1; ci <= n; ci++) {
      cim1s = ci - 1;
      if (cim1s == 0) cim1s = cim1s + n;
      A1(Nx, ci) = (1.0 / (double)n) * (NxTri[ci - 1][1] + NxTri[cim1s - 1][2]); /* Eq. A7b */
      A1(Ny, ci) = (1.0 / (double)n) * (NyTri[ci - 1][1] + NyTri[cim1s - 1][2]);
    }
  } else {
    s = 0.0;
    for (ti = 1; ti <= n - 1; ti++) s = s + NxTri[ti - 1][0];
    A1(Nx, n + 1) = (1.0 / (double)(n - 1)) * s;                            /* Eq. A9a */
    s = 0.0;
    for (ti = 1; ti <= n - 1; ti++) s = s + NyTri[ti - 1][0];
    A1(Ny, n + 1) = (1.0 / (double)(n - 1)) * s;
    for (ci = 1; ci <= n; ci++) {
      if (ci == 1) {
        A1(Nx, ci) = (1.0 / (double)(n - 1)) * NxTri[0][1];                 /* Eq. A9b */
        A1(Ny, ci) = (1.0 / (double)(n - 1)) * NyTri[0][1];
      } else if (ci == n) {
        A1(Nx, ci) = (1.0 / (double)(n - 1)) * NxTri[n - 2][2];
        A1(Ny, ci) = (1.0 / (double)(n - 1)) * NyTri[n - 2][2];
      } else {
        A1(Nx, ci) = (1.0 / (double)(n - 1)) * (NxTri[ci - 1][1] + NxTri[ci - 2][2]);
        A1(Ny, ci) = (1.0 / (double)(n - 1)) * (NyTri[ci - 1][1] + NyTri[ci - 2][2]);
      }
    }
  }

  /* Second-order neighbour functions on the vertex */
  if (!is_edge) {
    const double rn = 1.0 / (double)n;
    for (si = 1; si <= n; si++) {
      sip1s = si + 1;
      if (sip1s > n) sip1s = sip1s - n;
      A1(Nxx, n + 1) = A1(Nxx, n + 1) + (rn * (((NxSub[si - 1][0] * A1(Nx, n + 1)) +     /* Eq. A23a */
                                                (NxSub[si - 1][1] * NxTri[si - 1][0])) +
                                               (NxSub[si - 1][2] * NxTri[sip1s - 1][0])));
      A1(Nxy, n + 1) = A1(Nxy, n + 1) + (rn * (((NySub[si - 1][0] * A1(Nx, n + 1)) +     /* Eq. A23b */
                                                (NySub[si - 1][1] * NxTri[si - 1][0])) +
                                               (NySub[si - 1][2] * NxTri[sip1s - 1][0])));
      A1(Nyy, n + 1) = A1(Nyy, n + 1) + (rn * (((NySub[si - 1][0] * A1(Ny, n + 1)) +     /* Eq. A23c */
                                                (NySub[si - 1][1] * NyTri[si - 1][0])) +
                                               (NySub[si - 1][2] * NyTri[sip1s - 1][0])));
    }
    double sumNxSub1 = 0.0, sumNySub1 = 0.0;
    for (si = 1; si <= n; si++) sumNxSub1 = sumNxSub1 + NxSub[si - 1][0];
    for (si = 1; si <= n; si++) sumNySub1 = sumNySub1 + NySub[si - 1][0];
    for (si = 1; si <= n; si++) {
      sim1s = si - 1;
      if (sim1s < 1) sim1s = sim1s + n;
      sim2s = sim1s - 1;
      if (sim2s < 1) sim2s = sim2s + n;
      A1(Nxx, si) = rn * (((NxTri[si - 1][1] * (NxSub[si - 1][1] + NxSub[sim1s - 1][2])) +       /* Eq. A23d */
                           (NxTri[sim1s - 1][2] * (NxSub[sim1s - 1][1] + NxSub[sim2s - 1][2]))) +
                          (A1(Nx, si) * sumNxSub1));
      A1(Nxy, si) = rn * (((NxTri[si - 1][1] * (NySub[si - 1][1] + NySub[sim1s - 1][2])) +       /* Eq. A23e */
                           (NxTri[sim1s - 1][2] * (NySub[sim1s - 1][1] + NySub[sim2s - 1][2]))) +
                          (A1(Nx, si) * sumNySub1));
      A1(Nyy, si) = rn * (((NyTri[si - 1][1] * (NySub[si - 1][1] + NySub[sim1s - 1][2])) +       /* Eq. A23f */
                           (NyTri[sim1s - 1][2] * (NySub[sim1s - 1][1] + NySub[sim2s - 1][2]))) +
                          (A1(Ny, si) * sumNySub1));
    }
  } else {
    const double rn2 = 1.0 / (double)(n - 2);
    for (si = 1; si <= n - 2; si++) {
      A1(Nxx, n + 1) = A1(Nxx, n + 1) + (rn2 * (((NxSub[si - 1][0] * A1(Nx, n + 1)) +    /* Eq. A24a */
                                                 (NxSub[si - 1][1] * NxTri[si - 1][0])) +
                                                (NxSub[si - 1][2] * NxTri[si][0])));
      A1(Nxy, n + 1) = A1(Nxy, n + 1) + (rn2 * (((NySub[si - 1][0] * A1(Nx, n + 1)) +    /* Eq. A24b */
                                                 (NySub[si - 1][1] * NxTri[si - 1][0])) +
                                                (NySub[si - 1][2] * NxTri[si][0])));
      A1(Nyy, n + 1) = A1(Nyy, n + 1) + (rn2 * (((NySub[si - 1][0] * A1(Ny, n + 1)) +    /* Eq. A24c */
                                                 (NySub[si - 1][1] * NyTri[si - 1][0])) +
                                                (NySub[si - 1][2] * NyTri[si][0])));
    }
    double sumNxSub1 = 0.0, sumNySub1 = 0.0;
    for (si = 1; si <= n - 2; si++) sumNxSub1 = sumNxSub1 + NxSub[si - 1][0];
    for (si = 1; si <= n - 2; si++) sumNySub1 = sumNySub1 + NySub[si - 1][0];
    for (si = 1; si <= n; si++) {
      if (si < n - 1) {
        Axxis = NxSub[si - 1][1] * NxTri[si - 1][1];   /* Eq. A25a */
        Axyis = NySub[si - 1][1] * NxTri[si - 1][1];   /* Eq. A25b */
        Ayyis = NySub[si - 1][1] * NyTri[si - 1][1];   /* Eq. A25c */
      } else {
        Axxis = 0.0; Axyis = 0.0; Ayyis = 0.0;
      }
      if (si > 1 && si < n) {
        Bxxis = (NxSub[si - 2][1] * NxTri[si - 2][2]) + (NxSub[si - 2][2] * NxTri[si - 1][1]); /* Eq. A25d */
        Bxyis = (NySub[si - 2][1] * NxTri[si - 2][2]) + (NySub[si - 2][2] * NxTri[si - 1][1]); /* Eq. A25e */
        Byyis = (NySub[si - 2][1] * NyTri[si - 2][2]) + (NySub[si - 2][2] * NyTri[si - 1][1]); /* Eq. A25f */
      } else {
        Bxxis = 0.0; Bxyis = 0.0; Byyis = 0.0;
      }
      if (si > 2) {
        Cxxis = NxSub[si - 3][2] * NxTri[si - 2][2];   /* Eq. A25g */
        Cxyis = NySub[si - 3][2] * NxTri[si - 2][2];   /* Eq. A25h */
        Cyyis = NySub[si - 3][2] * NyTri[si - 2][2];   /* Eq. A25i */
      } else {
        Cxxis = 0.0; Cxyis = 0.0; Cyyis = 0.0;
      }
      A1(Nxx, si) = rn2 * (((Axxis + Bxxis) + Cxxis) + (A1(Nx, si) * sumNxSub1)); /* Eq. A24d */
      A1(Nxy, si) = rn2 * (((Axyis + Bxyis) + Cxyis) + (A1(Nx, si) * sumNySub1)); /* Eq. A24e */
      A1(Nyy, si) = rn2 * (((Ayyis + Byyis) + Cyyis) + (A1(Ny, si) * sumNySub1)); /* Eq. A24f */
    }
  }
#undef VC
}

/* Neighbour functions for one row of a (n_rows, nC_mem+1) column-major coefficient set. */
static void nf_row(int ai, int n_rows, int nC_mem, const double *V_vi, int n, const double *V_vc,
                   int is_edge, double *Nx, double *Ny, double *Nxx, double *Nxy, double *Nyy) {
  double tx[65], ty[65], txx[65], txy[65], tyy[65];
  int ci;
  or_neighbour_functions_vertex(V_vi, n, V_vc, nC_mem, is_edge, tx, ty, txx, txy, tyy);
  /* The Fortran dummy arguments are whole rows (nC_mem+1 entries) set to zero first. */
  for (ci = 1; ci <= nC_mem + 1; ci++) {
    double vx = 0.0, vy = 0.0, vxx = 0.0, vxy = 0.0, vyy = 0.0;
    if (ci <= n + 1) { vx = tx[ci - 1]; vy = ty[ci - 1]; vxx = txx[ci - 1]; vxy = txy[ci - 1]; vyy = tyy[ci - 1]; }
    A2(Nx, n_rows, ai, ci) = vx;
    A2(Ny, n_rows, ai, ci) = vy;
    A2(Nxx, n_rows, ai, ci) = vxx;
    A2(Nxy, n_rows, ai, ci) = vxy;
    A2(Nyy, n_rows, ai, ci) = vyy;
  }
}

int or_build_aaac(const or_base *b, or_aaac *m) {
  const int nV = b->nV, nCm = b->nC_mem, nTri = b->nTri;
  const double *V = b->V;
  int vi, ci, vj, cj, iti, ti, n1, n2, n3, vl = 0, vr = 0, k;
  int nAc = 0;
  const int nAc_cap = nTri * 3;
  double *V_vc = (double *)malloc(sizeof(double) * (size_t)nCm * 2);
  if (!V_vc) return OR_ERR_BAD_ARG;

  /* == get_neighbour_functions, vertex part (mesh_derivatives_module.f90:48-71) == */
  for (vi = 1; vi <= nV; vi++) {
    const double V_vi[2] = {A2(V, nV, vi, 1), A2(V, nV, vi, 2)};
    const int n = A1(b->nC, vi);
    for (ci = 1; ci <= n; ci++) {
      const int vc = A2(b->C, nV, vi, ci);
      A2(V_vc, nCm, ci, 1) = A2(V, nV, vc, 1);
      A2(V_vc, nCm, ci, 2) = A2(V, nV, vc, 2);
    }
    nf_row(vi, nV, nCm, V_vi, n, V_vc, A1(b->edge_index, vi) > 0, m->Nx, m->Ny, m->Nxx, m->Nxy, m->Nyy);
  }

  /* == make_Ac_mesh (mesh_ArakawaC_module.f90:24-241) == */
  memset(m->iAci, 0, sizeof(int32_t) * (size_t)nV * nCm);
  for (vi = 1; vi <= nV; vi++) {
    for (ci = 1; ci <= A1(b->nC, vi); ci++) {
      double Nxl[4], Nyl[4], Nxr[4], Nyr[4], Nzl, Nzr, Nx[4], Ny[4], Ux, Uy, U, Np, No[4];
      vj = A2(b->C, nV, vi, ci);
      if (A2(m->iAci, nV, vi, ci) > 0) continue;
      nAc = nAc + 1;
      if (nAc > nAc_cap || nAc > m->nAc) { free(V_vc); return OR_ERR_BAD_MESH; }
      A2(m->iAci, nV, vi, ci) = nAc;
      A2(m->VAc, m->nAc, nAc, 1) = (A2(V, nV, vi, 1) + A2(V, nV, vj, 1)) / 2.0;
      A2(m->VAc, m->nAc, nAc, 2) = (A2(V, nV, vi, 2) + A2(V, nV, vj, 2)) / 2.0;
      for (cj = 1; cj <= A1(b->nC, vj); cj++) {
        if (A2(b->C, nV, vj, cj) == vi) { A2(m->iAci, nV, vj, cj) = nAc; break; }
      }
#define VX(v) A2(V, nV, v, 1)
#define VY(v) A2(V, nV, v, 2)
      if (!is_boundary_segment(b, vi, vj)) {
        for (iti = 1; iti <= A1(b->niTri, vi); iti++) {
          ti = A2(b->iTri, nV, vi, iti);
          for (n1 = 1; n1 <= 3; n1++) {
            n2 = n1 + 1; if (n2 == 4) n2 = 1;
            n3 = n2 + 1; if (n3 == 4) n3 = 1;
            if (A2(b->Tri, nTri, ti, n1) == vi && A2(b->Tri, nTri, ti, n2) == vj) {
              vl = A2(b->Tri, nTri, ti, n3);
            } else if (A2(b->Tri, nTri, ti, n1) == vj && A2(b->Tri, nTri, ti, n2) == vi) {
              vr = A2(b->Tri, nTri, ti, n3);
            }
          }
        }
        A2(m->Aci, m->nAc, nAc, 1) = vi; A2(m->Aci, m->nAc, nAc, 2) = vj;
        A2(m->Aci, m->nAc, nAc, 3) = vl; A2(m->Aci, m->nAc, nAc, 4) = vr;
        Nxl[0] = VY(vl) - VY(vj); Nxl[1] = VY(vi) - VY(vl); Nxl[2] = VY(vj) - VY(vi); Nxl[3] = 0.0;
        Nyl[0] = VX(vj) - VX(vl); Nyl[1] = VX(vl) - VX(vi); Nyl[2] = VX(vi) - VX(vj); Nyl[3] = 0.0;
        Nxr[0] = VY(vj) - VY(vr); Nxr[1] = VY(vr) - VY(vi); Nxr[2] = 0.0; Nxr[3] = VY(vi) - VY(vj);
        Nyr[0] = VX(vr) - VX(vj); Nyr[1] = VX(vi) - VX(vr); Nyr[2] = 0.0; Nyr[3] = VX(vj) - VX(vi);
        Nzl = ((VX(vj) - VX(vi)) * (VY(vl) - VY(vi))) - ((VY(vj) - VY(vi)) * (VX(vl) - VX(vi)));
        Nzr = ((VX(vr) - VX(vi)) * (VY(vj) - VY(vi))) - ((VY(vr) - VY(vi)) * (VX(vj) - VX(vi)));
        for (k = 0; k < 4; k++) {
          Nx[k] = -((Nxl[k] / Nzl) + (Nxr[k] / Nzr)) / 2.0;
          Ny[k] = -((Nyl[k] / Nzl) + (Nyr[k] / Nzr)) / 2.0;
        }
      } else {
        for (iti = 1; iti <= A1(b->niTri, vi); iti++) {
          ti = A2(b->iTri, nV, vi, iti);
          for (n1 = 1; n1 <= 3; n1++) {
            n2 = n1 + 1; if (n2 == 4) n2 = 1;
            n3 = n2 + 1; if (n3 == 4) n3 = 1;
            if ((A2(b->Tri, nTri, ti, n1) == vi && A2(b->Tri, nTri, ti, n2) == vj) ||
                (A2(b->Tri, nTri, ti, n1) == vj && A2(b->Tri, nTri, ti, n2) == vi)) {
              vl = A2(b->Tri, nTri, ti, n3);
            }
          }
        }
        A2(m->Aci, m->nAc, nAc, 1) = vi; A2(m->Aci, m->nAc, nAc, 2) = vj;
        A2(m->Aci, m->nAc, nAc, 3) = vl; A2(m->Aci, m->nAc, nAc, 4) = 1;
        Nxl[0] = VY(vl) - VY(vj); Nxl[1] = VY(vi) - VY(vl); Nxl[2] = VY(vj) - VY(vi); Nxl[3] = 0.0;
        Nyl[0] = VX(vj) - VX(vl); Nyl[1] = VX(vl) - VX(vi); Nyl[2] = VX(vi) - VX(vj); Nyl[3] = 0.0;
        Nzl = ((VX(vj) - VX(vi)) * (VY(vl) - VY(vi))) - ((VY(vj) - VY(vi)) * (VX(vl) - VX(vi)));
        for (k = 0; k < 4; k++) {
          Nx[k] = -Nxl[k] / Nzl;
          Ny[k] = -Nyl[k] / Nzl;
        }
      }
      Ux = VX(vj) - VX(vi);
      Uy = VY(vj) - VY(vi);
      U = sqrt(Ux * Ux + Uy * Uy);
      Np = 1.0 / U;
      for (k = 0; k < 4; k++) No[k] = ((Ny[k] * Ux) - (Nx[k] * Uy)) / U;
      for (k = 0; k < 4; k++) {
        A2(m->Nx_Ac, m->nAc, nAc, k + 1) = Nx[k];
        A2(m->Ny_Ac, m->nAc, nAc, k + 1) = Ny[k];
        A2(m->No_Ac, m->nAc, nAc, k + 1) = No[k];
      }
      A1(m->Np_Ac, nAc) = Np;
#undef VX
#undef VY
    }
  }
  if (nAc != m->nAc) { free(V_vc); return OR_ERR_BAD_MESH; }

  /* == find_Ac_edge_indices (mesh_ArakawaC_module.f90:242-285) == */
  for (int aci = 1; aci <= nAc; aci++) {
    const int ei = A1(b->edge_index, A2(m->Aci, nAc, aci, 1));
    const int ej = A1(b->edge_index, A2(m->Aci, nAc, aci, 2));
#define IN3(e, a, b_, c) ((e) == (a) || (e) == (b_) || (e) == (c))
    if (IN3(ei, 8, 1, 2) && IN3(ej, 8, 1, 2)) A1(m->edge_index_Ac, aci) = 1;
    else if (IN3(ei, 2, 3, 4) && IN3(ej, 2, 3, 4)) A1(m->edge_index_Ac, aci) = 3;
    else if (IN3(ei, 4, 5, 6) && IN3(ej, 4, 5, 6)) A1(m->edge_index_Ac, aci) = 5;
    else if (IN3(ei, 6, 7, 8) && IN3(ej, 6, 7, 8)) A1(m->edge_index_Ac, aci) = 7;
    else A1(m->edge_index_Ac, aci) = 0;
#undef IN3
  }

  /* == make_combined_AaAc_mesh (mesh_ArakawaC_module.f90:286-540) == */
  const int nA = nV + nAc;
  if (m->nVAaAc != nA) { free(V_vc); return OR_ERR_BAD_ARG; }
  memset(m->CAaAc, 0, sizeof(int32_t) * (size_t)nA * nCm);
  for (vi = 1; vi <= nV; vi++) {
    const int ai = vi;
    A2(m->VAaAc, nA, ai, 1) = A2(V, nV, vi, 1);
    A2(m->VAaAc, nA, ai, 2) = A2(V, nV, vi, 2);
    A1(m->nCAaAc, ai) = A1(b->nC, vi);
    for (ci = 1; ci <= A1(b->nC, vi); ci++) A2(m->CAaAc, nA, ai, ci) = A2(m->iAci, nV, vi, ci) + nV;
  }
  for (int aci = 1; aci <= nAc; aci++) {
    const int ai = aci + nV;
    int aci1, aci2, aci3, aci4, vk;
    A2(m->VAaAc, nA, ai, 1) = A2(m->VAc, nAc, aci, 1);
    A2(m->VAaAc, nA, ai, 2) = A2(m->VAc, nAc, aci, 2);
    if (A1(m->edge_index_Ac, aci) > 0) {
      int switchthem = 0;
      vi = A2(m->Aci, nAc, aci, 1);
      vj = A2(m->Aci, nAc, aci, 2);
      const int eac = A1(m->edge_index_Ac, aci);
      if (eac == 1) { if (A2(V, nV, vi, 1) > A2(V, nV, vj, 1)) switchthem = 1; }
      else if (eac == 3) { if (A2(V, nV, vi, 2) < A2(V, nV, vj, 2)) switchthem = 1; }
      else if (eac == 5) { if (A2(V, nV, vi, 1) < A2(V, nV, vj, 1)) switchthem = 1; }
      else if (eac == 7) { if (A2(V, nV, vi, 2) > A2(V, nV, vj, 2)) switchthem = 1; }
      else { free(V_vc); return OR_ERR_BAD_MESH; }
      if (switchthem) { vi = vi + vj; vj = vi - vj; vi = vi - vj; }
      vk = A2(m->Aci, nAc, aci, 3);
      aci1 = 0; aci2 = 0;
      for (ci = 1; ci <= A1(b->nC, vk); ci++) {
        if (A2(b->C, nV, vk, ci) == vi) aci1 = A2(m->iAci, nV, vk, ci);
        else if (A2(b->C, nV, vk, ci) == vj) aci2 = A2(m->iAci, nV, vk, ci);
      }
      if (aci1 == 0 || aci2 == 0) { free(V_vc); return OR_ERR_BAD_MESH; }
      A1(m->nCAaAc, ai) = 4;
      A2(m->CAaAc, nA, ai, 1) = vi;
      A2(m->CAaAc, nA, ai, 2) = aci1 + nV;
      A2(m->CAaAc, nA, ai, 3) = aci2 + nV;
      A2(m->CAaAc, nA, ai, 4) = vj;
    } else {
      vi = A2(m->Aci, nAc, aci, 1);
      vj = A2(m->Aci, nAc, aci, 2);
      vl = A2(m->Aci, nAc, aci, 3);
      vr = A2(m->Aci, nAc, aci, 4);
      aci1 = 0; aci2 = 0; aci3 = 0; aci4 = 0;
      for (ci = 1; ci <= A1(b->nC, vr); ci++) {
        if (A2(b->C, nV, vr, ci) == vi) aci1 = A2(m->iAci, nV, vr, ci);
        else if (A2(b->C, nV, vr, ci) == vj) aci2 = A2(m->iAci, nV, vr, ci);
      }
      for (ci = 1; ci <= A1(b->nC, vl); ci++) {
        if (A2(b->C, nV, vl, ci) == vj) aci3 = A2(m->iAci, nV, vl, ci);
        else if (A2(b->C, nV, vl, ci) == vi) aci4 = A2(m->iAci, nV, vl, ci);
      }
      if (aci1 == 0 || aci2 == 0 || aci3 == 0 || aci4 == 0) { free(V_vc); return OR_ERR_BAD_MESH; }
      A1(m->nCAaAc, ai) = 6;
      A2(m->CAaAc, nA, ai, 1) = vi;
      A2(m->CAaAc, nA, ai, 2) = aci1 + nV;
      A2(m->CAaAc, nA, ai, 3) = aci2 + nV;
      A2(m->CAaAc, nA, ai, 4) = vj;
      A2(m->CAaAc, nA, ai, 5) = aci3 + nV;
      A2(m->CAaAc, nA, ai, 6) = aci4 + nV;
    }
  }
  /* AaAc neighbour functions (mesh_ArakawaC_module.f90:511-538) */
  for (int ai = 1; ai <= nA; ai++) {
    const double V_vi[2] = {A2(m->VAaAc, nA, ai, 1), A2(m->VAaAc, nA, ai, 2)};
    const int n = A1(m->nCAaAc, ai);
    int is_edge;
    for (ci = 1; ci <= n; ci++) {
      const int aj = A2(m->CAaAc, nA, ai, ci);
      A2(V_vc, nCm, ci, 1) = A2(m->VAaAc, nA, aj, 1);
      A2(V_vc, nCm, ci, 2) = A2(m->VAaAc, nA, aj, 2);
    }
    if (ai <= nV) is_edge = A1(b->edge_index, ai) > 0;
    else is_edge = A1(m->edge_index_Ac, ai - nV) > 0;
    nf_row(ai, nA, nCm, V_vi, n, V_vc, is_edge, m->Nx_AaAc, m->Ny_AaAc, m->Nxx_AaAc,
           m->Nxy_AaAc, m->Nyy_AaAc);
  }
  free(V_vc);
  return OR_OK;
}

/* ===================== five-colouring (Williams 1985, as coded) ===================== */

typedef struct colour_ctx {
  jmp_buf jb;
  int nA, nCm;
  int32_t *deg, *L, *Q4, *Q5, *LDP, *S_vi, *S_L, *S_u;
  unsigned char *mark;
  int Q4n, Q5n, Sn, noofvert;
} colour_ctx;

#define FAIL(ctx, code) longjmp((ctx)->jb, (code))
#define LL(ctx, i, j) A2((ctx)->L, (ctx)->nA, i, j)

static int is_in_Q4(colour_ctx *x, int vi) {
  int isso = 0;
  const int qi = A1(x->LDP, vi);
  if (qi == 0) return 0;
  if (A1(x->Q4, qi) == vi) isso = 1;
  if (A1(x->Q5, qi) == vi && isso) FAIL(x, OR_ERR_COLOUR_QUEUE);
  return isso;
}
static int is_in_Q5(colour_ctx *x, int vi) {
  int isso = 0;
  const int qi = A1(x->LDP, vi);
  if (qi == 0) return 0;
  if (A1(x->Q5, qi) == vi) isso = 1;
  if (A1(x->Q4, qi) == vi && isso) FAIL(x, OR_ERR_COLOUR_QUEUE);
  return isso;
}
static void add_to_Q4(colour_ctx *x, int vi) {
  if (A1(x->deg, vi) > 4) FAIL(x, OR_ERR_COLOUR_QUEUE);
  if (A1(x->LDP, vi) > 0) FAIL(x, OR_ERR_COLOUR_QUEUE);
  x->Q4n = x->Q4n + 1;
  A1(x->Q4, x->Q4n) = vi;
  A1(x->LDP, vi) = x->Q4n;
}
static void add_to_Q5(colour_ctx *x, int vi) {
  if (A1(x->deg, vi) != 5) FAIL(x, OR_ERR_COLOUR_QUEUE);
  if (A1(x->LDP, vi) > 0) FAIL(x, OR_ERR_COLOUR_QUEUE);
  x->Q5n = x->Q5n + 1;
  A1(x->Q5, x->Q5n) = vi;
  A1(x->LDP, vi) = x->Q5n;
}
static void remove_from_Q4(colour_ctx *x, int vi) {
  const int qi = A1(x->LDP, vi);
  int qii;
  if (qi == 0) FAIL(x, OR_ERR_COLOUR_QUEUE);
  if (A1(x->Q5, qi) == vi) FAIL(x, OR_ERR_COLOUR_QUEUE);
  if (A1(x->Q4, qi) != vi) FAIL(x, OR_ERR_COLOUR_QUEUE);
  for (qii = qi; qii <= x->Q4n - 1; qii++) A1(x->Q4, qii) = A1(x->Q4, qii + 1);
  A1(x->Q4, x->Q4n) = 0;
  x->Q4n = x->Q4n - 1;
  A1(x->LDP, vi) = 0;
  for (qii = qi; qii <= x->Q4n; qii++) A1(x->LDP, A1(x->Q4, qii)) = qii;
}
static void remove_from_Q5(colour_ctx *x, int vi) {
  const int qi = A1(x->LDP, vi);
  int qii;
  if (qi == 0) FAIL(x, OR_ERR_COLOUR_QUEUE);
  if (A1(x->Q4, qi) == vi) FAIL(x, OR_ERR_COLOUR_QUEUE);
  if (A1(x->Q5, qi) != vi) FAIL(x, OR_ERR_COLOUR_QUEUE);
  for (qii = qi; qii <= x->Q5n - 1; qii++) A1(x->Q5, qii) = A1(x->Q5, qii + 1);
  A1(x->Q5, x->Q5n) = 0;
  x->Q5n = x->Q5n - 1;
  A1(x->LDP, vi) = 0;
  for (qii = qi; qii <= x->Q5n; qii++) A1(x->LDP, A1(x->Q5, qii)) = qii;
}
static void check(colour_ctx *x, int vi) {
  const int d = A1(x->deg, vi);
  if (d <= 4) {
    if (is_in_Q5(x, vi)) remove_from_Q5(x, vi);
    if (!is_in_Q4(x, vi)) add_to_Q4(x, vi);
  } else if (d == 5) {
    if (is_in_Q4(x, vi)) remove_from_Q4(x, vi);
    if (!is_in_Q5(x, vi)) add_to_Q5(x, vi);
  } else {
    if (is_in_Q4(x, vi)) FAIL(x, OR_ERR_COLOUR_QUEUE);
    if (is_in_Q5(x, vi)) remove_from_Q5(x, vi);
  }
}
static void delete_v(colour_ctx *x, int vi) {
  int ci, ci2, wi, k;
  for (ci = 1; ci <= A1(x->deg, vi); ci++) {
    wi = LL(x, vi, ci);
    for (ci2 = 1; ci2 <= A1(x->deg, wi); ci2++) {
      if (LL(x, wi, ci2) == vi) {
        /* L(wi, ci2:deg-1) = L(wi, ci2+1:deg) */
        for (k = ci2; k <= A1(x->deg, wi) - 1; k++) LL(x, wi, k) = LL(x, wi, k + 1);
        LL(x, wi, A1(x->deg, wi)) = 0;
        A1(x->deg, wi) = A1(x->deg, wi) - 1;
        check(x, wi);
        break;
      }
    }
  }
  x->Sn = x->Sn + 1;
  A1(x->S_vi, x->Sn) = vi;
  for (k = 1; k <= x->nCm; k++) A2(x->S_L, x->nA, x->Sn, k) = LL(x, vi, k);
  if (A1(x->deg, vi) <= 4) remove_from_Q4(x, vi);
  else if (A1(x->deg, vi) == 5) remove_from_Q5(x, vi);
  else FAIL(x, OR_ERR_COLOUR_QUEUE);
  x->noofvert = x->noofvert - 1;
}

static void reduce(colour_ctx *x, int32_t *iters) {
  int vi, ci1, ci2, ci3, xi = 0, yi = 0, it = 0, qii;
  const int k = x->nCm; /* k = C%nconmax */
  while (x->noofvert > 5) {
    it = it + 1;
    if (iters) *iters = it;
    if (it > x->nA * 2) FAIL(x, OR_ERR_COLOUR_STUCK);
    if (x->Q4n > 0) {
      vi = A1(x->Q4, x->Q4n);
      delete_v(x, vi);
    } else {
      int found_pair = 0;
      vi = A1(x->Q5, x->Q5n);
      for (ci1 = 1; ci1 <= A1(x->deg, vi); ci1++) {
        xi = LL(x, vi, ci1);
        for (ci2 = ci1 + 1; ci2 <= A1(x->deg, vi); ci2++) {
          int adj = 0;
          yi = LL(x, vi, ci2);
          for (ci3 = 1; ci3 <= A1(x->deg, yi); ci3++) {
            if (LL(x, yi, ci3) == xi) { adj = 1; break; }
          }
          if (adj) continue;
          if (A1(x->deg, xi) < k && A1(x->deg, yi) < k) { found_pair = 1; break; }
        }
        if (found_pair) break;
      }
      if (found_pair) {
        /* delete(v) then identify(x,y): the reference's identify ends in an
         * unconditional MPI_ABORT (mesh_five_colour_module.f90:452), so the run
         * stops here. */
        FAIL(x, OR_ERR_COLOUR_IDENTIFY);
      } else {
        /* Return v to the rear of Q5: Q5(2:Q5n) = Q5(1:Q5n-1); Q5(1) = vi */
        for (qii = x->Q5n; qii >= 2; qii--) A1(x->Q5, qii) = A1(x->Q5, qii - 1);
        A1(x->Q5, 1) = vi;
        for (qii = 1; qii <= x->Q5n; qii++) A1(x->LDP, A1(x->Q5, qii)) = qii;
      }
    }
  }
}

static void colour_pass(colour_ctx *x, int32_t *colour) {
  int vi, ui, col, ci, it = 0;
  A1(colour, A1(x->Q4, 1)) = 1;
  A1(colour, A1(x->Q4, 2)) = 2;
  A1(colour, A1(x->Q4, 3)) = 3;
  A1(colour, A1(x->Q4, 4)) = 4;
  A1(colour, A1(x->Q4, 5)) = 5;
  while (x->Sn > 0) {
    it = it + 1;
    if (it > x->nA * 2) FAIL(x, OR_ERR_COLOUR_STUCK);
    vi = A1(x->S_vi, x->Sn);
    ui = A1(x->S_u, x->Sn);
    if (A1(x->S_u, x->Sn) > 0) {
      A1(colour, ui) = A1(colour, vi);
    } else {
      int L_colours[5] = {0, 0, 0, 0, 0};
      for (ci = 1; ci <= x->nCm; ci++) {
        ui = A2(x->S_L, x->nA, x->Sn, ci);
        if (ui == 0) break;
        col = A1(colour, ui);
        if (col == 0) continue;
        L_colours[col - 1] = 1;
      }
      if (L_colours[0] + L_colours[1] + L_colours[2] + L_colours[3] + L_colours[4] > 4)
        FAIL(x, OR_ERR_COLOUR_STUCK);
      for (ci = 1; ci <= 5; ci++) {
        if (L_colours[ci - 1] == 0) { A1(colour, vi) = ci; break; }
      }
    }
    x->Sn = x->Sn - 1;
  }
}

int or_five_colouring(const or_base *b, or_aaac *m, int32_t *reduce_iterations) {
  colour_ctx x;
  const int nA = m->nVAaAc, nCm = b->nC_mem;
  int rc, vi, ci;
  memset(&x, 0, sizeof(x));
  x.nA = nA;
  x.nCm = nCm;
  x.deg = (int32_t *)calloc((size_t)nA, sizeof(int32_t));
  x.L = (int32_t *)calloc((size_t)nA * nCm, sizeof(int32_t));
  x.Q4 = (int32_t *)calloc((size_t)nA, sizeof(int32_t));
  x.Q5 = (int32_t *)calloc((size_t)nA, sizeof(int32_t));
  x.LDP = (int32_t *)calloc((size_t)nA, sizeof(int32_t));
  x.mark = (unsigned char *)calloc((size_t)nA, 1);
  x.S_vi = (int32_t *)calloc((size_t)nA, sizeof(int32_t));
  x.S_L = (int32_t *)calloc((size_t)nA * nCm, sizeof(int32_t));
  x.S_u = (int32_t *)calloc((size_t)nA, sizeof(int32_t));
  if (!x.deg || !x.L || !x.Q4 || !x.Q5 || !x.LDP || !x.mark || !x.S_vi || !x.S_L || !x.S_u) {
    rc = OR_ERR_BAD_ARG;
    goto done;
  }
  memcpy(x.deg, m->nCAaAc, sizeof(int32_t) * (size_t)nA);
  memcpy(x.L, m->CAaAc, sizeof(int32_t) * (size_t)nA * nCm);
  x.noofvert = nA;
  /* Fresh shared windows read as zero: colour starts at 0 everywhere. */
  memset(m->colour, 0, sizeof(int32_t) * (size_t)nA);
  if (reduce_iterations) *reduce_iterations = 0;

  rc = setjmp(x.jb);
  if (rc != 0) goto done;

  for (vi = 1; vi <= nA; vi++) {
    if (A1(x.deg, vi) <= 4) add_to_Q4(&x, vi);
    else if (A1(x.deg, vi) == 5) add_to_Q5(&x, vi);
  }
  reduce(&x, reduce_iterations);
  colour_pass(&x, m->colour);

  /* check_solution (mesh_five_colour_module.f90:318-343) */
  for (vi = 1; vi <= nA; vi++) {
    if (A1(m->colour, vi) == 0) FAIL(&x, OR_ERR_COLOUR_INVALID);
    for (ci = 1; ci <= A1(m->nCAaAc, vi); ci++) {
      const int vj = A2(m->CAaAc, nA, vi, ci);
      if (A1(m->colour, vi) == A1(m->colour, vj)) FAIL(&x, OR_ERR_COLOUR_INVALID);
    }
  }
  /* Same-coloured domains, ascending vi within each colour */
  memset(m->colour_vi, 0, sizeof(int32_t) * (size_t)nA * 5);
  for (ci = 1; ci <= 5; ci++) A1(m->colour_nV, ci) = 0;
  for (vi = 1; vi <= nA; vi++) {
    ci = A1(m->colour, vi);
    A1(m->colour_nV, ci) = A1(m->colour_nV, ci) + 1;
    A2(m->colour_vi, nA, A1(m->colour_nV, ci), ci) = vi;
  }
  rc = OR_OK;
done:
  free(x.deg); free(x.L); free(x.Q4); free(x.Q5); free(x.LDP); free(x.mark);
  free(x.S_vi); free(x.S_L); free(x.S_u);
  return rc;
}
