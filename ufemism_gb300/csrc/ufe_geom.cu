// Geometry preparation on the device: the part of update_general_ice_model_data
// (general_ice_model_data_module.f90:23-96) that the velocity solve reads — the Aa-to-Ac maps
// of Hi, Hb, SL (map_Aa_to_Ac, mesh_ArakawaC_module.f90:726-747), the surface Hs, the
// ocean / ice / sheet / shelf masks on Aa and Ac and the grounding-line mask on Ac
// (determine_masks, 97-297), the Aa slopes of Hi and Hs (get_mesh_derivatives,
// mesh_derivatives_module.f90:315-371), the Ac slopes of Hi, Hb, Hs, SL
// (get_mesh_derivatives_Ac, mesh_ArakawaC_module.f90:542-581) and the shelf-slope rule
// (general_ice_model_data_module.f90:70-87). Same expression order as the reference and
// built without FMA contraction, so the fields are bit-identical to its.
//
// With it a time step uploads Hi, Hb, SL (and the flow factor) instead of about twenty
// derived fields, and the solve's inputs are born on the device.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <vector>

#include "ufe_internal.h"

namespace ufe {

struct GeomWork {
  int nV = 0, nAc = 0, ncm = 0;
  // stencils
  int *nC = nullptr, *C = nullptr, *Aci = nullptr;
  double *Nx = nullptr, *Ny = nullptr, *Nx_Ac = nullptr, *Ny_Ac = nullptr, *No_Ac = nullptr, *Np_Ac = nullptr;
  // fields (see GeomFields)
  double *dbl = nullptr;
  int *msk = nullptr;
  double *beta = nullptr;      // (nV + nAc), allocated on first use
  double *thk = nullptr;       // thickness-update work, allocated on first use
  int *thk_int = nullptr;
  double *sia3d = nullptr;     // 3-D SIA work (A_flow, dHb_dt, U, V, W), allocated on first use
  int sia3d_nZ = 0;
  // ice physical properties: Ti, A_flow, Ti_pmp, Cpi, Ki (nV x nZ each), A_flow_Ac, Ti_Ac (nAc x nZ each)
  double *props = nullptr;
  int props_nZ = 0;
  int props_law = -1;          // flow law of the last ufe_ice_physical_properties, -1: none
  bool af_set = false;         // A_flow_mean(_Ac) present on the device (physical properties or an upload)
  bool sia3d_done = false;     // U_3D, V_3D, W_3D of a successful ufe_sia3d_solve in sia3d
  // triangles (ufe_triangles_attach) and the upwind-derivative work
  int nTri = 0;
  double *tV = nullptr, *tR = nullptr, *NxTri = nullptr, *NyTri = nullptr;
  int *niTri = nullptr, *iTri = nullptr, *Tri = nullptr;
  double *upw = nullptr;       // U, V, d in; ddx, ddy out (nV x nZ each)
  int upw_nZ = 0;
  unsigned long long *upw_missing = nullptr;
  // determine_masks in full: one 16-bit word per Aa vertex then per Ac edge (mask bits and
  // the type mask), and a staging array for handing single masks back
  unsigned short *pk = nullptr;
  int *mask_stage = nullptr;
  bool computed = false;
};

void geom_free(GeomWork *w) {
  if (!w) return;
  void *ptrs[] = {w->nC, w->C, w->Aci, w->Nx, w->Ny, w->Nx_Ac, w->Ny_Ac, w->No_Ac, w->Np_Ac, w->dbl, w->msk, w->beta, w->thk, w->thk_int, w->sia3d, w->props,
                   w->tV, w->tR, w->NxTri, w->NyTri, w->niTri, w->iTri, w->Tri, w->upw, w->upw_missing, w->pk,
                   w->mask_stage};
  for (void *p : ptrs)
    if (p) cudaFree(p);
  delete w;
}

namespace {

// Double fields: Aa (nV each) then Ac (nAc each), in the order of the enums.
enum AaD { A_HI, A_HB, A_SL, A_HS, A_AF, A_DHI_DX, A_DHI_DY, A_DHS_DX, A_DHS_DY, A_DHS_DX_SH, A_DHS_DY_SH, A_COUNT };
enum AcD {
  C_HI, C_HB, C_SL, C_HS, C_AF,
  C_DHI_DX, C_DHI_DY, C_DHI_DP, C_DHI_DO, C_DHB_DX, C_DHB_DY, C_DHB_DP, C_DHB_DO,
  C_DHS_DX, C_DHS_DY, C_DHS_DP, C_DHS_DO, C_DSL_DX, C_DSL_DY, C_DSL_DP, C_DSL_DO,
  C_DHS_DX_SH, C_DHS_DY_SH, C_COUNT
};
// Integer masks: Aa ocean, ice, sheet, shelf (nV each), then Ac ocean, ice, sheet, shelf, gl.
enum AaM { M_OCEAN, M_ICE, M_SHEET, M_SHELF, M_COUNT };
enum AcM { MC_OCEAN, MC_ICE, MC_SHEET, MC_SHELF, MC_GL, MC_COUNT };

struct GeomArgs {
  int nV, nAc, ncm;
  const int *nC, *C, *Aci;
  const double *Nx, *Ny, *Nx_Ac, *Ny_Ac, *No_Ac, *Np_Ac;
  double *aa, *ac;     // field bases
  int *ma, *mc;
};

__device__ __forceinline__ bool floating(double Hi, double Hb, double SL) {
  return Hi < ((SL - Hb) * kSeawaterDensity) / kIceDensity;   // is_floating, general_ice_model_data_module.f90:464-475
}

#define AAF(a, k) ((a).aa + (size_t)(k) * (a).nV)
#define ACF(a, k) ((a).ac + (size_t)(k) * (a).nAc)
#define AAM(a, k) ((a).ma + (size_t)(k) * (a).nV)
#define ACM(a, k) ((a).mc + (size_t)(k) * (a).nAc)

// Hs and the Aa masks (general_ice_model_data_module.f90:45-47, determine_masks 136-160).
__global__ void k_geom_aa1(const GeomArgs a) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= a.nV) return;
  const double Hi = AAF(a, A_HI)[v], Hb = AAF(a, A_HB)[v], SL = AAF(a, A_SL)[v];
  AAF(a, A_HS)[v] = Hi + fmax(SL - kIceDensity / kSeawaterDensity * Hi, Hb);
  const int ocean = floating(Hi, Hb, SL);
  const int ice = Hi > 0.0;
  AAM(a, M_OCEAN)[v] = ocean;
  AAM(a, M_ICE)[v] = ice;
  AAM(a, M_SHEET)[v] = ice && !ocean;
  AAM(a, M_SHELF)[v] = ice && ocean;
}

// Ac maps, Hs_Ac and the Ac masks (map_Aa_to_Ac; determine_masks 207-235 and the grounding
// line of 236-297: a sheet vertex on one end and a shelf vertex on the other).
__global__ void k_geom_ac1(const GeomArgs a) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= a.nAc) return;
  const int vi = a.Aci[c] - 1, vj = a.Aci[c + a.nAc] - 1;
  const double Hi = (AAF(a, A_HI)[vi] + AAF(a, A_HI)[vj]) / 2.0;
  const double Hb = (AAF(a, A_HB)[vi] + AAF(a, A_HB)[vj]) / 2.0;
  const double SL = (AAF(a, A_SL)[vi] + AAF(a, A_SL)[vj]) / 2.0;
  ACF(a, C_HI)[c] = Hi;
  ACF(a, C_HB)[c] = Hb;
  ACF(a, C_SL)[c] = SL;
  ACF(a, C_HS)[c] = Hi + fmax(SL - kIceDensity / kSeawaterDensity * Hi, Hb);
  const int ocean = floating(Hi, Hb, SL);
  const int ice = Hi > 0.0;
  ACM(a, MC_OCEAN)[c] = ocean;
  ACM(a, MC_ICE)[c] = ice;
  ACM(a, MC_SHEET)[c] = ice && !ocean;
  ACM(a, MC_SHELF)[c] = ice && ocean;
  const int *sheet = AAM(a, M_SHEET), *shelf = AAM(a, M_SHELF);
  ACM(a, MC_GL)[c] = (sheet[vi] == 1 && shelf[vj] == 1) || (sheet[vj] == 1 && shelf[vi] == 1);
}

// Aa slopes of Hi and Hs (home term first, then the neighbours in C order) and the shelf rule.
__global__ void k_geom_aa2(const GeomArgs a) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= a.nV) return;
  const int n = a.nC[v];
  const double *Hi = AAF(a, A_HI), *Hs = AAF(a, A_HS);
  const size_t ld = a.nV;
  double ix = a.Nx[v + n * ld] * Hi[v], iy = a.Ny[v + n * ld] * Hi[v];
  double sx = a.Nx[v + n * ld] * Hs[v], sy = a.Ny[v + n * ld] * Hs[v];
  for (int c = 0; c < n; ++c) {
    const int j = a.C[v + c * ld] - 1;
    const double nx = a.Nx[v + c * ld], ny = a.Ny[v + c * ld];
    ix = ix + nx * Hi[j];
    iy = iy + ny * Hi[j];
    sx = sx + nx * Hs[j];
    sy = sy + ny * Hs[j];
  }
  AAF(a, A_DHI_DX)[v] = ix; AAF(a, A_DHI_DY)[v] = iy;
  AAF(a, A_DHS_DX)[v] = sx; AAF(a, A_DHS_DY)[v] = sy;
  if (AAM(a, M_OCEAN)[v] == 0) {
    AAF(a, A_DHS_DX_SH)[v] = sx;
    AAF(a, A_DHS_DY_SH)[v] = sy;
  } else {
    AAF(a, A_DHS_DX_SH)[v] = (1.0 - kIceDensity / kSeawaterDensity) * ix;
    AAF(a, A_DHS_DY_SH)[v] = (1.0 - kIceDensity / kSeawaterDensity) * iy;
  }
}

// Ac slopes of Hi, Hb, Hs, SL (4-point stencil in Aci order; p along the edge) and the shelf rule.
__global__ void k_geom_ac2(const GeomArgs a) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= a.nAc) return;
  const size_t ld = a.nAc;
  int idx[4];
  for (int k = 0; k < 4; ++k) idx[k] = a.Aci[c + k * ld] - 1;
  const double *src[4] = {AAF(a, A_HI), AAF(a, A_HB), AAF(a, A_HS), AAF(a, A_SL)};
  const int dst[4] = {C_DHI_DX, C_DHB_DX, C_DHS_DX, C_DSL_DX};
  const double np = a.Np_Ac[c];
  for (int f = 0; f < 4; ++f) {
    const double *d = src[f];
    double dx = 0.0, dy = 0.0, dO = 0.0;
    for (int k = 0; k < 4; ++k) {
      const double dv = d[idx[k]];
      dx = dx + a.Nx_Ac[c + k * ld] * dv;
      dy = dy + a.Ny_Ac[c + k * ld] * dv;
      dO = dO + a.No_Ac[c + k * ld] * dv;
    }
    ACF(a, dst[f])[c] = dx;
    ACF(a, dst[f] + 1)[c] = dy;
    ACF(a, dst[f] + 2)[c] = np * (d[idx[1]] - d[idx[0]]);
    ACF(a, dst[f] + 3)[c] = dO;
  }
  if (ACM(a, MC_OCEAN)[c] == 0) {
    ACF(a, C_DHS_DX_SH)[c] = ACF(a, C_DHS_DX)[c];
    ACF(a, C_DHS_DY_SH)[c] = ACF(a, C_DHS_DY)[c];
  } else {
    ACF(a, C_DHS_DX_SH)[c] = (1.0 - kIceDensity / kSeawaterDensity) * ACF(a, C_DHI_DX)[c];
    ACF(a, C_DHS_DY_SH)[c] = (1.0 - kIceDensity / kSeawaterDensity) * ACF(a, C_DHI_DY)[c];
  }
}

// ---------------------------------------------------------------------------------------
// determine_masks in full (general_ice_model_data_module.f90:97-297). Every mask of a vertex
// or edge is one bit of a 16-bit word, the type mask (the last type the routine assigns, in
// its order) in the top four bits. The Aa pass reads the neighbours' ocean / ice / sheet /
// shelf masks that k_geom_aa1 wrote (the reference's first loop, 146-167, completes before
// the neighbour loop, 171-225, reads it); the Ac pass reads its own maps and the two end
// vertices' masks (230-294). mask_lake is never set by the routine and stays 0.
// ---------------------------------------------------------------------------------------
enum MaskBit : int {
  kMkLand = 0, kMkOcean, kMkLake, kMkIce, kMkSheet, kMkShelf, kMkCoast, kMkMargin, kMkGl, kMkCf, kMkBits
};
enum MaskType : int {
  kTypeLand = 0, kTypeOcean = 1, kTypeLake = 2, kTypeSheet = 3, kTypeShelf = 4, kTypeCoast = 5, kTypeMargin = 6,
  kTypeGl = 7, kTypeCf = 8
};
constexpr int kTypeShift = 12;

__device__ __forceinline__ unsigned short mask_word(unsigned bits, int type) {
  return (unsigned short)(bits | ((unsigned)type << kTypeShift));
}

__global__ void k_masks_aa(const GeomArgs a, unsigned short *pk) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= a.nV) return;
  const int *ocean = AAM(a, M_OCEAN), *ice = AAM(a, M_ICE), *sheet = AAM(a, M_SHEET), *shelf = AAM(a, M_SHELF);
  const int o = ocean[v], i = ice[v], sh = sheet[v], sf = shelf[v];
  const int land = !o;
  int type = kTypeLand;
  unsigned bits = (land << kMkLand) | (o << kMkOcean) | (i << kMkIce) | (sh << kMkSheet) | (sf << kMkShelf);
  if (o) type = kTypeOcean;
  if (sh) type = kTypeSheet;
  if (sf) type = kTypeShelf;
  // neighbour conditions, each over all neighbours, in the routine's order
  int coast = 0, margin = 0, gl = 0, cf = 0;
  const int n = a.nC[v];
  const size_t ld = a.nV;
  for (int c = 0; c < n; ++c) {
    const int j = a.C[v + c * ld] - 1;
    const int oj = ocean[j];
    coast |= land & oj;
    margin |= i & (ice[j] == 0);
    gl |= sh & shelf[j];
    cf |= i & oj;
  }
  if (coast) type = kTypeCoast;
  if (margin) type = kTypeMargin;
  if (gl) type = kTypeGl;
  if (cf) type = kTypeCf;
  bits |= (coast << kMkCoast) | (margin << kMkMargin) | (gl << kMkGl) | (cf << kMkCf);
  pk[v] = mask_word(bits, type);
}

__global__ void k_masks_ac(const GeomArgs a, unsigned short *pk) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= a.nAc) return;
  const int o = ACM(a, MC_OCEAN)[c], i = ACM(a, MC_ICE)[c], sh = ACM(a, MC_SHEET)[c], sf = ACM(a, MC_SHELF)[c];
  const int land = !o;
  int type = kTypeLand;
  unsigned bits = (land << kMkLand) | (o << kMkOcean) | (i << kMkIce) | (sh << kMkSheet) | (sf << kMkShelf);
  if (o) type = kTypeOcean;
  if (sh) type = kTypeSheet;
  if (sf) type = kTypeShelf;
  const int vi = a.Aci[c] - 1, vj = a.Aci[c + a.nAc] - 1;
  const unsigned wi = pk[vi], wj = pk[vj];
  auto bit = [](unsigned w, int k) { return (int)((w >> k) & 1u); };
  const int coast = (bit(wi, kMkLand) && bit(wj, kMkOcean)) || (bit(wj, kMkLand) && bit(wi, kMkOcean));
  const int margin = (bit(wi, kMkIce) && !bit(wj, kMkIce)) || (bit(wj, kMkIce) && !bit(wi, kMkIce));
  const int gl = (bit(wi, kMkSheet) && bit(wj, kMkShelf)) || (bit(wj, kMkSheet) && bit(wi, kMkShelf));
  const int cf = (bit(wi, kMkIce) && !bit(wj, kMkShelf) && bit(wj, kMkOcean)) ||
                 (bit(wj, kMkIce) && !bit(wi, kMkShelf) && bit(wi, kMkOcean));
  if (coast) type = kTypeCoast;
  if (margin) type = kTypeMargin;
  if (gl) type = kTypeGl;
  if (cf) type = kTypeCf;
  bits |= (coast << kMkCoast) | (margin << kMkMargin) | (gl << kMkGl) | (cf << kMkCf);
  pk[a.nV + c] = mask_word(bits, type);
}

// One mask (bit k, or the type for k = kMkBits) of n words as the reference's INTEGER array.
__global__ void k_mask_unpack(int n, const unsigned short *pk, int k, int *out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const unsigned w = pk[i];
  out[i] = k == kMkBits ? (int)(w >> kTypeShift) : (int)((w >> k) & 1u);
}

GeomArgs args_of(GeomWork *w) {
  GeomArgs a;
  a.nV = w->nV; a.nAc = w->nAc; a.ncm = w->ncm;
  a.nC = w->nC; a.C = w->C; a.Aci = w->Aci; a.Nx = w->Nx; a.Ny = w->Ny;
  a.Nx_Ac = w->Nx_Ac; a.Ny_Ac = w->Ny_Ac; a.No_Ac = w->No_Ac; a.Np_Ac = w->Np_Ac;
  a.aa = w->dbl; a.ac = w->dbl + (size_t)A_COUNT * w->nV;
  a.ma = w->msk; a.mc = w->msk + (size_t)M_COUNT * w->nV;
  return a;
}

template <class T>
int up(T *dst, const T *src, size_t n, cudaStream_t s) {
  return cuda_status(cudaMemcpyAsync(dst, src, n * sizeof(T), cudaMemcpyHostToDevice, s), "geometry H2D");
}

// Upload Hi, Hb, SL and compute every derived field on the handle's stream.
int compute(ufe_mesh_h h, const double *Hi, const double *Hb, const double *SL) {
  GeomWork *w = h->geom;
  cudaStream_t s = h->stream;
  GeomArgs a = args_of(w);
  const size_t nV = w->nV;
  int rc = up(AAF(a, A_HI), Hi, nV, s);
  if (!rc) rc = up(AAF(a, A_HB), Hb, nV, s);
  if (!rc) rc = up(AAF(a, A_SL), SL, nV, s);
  const unsigned gv = (unsigned)((w->nV + 255) / 256), gc = (unsigned)((w->nAc + 255) / 256);
  if (!rc) { k_geom_aa1<<<gv, 256, 0, s>>>(a); rc = cuda_status(cudaGetLastError(), "k_geom_aa1"); }
  if (!rc) { k_geom_ac1<<<gc, 256, 0, s>>>(a); rc = cuda_status(cudaGetLastError(), "k_geom_ac1"); }
  if (!rc) { k_geom_aa2<<<gv, 256, 0, s>>>(a); rc = cuda_status(cudaGetLastError(), "k_geom_aa2"); }
  if (!rc) { k_geom_ac2<<<gc, 256, 0, s>>>(a); rc = cuda_status(cudaGetLastError(), "k_geom_ac2"); }
  if (!rc) { k_masks_aa<<<gv, 256, 0, s>>>(a, w->pk); rc = cuda_status(cudaGetLastError(), "k_masks_aa"); }
  if (!rc) { k_masks_ac<<<gc, 256, 0, s>>>(a, w->pk); rc = cuda_status(cudaGetLastError(), "k_masks_ac"); }
  w->computed = rc == UFE_OK;
  return rc;
}

// ---------------------------------------------------------------------------------------
// ice_physical_properties (general_ice_model_data_module.f90:298-462): the flow factor, the
// pressure-melting point, the specific heat and the conductivity of the ice, one thread per
// Aa vertex and one per Ac edge, each walking its nZ layers (column-major, so every layer is
// a coalesced row across the warp). Constants from parameters_module.f90:10-21 and the
// routine's own Arrhenius constants (318-322).
// ---------------------------------------------------------------------------------------
constexpr int kMaxZP = 64;
constexpr double kT0 = 273.16, kCC = 8.7E-04, kSMT = 271.15, kSecPerYear = 31556943.36;
constexpr double kALow = 1.14E-05, kAHigh = 5.47E+10, kQLow = 6.0E+04, kQHigh = 13.9E+04, kRGas = 8.314;

struct PropArgs {
  int nV, nAc, nZ, law;
  double A_const;                     // the benchmark laws' flow factor
  const int *Aci;                     // (nAc, 4), 1-based
  const double *Hi;                   // (nV)
  const int *mask_sheet, *mask_sheet_Ac;
  const double *Ti;                   // (nV, nZ)
  double *A_flow, *Ti_pmp, *Cpi, *Ki, *A_mean;   // Aa
  double *A_flow_Ac, *Ti_Ac, *A_mean_Ac;         // Ac
  double zeta[kMaxZP];
};

__device__ __forceinline__ double arrhenius(double T) {
  return T < 263.15 ? kALow * exp(-kQLow / (kRGas * T)) : kAHigh * exp(-kQHigh / (kRGas * T));
}

__global__ void k_physprop_aa(const PropArgs a) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= a.nV) return;
  const size_t n = a.nV;
  const double H = a.Hi[v];
  if (a.law != UFE_FLOW_ARRHENIUS) {
    for (int k = 0; k < a.nZ; ++k) a.A_flow[v + k * n] = a.A_const;
    a.A_mean[v] = a.A_const;
    if (a.law == UFE_FLOW_EISMINT)
      for (int k = 0; k < a.nZ; ++k) {
        a.Ki[v + k * n] = 2.1 * kSecPerYear;
        a.Cpi[v + k * n] = 2009.0;
        a.Ti_pmp[v + k * n] = kT0 - (a.zeta[k] * H * 8.7E-04);
      }
    return;
  }
  // the vertical average (zeta_module.f90:33-57) accumulates layer by layer, base upwards
  double avg = 0.0, below = 0.0;
  for (int k = 0; k < a.nZ; ++k) {
    const double T = a.Ti[v + k * n];
    a.Ti_pmp[v + k * n] = kT0 - kCC * H * a.zeta[k];
    const double A = arrhenius(T);
    a.A_flow[v + k * n] = A;
    a.Cpi[v + k * n] = 2115.3 + 7.79293 * (T - kT0);
    a.Ki[v + k * n] = 3.101E+08 * exp(-0.0057 * T);
    if (k > 0) avg = avg + 0.5 * (A + below) * (a.zeta[k] - a.zeta[k - 1]);
    below = A;
  }
  a.A_mean[v] = a.mask_sheet[v] == 1 ? avg : arrhenius((a.Ti[v] + kSMT) / 2.0);
}

__global__ void k_physprop_ac(const PropArgs a) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= a.nAc) return;
  const size_t n = a.nAc, nv = a.nV;
  if (a.law != UFE_FLOW_ARRHENIUS) {
    for (int k = 0; k < a.nZ; ++k) a.A_flow_Ac[c + k * n] = a.A_const;
    a.A_mean_Ac[c] = a.A_const;
    return;
  }
  const int vi = a.Aci[c] - 1, vj = a.Aci[c + n] - 1;
  double avg = 0.0, below = 0.0, T1 = 0.0;
  for (int k = 0; k < a.nZ; ++k) {
    const double T = (a.Ti[vi + k * nv] + a.Ti[vj + k * nv]) / 2.0;   // map_Aa_to_Ac_3D
    a.Ti_Ac[c + k * n] = T;
    if (k == 0) T1 = T;
    const double A = arrhenius(T);
    a.A_flow_Ac[c + k * n] = A;
    if (k > 0) avg = avg + 0.5 * (A + below) * (a.zeta[k] - a.zeta[k - 1]);
    below = A;
  }
  a.A_mean_Ac[c] = a.mask_sheet_Ac[c] == 1 ? avg : arrhenius((T1 + kSMT) / 2.0);
}

// Device copies of the last physical properties, or null when none match this nZ.
const double *props_A_flow(const GeomWork *w, const ufe_params *p) {
  return (w->props_law >= 0 && w->props_nZ == p->nZ) ? w->props + (size_t)w->nV * w->props_nZ : nullptr;
}
const double *props_A_flow_Ac(const GeomWork *w, const ufe_params *p) {
  return (w->props_law >= 0 && w->props_nZ == p->nZ) ? w->props + 5 * (size_t)w->nV * w->props_nZ : nullptr;
}

}  // namespace
}  // namespace ufe

using namespace ufe;

extern "C" int ufe_ice_physical_properties(ufe_mesh_h h, const ufe_params *p, int flow_law, double time,
                                           const double *Ti, ufe_physprop_out *out) {
  if (!h || !p || !p->zeta) { set_error("ufe_ice_physical_properties: null argument"); return UFE_BAD_ARG; }
  if (flow_law < UFE_FLOW_ARRHENIUS || flow_law > UFE_FLOW_MISMIP_MOD) {
    set_error("ufe_ice_physical_properties: unknown flow law");
    return UFE_BAD_ARG;
  }
  if (flow_law == UFE_FLOW_ARRHENIUS && !Ti) { set_error("ufe_ice_physical_properties: Ti is required"); return UFE_BAD_ARG; }
  if (p->nZ < 2 || p->nZ > kMaxZP) { set_error("ufe_ice_physical_properties: nZ must be in [2, 64]"); return UFE_BAD_ARG; }
  if (!h->geom || !h->geom->computed) {
    set_error("ufe_ice_physical_properties: no device geometry (ufe_geometry_update or ufe_ssa_upload_geometry first)");
    return UFE_BAD_ARG;
  }
  GeomWork *w = h->geom;
  const size_t nV = w->nV, nAc = w->nAc, nZ = p->nZ;
  cudaStream_t s = h->stream;
  int rc = UFE_OK;
  if (w->props_nZ != (int)nZ) {
    if (w->props) { cudaFree(w->props); w->props = nullptr; }
    w->props_nZ = 0;
    w->props_law = -1;
    rc = cuda_status(cudaMalloc(&w->props, (5 * nV + 2 * nAc) * nZ * sizeof(double)), "physical properties");
    if (rc) return rc;
    w->props_nZ = (int)nZ;
  }
  GeomArgs ga = args_of(w);
  PropArgs a;
  a.nV = (int)nV; a.nAc = (int)nAc; a.nZ = (int)nZ; a.law = flow_law;
  a.A_const = 1.0E-16;
  if (flow_law == UFE_FLOW_MISMIP_MOD && time >= 25000.0 && time < 50000.0) a.A_const = 1.0E-17;
  a.Aci = w->Aci; a.Hi = AAF(ga, A_HI); a.mask_sheet = AAM(ga, M_SHEET); a.mask_sheet_Ac = ACM(ga, MC_SHEET);
  double *Ti_d = w->props;
  a.Ti = Ti_d;
  a.A_flow = Ti_d + nV * nZ; a.Ti_pmp = a.A_flow + nV * nZ; a.Cpi = a.Ti_pmp + nV * nZ; a.Ki = a.Cpi + nV * nZ;
  a.A_flow_Ac = a.Ki + nV * nZ; a.Ti_Ac = a.A_flow_Ac + nAc * nZ;
  a.A_mean = AAF(ga, A_AF); a.A_mean_Ac = ACF(ga, C_AF);
  for (size_t k = 0; k < nZ; ++k) a.zeta[k] = p->zeta[k];
  if (flow_law == UFE_FLOW_ARRHENIUS) rc = up(Ti_d, Ti, nV * nZ, s);
  if (!rc) { k_physprop_aa<<<(unsigned)((nV + 127) / 128), 128, 0, s>>>(a); rc = cuda_status(cudaGetLastError(), "k_physprop_aa"); }
  if (!rc) { k_physprop_ac<<<(unsigned)((nAc + 127) / 128), 128, 0, s>>>(a); rc = cuda_status(cudaGetLastError(), "k_physprop_ac"); }
  // the A fields stay valid on the device whatever the copies back do
  if (!rc) { w->props_law = flow_law; w->af_set = true; }
  if (out) {
    auto dn = [&](double *dst, const double *src, size_t n) {
      if (!dst || rc) return;
      rc = cuda_status(cudaMemcpyAsync(dst, src, n * sizeof(double), cudaMemcpyDeviceToHost, s), "physical properties D2H");
    };
    dn(out->A_flow, a.A_flow, nV * nZ);
    dn(out->A_flow_mean, a.A_mean, nV);
    dn(out->A_flow_Ac, a.A_flow_Ac, nAc * nZ);
    dn(out->A_flow_mean_Ac, a.A_mean_Ac, nAc);
    if (flow_law != UFE_FLOW_MISMIP_MOD) {
      dn(out->Ti_pmp, a.Ti_pmp, nV * nZ);
      dn(out->Cpi, a.Cpi, nV * nZ);
      dn(out->Ki, a.Ki, nV * nZ);
    }
    if (flow_law == UFE_FLOW_ARRHENIUS) dn(out->Ti_Ac, a.Ti_Ac, nAc * nZ);
  }
  if (!rc) rc = cuda_status(cudaStreamSynchronize(s), "physical properties");
  return rc;
}

extern "C" int ufe_geometry_attach(ufe_mesh_h h, const ufe_geometry_mesh *g) {
  if (!h || !g || !g->nC || !g->C || !g->Nx || !g->Ny || !g->Aci || !g->Nx_Ac || !g->Ny_Ac || !g->No_Ac || !g->Np_Ac) {
    set_error("ufe_geometry_attach: missing array");
    return UFE_BAD_ARG;
  }
  const DevMesh &m = h->m;
  const int nV = m.nV, nAc = m.nAc, ncm = m.ncm;
  // validate the index arrays on the host before any kernel reads them
  for (int v = 0; v < nV; ++v) {
    if (g->nC[v] < 2 || g->nC[v] > ncm) { set_error("ufe_geometry_attach: nC out of range"); return UFE_BAD_MESH; }
    for (int c = 0; c < g->nC[v]; ++c) {
      const int j = g->C[v + (size_t)c * nV];
      if (j < 1 || j > nV) { set_error("ufe_geometry_attach: C out of range"); return UFE_BAD_MESH; }
    }
  }
  for (size_t k = 0; k < 4 * (size_t)nAc; ++k)
    if (g->Aci[k] < 1 || g->Aci[k] > nV) { set_error("ufe_geometry_attach: Aci out of range"); return UFE_BAD_MESH; }
  // every Ac edge joins two connected vertices (the thickness update looks them up in C)
  auto connected = [&](int v, int w) {
    for (int c = 0; c < g->nC[v]; ++c)
      if (g->C[v + (size_t)c * nV] - 1 == w) return true;
    return false;
  };
  for (int c = 0; c < nAc; ++c) {
    const int vi = g->Aci[c] - 1, vj = g->Aci[c + (size_t)nAc] - 1;
    if (!connected(vi, vj) || !connected(vj, vi)) { set_error("ufe_geometry_attach: Aci(:,1:2) not connected in C"); return UFE_BAD_MESH; }
  }
  if (h->geom) { geom_free(h->geom); h->geom = nullptr; }
  GeomWork *w = new GeomWork();
  w->nV = nV; w->nAc = nAc; w->ncm = ncm;
  cudaStream_t s = h->stream;
  const size_t nv = nV, nac = nAc, nc = ncm;
  int rc = cuda_status(cudaMalloc(&w->nC, nv * sizeof(int)), "geometry");
  if (!rc) rc = cuda_status(cudaMalloc(&w->C, nv * nc * sizeof(int)), "geometry");
  if (!rc) rc = cuda_status(cudaMalloc(&w->Aci, 4 * nac * sizeof(int)), "geometry");
  if (!rc) rc = cuda_status(cudaMalloc(&w->Nx, nv * (nc + 1) * sizeof(double)), "geometry");
  if (!rc) rc = cuda_status(cudaMalloc(&w->Ny, nv * (nc + 1) * sizeof(double)), "geometry");
  if (!rc) rc = cuda_status(cudaMalloc(&w->Nx_Ac, 4 * nac * sizeof(double)), "geometry");
  if (!rc) rc = cuda_status(cudaMalloc(&w->Ny_Ac, 4 * nac * sizeof(double)), "geometry");
  if (!rc) rc = cuda_status(cudaMalloc(&w->No_Ac, 4 * nac * sizeof(double)), "geometry");
  if (!rc) rc = cuda_status(cudaMalloc(&w->Np_Ac, nac * sizeof(double)), "geometry");
  if (!rc) rc = cuda_status(cudaMalloc(&w->dbl, ((size_t)A_COUNT * nv + (size_t)C_COUNT * nac) * sizeof(double)), "geometry");
  if (!rc) rc = cuda_status(cudaMalloc(&w->msk, ((size_t)M_COUNT * nv + (size_t)MC_COUNT * nac) * sizeof(int)), "geometry");
  if (!rc) rc = cuda_status(cudaMalloc(&w->pk, (nv + nac) * sizeof(unsigned short)), "geometry masks");
  if (!rc) rc = cuda_status(cudaMalloc(&w->mask_stage, std::max(nv, nac) * sizeof(int)), "geometry masks");
  if (!rc) rc = up(w->nC, g->nC, nv, s);
  if (!rc) rc = up(w->C, g->C, nv * nc, s);
  if (!rc) rc = up(w->Aci, g->Aci, 4 * nac, s);
  if (!rc) rc = up(w->Nx, g->Nx, nv * (nc + 1), s);
  if (!rc) rc = up(w->Ny, g->Ny, nv * (nc + 1), s);
  if (!rc) rc = up(w->Nx_Ac, g->Nx_Ac, 4 * nac, s);
  if (!rc) rc = up(w->Ny_Ac, g->Ny_Ac, 4 * nac, s);
  if (!rc) rc = up(w->No_Ac, g->No_Ac, 4 * nac, s);
  if (!rc) rc = up(w->Np_Ac, g->Np_Ac, nac, s);
  if (!rc) rc = cuda_status(cudaStreamSynchronize(s), "geometry attach");
  if (rc) { geom_free(w); return rc; }
  h->geom = w;
  return UFE_OK;
}

extern "C" int ufe_geometry_update(ufe_mesh_h h, const double *Hi, const double *Hb, const double *SL,
                                   ufe_geometry_out *out) {
  if (!h || !Hi || !Hb || !SL) { set_error("ufe_geometry_update: null argument"); return UFE_BAD_ARG; }
  if (!h->geom) { set_error("ufe_geometry_update: call ufe_geometry_attach first"); return UFE_BAD_ARG; }
  int rc = compute(h, Hi, Hb, SL);
  if (rc) return rc;
  GeomWork *w = h->geom;
  GeomArgs a = args_of(w);
  cudaStream_t s = h->stream;
  if (out) {
    const size_t nV = w->nV, nAc = w->nAc;
    auto dd = [&](double *dst, const double *src, size_t n) {
      if (!dst || rc) return;
      rc = cuda_status(cudaMemcpyAsync(dst, src, n * sizeof(double), cudaMemcpyDeviceToHost, s), "geometry D2H");
    };
    auto di = [&](int32_t *dst, const int *src, size_t n) {
      if (!dst || rc) return;
      rc = cuda_status(cudaMemcpyAsync(dst, src, n * sizeof(int), cudaMemcpyDeviceToHost, s), "geometry D2H");
    };
    dd(out->Hs, AAF(a, A_HS), nV);
    dd(out->dHi_dx, AAF(a, A_DHI_DX), nV); dd(out->dHi_dy, AAF(a, A_DHI_DY), nV);
    dd(out->dHs_dx, AAF(a, A_DHS_DX), nV); dd(out->dHs_dy, AAF(a, A_DHS_DY), nV);
    dd(out->dHs_dx_shelf, AAF(a, A_DHS_DX_SH), nV); dd(out->dHs_dy_shelf, AAF(a, A_DHS_DY_SH), nV);
    di(out->mask_ocean, AAM(a, M_OCEAN), nV); di(out->mask_ice, AAM(a, M_ICE), nV);
    di(out->mask_sheet, AAM(a, M_SHEET), nV); di(out->mask_shelf, AAM(a, M_SHELF), nV);
    dd(out->Hi_Ac, ACF(a, C_HI), nAc); dd(out->Hb_Ac, ACF(a, C_HB), nAc); dd(out->SL_Ac, ACF(a, C_SL), nAc);
    dd(out->Hs_Ac, ACF(a, C_HS), nAc);
    double *acd[16] = {out->dHi_dx_Ac, out->dHi_dy_Ac, out->dHi_dp_Ac, out->dHi_do_Ac,
                       out->dHb_dx_Ac, out->dHb_dy_Ac, out->dHb_dp_Ac, out->dHb_do_Ac,
                       out->dHs_dx_Ac, out->dHs_dy_Ac, out->dHs_dp_Ac, out->dHs_do_Ac,
                       out->dSL_dx_Ac, out->dSL_dy_Ac, out->dSL_dp_Ac, out->dSL_do_Ac};
    for (int k = 0; k < 16; ++k) dd(acd[k], ACF(a, C_DHI_DX + k), nAc);
    dd(out->dHs_dx_shelf_Ac, ACF(a, C_DHS_DX_SH), nAc); dd(out->dHs_dy_shelf_Ac, ACF(a, C_DHS_DY_SH), nAc);
    di(out->mask_ocean_Ac, ACM(a, MC_OCEAN), nAc); di(out->mask_ice_Ac, ACM(a, MC_ICE), nAc);
    di(out->mask_sheet_Ac, ACM(a, MC_SHEET), nAc); di(out->mask_shelf_Ac, ACM(a, MC_SHELF), nAc);
    di(out->mask_gl_Ac, ACM(a, MC_GL), nAc);
  }
  if (!rc) rc = cuda_status(cudaStreamSynchronize(s), "geometry update");
  return rc;
}

extern "C" int ufe_geometry_masks(ufe_mesh_h h, ufe_mask_out *out) {
  if (!h || !out) { set_error("ufe_geometry_masks: null argument"); return UFE_BAD_ARG; }
  if (!h->geom || !h->geom->computed) {
    set_error("ufe_geometry_masks: no device geometry (ufe_geometry_update or ufe_ssa_upload_geometry first)");
    return UFE_BAD_ARG;
  }
  GeomWork *w = h->geom;
  cudaStream_t s = h->stream;
  int32_t *aa[kMkBits + 1] = {out->mask_land, out->mask_ocean, out->mask_lake, out->mask_ice, out->mask_sheet,
                              out->mask_shelf, out->mask_coast, out->mask_margin, out->mask_gl, out->mask_cf,
                              out->mask};
  int32_t *ac[kMkBits + 1] = {out->mask_land_Ac, out->mask_ocean_Ac, out->mask_lake_Ac, out->mask_ice_Ac,
                              out->mask_sheet_Ac, out->mask_shelf_Ac, out->mask_coast_Ac, out->mask_margin_Ac,
                              out->mask_gl_Ac, out->mask_cf_Ac, out->mask_Ac};
  int rc = UFE_OK;
  // one staging array, reused in stream order: each unpack waits for the previous copy
  auto one = [&](int32_t *dst, const unsigned short *src, int n, int k) {
    if (!dst || rc) return;
    k_mask_unpack<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(n, src, k, w->mask_stage);
    rc = cuda_status(cudaGetLastError(), "k_mask_unpack");
    if (!rc) rc = cuda_status(cudaMemcpyAsync(dst, w->mask_stage, (size_t)n * sizeof(int), cudaMemcpyDeviceToHost, s),
                              "masks D2H");
  };
  for (int k = 0; k <= kMkBits; ++k) {
    one(aa[k], w->pk, w->nV, k);
    one(ac[k], w->pk + w->nV, w->nAc, k);
  }
  if (!rc) rc = cuda_status(cudaStreamSynchronize(s), "geometry masks");
  return rc;
}

extern "C" int ufe_ssa_upload_geometry(ufe_mesh_h h, const ufe_params *p, const double *Hi, const double *Hb,
                                       const double *SL, const double *A_flow_mean, const double *A_flow_mean_Ac,
                                       const double *beta_sq_AaAc, const ufe_ssa_inout *io) {
  if (!h || !p || !Hi || !Hb || !SL || !io || (!A_flow_mean) != (!A_flow_mean_Ac)) {
    set_error("ufe_ssa_upload_geometry: null argument");
    return UFE_BAD_ARG;
  }
  if (!h->geom) { set_error("ufe_ssa_upload_geometry: call ufe_geometry_attach first"); return UFE_BAD_ARG; }
  if (!A_flow_mean && !h->geom->af_set) {
    set_error("ufe_ssa_upload_geometry: no flow factor on the device (ufe_ice_physical_properties first)");
    return UFE_BAD_ARG;
  }
  int rc = compute(h, Hi, Hb, SL);
  if (rc) return rc;
  GeomWork *w = h->geom;
  GeomArgs a = args_of(w);
  cudaStream_t s = h->stream;
  const size_t nV = w->nV, nAc = w->nAc, nA = nV + nAc;
  if (A_flow_mean) {
    rc = up(AAF(a, A_AF), A_flow_mean, nV, s);
    if (!rc) rc = up(ACF(a, C_AF), A_flow_mean_Ac, nAc, s);
    w->af_set = rc == UFE_OK;
  }
  double *beta_dev = nullptr;
  if (!rc && beta_sq_AaAc) {
    if (!w->beta) rc = cuda_status(cudaMalloc(&w->beta, nA * sizeof(double)), "geometry beta");
    beta_dev = w->beta;
    if (!rc) rc = up(beta_dev, beta_sq_AaAc, nA, s);
  }
  if (rc) return rc;
  // grounded-ice vertices (the early-out of solve_SSA), counted on the host from the inputs
  long long sheet = 0;
  for (size_t v = 0; v < nV; ++v)
    sheet += (Hi[v] > 0.0) && !(Hi[v] < ((SL[v] - Hb[v]) * kSeawaterDensity) / kIceDensity);
  ufe_ssa_in in;
  std::memset(&in, 0, sizeof(in));
  in.Hi = AAF(a, A_HI); in.Hb = AAF(a, A_HB); in.SL = AAF(a, A_SL);
  in.dHs_dx_shelf = AAF(a, A_DHS_DX_SH); in.dHs_dy_shelf = AAF(a, A_DHS_DY_SH); in.A_flow_mean = AAF(a, A_AF);
  in.mask_sheet = AAM(a, M_SHEET);
  in.Hi_Ac = ACF(a, C_HI); in.Hb_Ac = ACF(a, C_HB); in.SL_Ac = ACF(a, C_SL);
  in.dHs_dx_shelf_Ac = ACF(a, C_DHS_DX_SH); in.dHs_dy_shelf_Ac = ACF(a, C_DHS_DY_SH); in.A_flow_mean_Ac = ACF(a, C_AF);
  in.beta_sq_AaAc = beta_dev;
  in.mask_gl_Ac = ACM(a, MC_GL);
  in.dHi_dx_Ac = ACF(a, C_DHI_DX); in.dHi_dy_Ac = ACF(a, C_DHI_DY);
  in.dSL_dx_Ac = ACF(a, C_DSL_DX); in.dSL_dy_Ac = ACF(a, C_DSL_DY);
  in.dHb_dx_Ac = ACF(a, C_DHB_DX); in.dHb_dy_Ac = ACF(a, C_DHB_DY);
  return ssa_upload_impl(h, p, &in, io, true, sheet);
}

extern "C" int ufe_sia_solve_geometry(ufe_mesh_h h, const ufe_params *p, const double *A_flow_Ac, ufe_sia_out *out) {
  if (!h || !p || !out) { set_error("ufe_sia_solve_geometry: null argument"); return UFE_BAD_ARG; }
  if (!h->geom || !h->geom->computed) {
    set_error("ufe_sia_solve_geometry: no device geometry (ufe_geometry_update or ufe_ssa_upload_geometry first)");
    return UFE_BAD_ARG;
  }
  const double *A_dev = A_flow_Ac ? nullptr : props_A_flow_Ac(h->geom, p);
  if (!A_flow_Ac && !A_dev) {
    set_error("ufe_sia_solve_geometry: no A_flow_Ac on the device for this nZ (ufe_ice_physical_properties first)");
    return UFE_BAD_ARG;
  }
  GeomArgs a = args_of(h->geom);
  ufe_sia_in in;
  in.mask_sheet_Ac = ACM(a, MC_SHEET);
  in.Hi_Ac = ACF(a, C_HI);
  in.dHs_dx_Ac = ACF(a, C_DHS_DX); in.dHs_dy_Ac = ACF(a, C_DHS_DY);
  in.dHs_dp_Ac = ACF(a, C_DHS_DP); in.dHs_do_Ac = ACF(a, C_DHS_DO);
  in.A_flow_Ac = A_flow_Ac ? A_flow_Ac : A_dev;
  return sia_solve_impl(h, p, &in, out, true, A_dev != nullptr);
}

// ---------------------------------------------------------------------------------------
// Ice thickness update: calculate_ice_thickness_change (ice_dynamics_module.f90:31-237).
//
// The reference rescales outfluxes vertex by vertex; the rescale factor of a vertex depends
// only on its own outfluxes, its ice volume and its SMB/BMB (inflow entries are what other
// vertices change), and every connection's flux is owned by the vertex it leaves. So the
// device computes every factor in parallel and applies them when it sums: an outflux entry
// is scaled by its own vertex's factor, an influx entry by the factor of the vertex it came
// from — the same products the sequential loop forms, summed in the same order.
// ---------------------------------------------------------------------------------------
namespace ufe {
namespace {

struct ThkArgs {
  int nV, nAc, ncm;
  const int *nC, *C, *Aci;          // 1-based
  const double *A, *Cw, *Up_SIA, *Up_SSA, *SMB, *BMB;
  const int *noice;                 // may be null
  const int *dev_of_orig;
  const uint8_t *slice_g;           // edge rows: group 5
  double dt;
  int zero_edges;
  double *Hi, *Hi_prev, *dHi_dt;
  double *dVi;                      // (nV, ncm) column-major, zeroed
  double *factor, *Vi_SMB;          // (nV)
};

__device__ __forceinline__ int slot_of(const ThkArgs &a, int v, int w) {
  const int n = a.nC[v];
  for (int c = 0; c < n; ++c)
    if (a.C[v + (size_t)c * a.nV] - 1 == w) return c;
  return -1;
}

__global__ void k_thk_flux(const ThkArgs a) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= a.nAc) return;
  const int vi = a.Aci[c] - 1, vj = a.Aci[c + a.nAc] - 1;
  const int ci = slot_of(a, vi, vj), cj = slot_of(a, vj, vi);
  if (ci < 0 || cj < 0) return;   // ruled out by the host check of the connectivity
  const double Upar = a.Up_SIA[c] + a.Up_SSA[c];
  const double cw = a.Cw[vi + (size_t)ci * a.nV];
  const double dVi = Upar > 0.0 ? ((a.Hi[vi] * Upar) * cw) * a.dt : ((a.Hi[vj] * Upar) * cw) * a.dt;
  a.dVi[vi + (size_t)ci * a.nV] = -dVi;
  a.dVi[vj + (size_t)cj * a.nV] = dVi;
}

__global__ void k_thk_factor(const ThkArgs a) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= a.nV) return;
  double smb = ((a.SMB[v] + a.BMB[v]) * a.A[v]) * a.dt;
  const double avail = a.A[v] * a.Hi[v];
  double out = 0.0;
  for (int c = 0; c < a.nC[v]; ++c) {
    const double d = a.dVi[v + (size_t)c * a.nV];
    if (!(d > 0.0)) out = out - d;
  }
  double f = 1.0;
  if (-smb >= avail) {
    smb = -avail;
    f = 0.0;
  }
  if (out > avail + smb) f = (avail + smb) / out;
  a.factor[v] = f;
  a.Vi_SMB[v] = smb;
}

__global__ void k_thk_apply(const ThkArgs a) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= a.nV) return;
  const double fv = a.factor[v];
  double sum = 0.0;
  for (int c = 0; c < a.ncm; ++c) {
    double d = a.dVi[v + (size_t)c * a.nV];
    if (c < a.nC[v]) {
      if (d < 0.0) {
        if (fv < 1.0) d = d * fv;
      } else if (d > 0.0) {
        const int w = a.C[v + (size_t)c * a.nV] - 1;
        const double fw = a.factor[w];
        if (fw < 1.0) d = -((-d) * fw);   // the neighbour's scaled outflux, negated
      }
    }
    sum = sum + d;
  }
  double rate = (sum + a.Vi_SMB[v]) / (a.A[v] * a.dt);
  if (a.dt == 0.0) rate = 0.0;
  a.dHi_dt[v] = rate;
  const double h = a.Hi[v];
  a.Hi_prev[v] = h;
  double hn = h + (rate * a.dt);
  if (a.zero_edges && a.slice_g[a.dev_of_orig[v] / kSlice] == 5) hn = 0.0;
  if (a.noice && a.noice[v] == 1) hn = 0.0;
  a.Hi[v] = hn;
}

// The scaled fluxes themselves, for callers that keep dVi_in (a separate pass so that the
// summation above reads the unscaled entries of every neighbour).
__global__ void k_thk_fluxes_out(const ThkArgs a, double *out) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= a.nV) return;
  const double fv = a.factor[v];
  for (int c = 0; c < a.ncm; ++c) {
    double d = a.dVi[v + (size_t)c * a.nV];
    if (c < a.nC[v]) {
      if (d < 0.0) {
        if (fv < 1.0) d = d * fv;
      } else if (d > 0.0) {
        const double fw = a.factor[a.C[v + (size_t)c * a.nV] - 1];
        if (fw < 1.0) d = -((-d) * fw);
      }
    }
    out[v + (size_t)c * a.nV] = d;
  }
}

}  // namespace
}  // namespace ufe

extern "C" int ufe_thickness_update(ufe_mesh_h h, const ufe_thickness_in *in, double *Hi, ufe_thickness_out *out) {
  if (!h || !in || !Hi || !in->A || !in->Cw || !in->SMB_year || !in->BMB) {
    set_error("ufe_thickness_update: null argument");
    return UFE_BAD_ARG;
  }
  if (!h->geom) { set_error("ufe_thickness_update: call ufe_geometry_attach first"); return UFE_BAD_ARG; }
  GeomWork *g = h->geom;
  const DevMesh &m = h->m;
  const double *up_ssa = in->Up_SSA_Ac ? nullptr : ssa_device_Up(h);
  const double *up_sia = in->Up_SIA_Ac ? nullptr : sia_device_Up(h);
  if ((!in->Up_SSA_Ac && !up_ssa) || (!in->Up_SIA_Ac && !up_sia)) {
    set_error("ufe_thickness_update: no velocities given and no solve on this handle to take them from");
    return UFE_BAD_ARG;
  }
  cudaStream_t s = h->stream;
  const size_t nV = m.nV, nAc = m.nAc, ncm = m.ncm;
  // work: dVi (nV ncm), factor, Vi_SMB, Hi, Hi_prev, dHi_dt, A, SMB, BMB (nV each), Cw (nV ncm),
  // Up_SIA, Up_SSA (nAc each), noice (nV ints)
  const size_t nd = 2 * nV * ncm + 8 * nV + 2 * nAc;
  if (!g->thk) {
    int rc = cuda_status(cudaMalloc(&g->thk, nd * sizeof(double)), "thickness work");
    if (!rc) rc = cuda_status(cudaMalloc(&g->thk_int, nV * sizeof(int)), "thickness work");
    if (rc) return rc;
  }
  double *d = g->thk;
  ThkArgs a;
  a.nV = (int)nV; a.nAc = (int)nAc; a.ncm = (int)ncm; a.nC = g->nC; a.C = g->C; a.Aci = g->Aci;
  a.dVi = d; double *Cw = d + nV * ncm; a.factor = Cw + nV * ncm; a.Vi_SMB = a.factor + nV;
  a.Hi = a.Vi_SMB + nV; a.Hi_prev = a.Hi + nV; a.dHi_dt = a.Hi_prev + nV;
  double *A = a.dHi_dt + nV, *SMB = A + nV, *BMB = SMB + nV, *usia = BMB + nV, *ussa = usia + nAc;
  a.A = A; a.Cw = Cw; a.SMB = SMB; a.BMB = BMB;
  a.Up_SIA = in->Up_SIA_Ac ? usia : up_sia;
  a.Up_SSA = in->Up_SSA_Ac ? ussa : up_ssa;
  a.noice = in->mask_noice ? g->thk_int : nullptr;
  a.dev_of_orig = m.dev_of_orig; a.slice_g = m.slice_g; a.dt = in->dt; a.zero_edges = in->zero_edges != 0;
  int rc = cuda_status(cudaMemsetAsync(a.dVi, 0, nV * ncm * sizeof(double), s), "memset fluxes");
  if (!rc) rc = up(Cw, in->Cw, nV * ncm, s);
  if (!rc) rc = up(A, in->A, nV, s);
  if (!rc) rc = up(SMB, in->SMB_year, nV, s);
  if (!rc) rc = up(BMB, in->BMB, nV, s);
  if (!rc) rc = up(a.Hi, (const double *)Hi, nV, s);
  if (!rc && in->Up_SIA_Ac) rc = up(usia, in->Up_SIA_Ac, nAc, s);
  if (!rc && in->Up_SSA_Ac) rc = up(ussa, in->Up_SSA_Ac, nAc, s);
  if (!rc && in->mask_noice) rc = up(g->thk_int, (const int *)in->mask_noice, nV, s);
  const unsigned gv = (unsigned)((nV + 255) / 256), gc = (unsigned)((nAc + 255) / 256);
  if (!rc) { k_thk_flux<<<gc, 256, 0, s>>>(a); rc = cuda_status(cudaGetLastError(), "k_thk_flux"); }
  if (!rc) { k_thk_factor<<<gv, 256, 0, s>>>(a); rc = cuda_status(cudaGetLastError(), "k_thk_factor"); }
  if (!rc && out && out->dVi_in) {
    // Cw is no longer needed after the flux kernel: the scaled fluxes go there.
    k_thk_fluxes_out<<<gv, 256, 0, s>>>(a, Cw);
    rc = cuda_status(cudaGetLastError(), "k_thk_fluxes_out");
  }
  if (!rc) { k_thk_apply<<<gv, 256, 0, s>>>(a); rc = cuda_status(cudaGetLastError(), "k_thk_apply"); }
  auto dn = [&](double *dst, const double *src, size_t n) {
    if (!dst || rc) return;
    rc = cuda_status(cudaMemcpyAsync(dst, src, n * sizeof(double), cudaMemcpyDeviceToHost, s), "thickness D2H");
  };
  dn(Hi, a.Hi, nV);
  if (out) {
    dn(out->Hi_prev, a.Hi_prev, nV);
    dn(out->dHi_dt, a.dHi_dt, nV);
    dn(out->dVi_in, Cw, nV * ncm);
  }
  if (!rc) rc = cuda_status(cudaStreamSynchronize(s), "thickness update");
  return rc;
}

// ---------------------------------------------------------------------------------------
// 3-D SIA velocities: solve_SIA_3D (ice_dynamics_module.f90:317-405) on the device geometry,
// with apply_Neumann_boundary_3D (mesh_derivatives_module.f90:541-597) and the level
// derivatives of get_mesh_derivatives_vertex_3D (372-391). Fields (nV, nZ) column-major.
// ---------------------------------------------------------------------------------------
namespace ufe {
namespace {

constexpr int kMaxZ3 = 64;

struct Sia3dArgs {
  int nV, nZ, ncm;
  const int *nC, *C;
  const double *Nx, *Ny;
  const int *dev_of_orig;
  const uint8_t *slice_g;
  const double *Hi, *dHs_dx, *dHs_dy, *dHi_dx, *dHi_dy;
  const int *mask_shelf, *mask_sheet;
  const double *A, *dHb_dt, *U_SSA, *V_SSA;   // U_SSA/V_SSA may be null (no SSA solve: zero)
  double m_enh;
  double zeta[kMaxZ3], zeta3[kMaxZ3];
  double *U3, *V3, *W3;
};

__device__ __forceinline__ bool aa_edge(const Sia3dArgs &a, int v) {
  return a.slice_g[a.dev_of_orig[v] / kSlice] == 5;
}

__global__ void k_sia3d_uv(const Sia3dArgs a) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= a.nV) return;
  const size_t ld = a.nV;
  const double us = a.U_SSA ? a.U_SSA[v] : 0.0, vs = a.V_SSA ? a.V_SSA[v] : 0.0;
  const double h = a.Hi[v];
  if (a.mask_shelf[v] == 1 || h == 0.0) {
    for (int k = 0; k < a.nZ; ++k) { a.U3[v + k * ld] = us; a.V3[v + k * ld] = vs; }
    return;
  }
  const double sx = a.dHs_dx[v], sy = a.dHs_dy[v];
  const double D0 = pow((kIceDensity * kGrav) * h, 3.0) * pow(sx * sx + sy * sy, 1.0);
  double dd[kMaxZ3];
  const int nZ = a.nZ;
  double f_hi = (a.m_enh * a.A[v + (size_t)(nZ - 1) * ld]) * a.zeta3[nZ - 1];
  double acc = 0.0;
  dd[nZ - 1] = 0.0;
  for (int k = nZ - 2; k >= 0; --k) {
    const double f_lo = (a.m_enh * a.A[v + (size_t)k * ld]) * a.zeta3[k];
    acc = acc - (0.5 * (f_hi + f_lo)) * (a.zeta[k + 1] - a.zeta[k]);
    dd[k] = acc;
    f_hi = f_lo;
  }
  for (int k = 0; k < nZ; ++k) {
    double D = D0 * ((2.0 * h) * dd[k]);
    if (D < -1e5) D = -1e5;
    a.U3[v + k * ld] = D * sx + us;
    a.V3[v + k * ld] = D * sy + vs;
  }
}

// Edge vertices (not the corners) from their non-edge neighbours, every level.
__global__ void k_neumann3d_edges(const Sia3dArgs a, double *d) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v < 4 || v >= a.nV || !aa_edge(a, v)) return;
  const size_t ld = a.nV;
  const int n = a.nC[v];
  for (int k = 0; k < a.nZ; ++k) {
    double s = 0.0;
    int nvals = 0;
    for (int c = 0; c < n; ++c) {
      const int j = a.C[v + (size_t)c * ld] - 1;
      if (aa_edge(a, j)) continue;
      ++nvals;
      s = s + d[j + k * ld];
    }
    if (nvals < a.ncm) s = s + 0.0;
    d[v + k * ld] = s / (double)nvals;
  }
}

// The four corners from all their neighbours (after the edges).
__global__ void k_neumann3d_corners(const Sia3dArgs a, double *d) {
  const int v = threadIdx.x;
  if (v >= 4) return;
  const size_t ld = a.nV;
  const int n = a.nC[v];
  for (int k = 0; k < a.nZ; ++k) {
    double s = 0.0;
    for (int c = 0; c < n; ++c) s = s + d[(a.C[v + (size_t)c * ld] - 1) + k * ld];
    if (n < a.ncm) s = s + 0.0;
    d[v + k * ld] = s / (double)n;
  }
}

__device__ __forceinline__ void ddxy3(const Sia3dArgs &a, const double *d, int v, int k, double *dx, double *dy) {
  const size_t ld = a.nV;
  const int n = a.nC[v];
  double x = a.Nx[v + (size_t)n * ld] * d[v + k * ld];
  double y = a.Ny[v + (size_t)n * ld] * d[v + k * ld];
  for (int c = 0; c < n; ++c) {
    const int j = a.C[v + (size_t)c * ld] - 1;
    x = x + a.Nx[v + (size_t)c * ld] * d[j + k * ld];
    y = y + a.Ny[v + (size_t)c * ld] * d[j + k * ld];
  }
  *dx = x;
  *dy = y;
}

__global__ void k_sia3d_w(const Sia3dArgs a) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= a.nV) return;
  const size_t ld = a.nV;
  const int nZ = a.nZ;
  for (int k = 0; k < nZ; ++k) a.W3[v + k * ld] = 0.0;
  if (aa_edge(a, v) || a.mask_sheet[v] == 0) return;
  const double bx = a.dHs_dx[v] - a.dHi_dx[v];
  const double by = a.dHs_dy[v] - a.dHi_dy[v];
  double w = (a.dHb_dt[v] + a.U3[v + (nZ - 1) * ld] * bx) + a.V3[v + (nZ - 1) * ld] * by;
  a.W3[v + (nZ - 1) * ld] = w;
  const double h = a.Hi[v];
  const double mH = h > 0.1 ? h : 0.1;
  for (int k = nZ - 2; k >= 0; --k) {
    double ux0, uy0, ux1, uy1, vx0, vy0, vx1, vy1;
    ddxy3(a, a.U3, v, k, &ux0, &uy0);
    ddxy3(a, a.U3, v, k + 1, &ux1, &uy1);
    ddxy3(a, a.V3, v, k, &vx0, &vy0);
    ddxy3(a, a.V3, v, k + 1, &vx1, &vy1);
    const double w1 = (ux0 + ux1) / 2.0;
    const double w2 = (vy0 + vy1) / 2.0;
    const double dz = a.zeta[k + 1] - a.zeta[k];
    const double zm = 0.5 * (a.zeta[k + 1] + a.zeta[k]);
    const double w3 = ((a.dHs_dx[v] - zm * a.dHi_dx[v]) / mH) * ((a.U3[v + (k + 1) * ld] - a.U3[v + k * ld]) / dz);
    const double w4 = ((a.dHs_dy[v] - zm * a.dHi_dy[v]) / mH) * ((a.V3[v + (k + 1) * ld] - a.V3[v + k * ld]) / dz);
    w = w - (h * (((w1 + w2) + w3) + w4)) * dz;
    a.W3[v + k * ld] = w;
  }
}

}  // namespace
}  // namespace ufe

extern "C" int ufe_sia3d_solve(ufe_mesh_h h, const ufe_params *p, const double *A_flow, const double *dHb_dt,
                               ufe_sia3d_out *out) {
  if (!h || !p || !dHb_dt || !out || !p->zeta) { set_error("ufe_sia3d_solve: null argument"); return UFE_BAD_ARG; }
  if (p->nZ < 2 || p->nZ > kMaxZ3) { set_error("ufe_sia3d_solve: nZ must be in [2, 64]"); return UFE_BAD_ARG; }
  if (!h->geom || !h->geom->computed) {
    set_error("ufe_sia3d_solve: no device geometry (ufe_geometry_update or ufe_ssa_upload_geometry first)");
    return UFE_BAD_ARG;
  }
  GeomWork *g = h->geom;
  const double *A_dev = A_flow ? nullptr : props_A_flow(g, p);
  if (!A_flow && !A_dev) {
    set_error("ufe_sia3d_solve: no A_flow on the device for this nZ (ufe_ice_physical_properties first)");
    return UFE_BAD_ARG;
  }
  const DevMesh &m = h->m;
  GeomArgs ga = args_of(g);
  const size_t nV = m.nV, nZ = p->nZ;
  cudaStream_t s = h->stream;
  g->sia3d_done = false;
  if (g->sia3d_nZ != (int)nZ) {
    if (g->sia3d) { cudaFree(g->sia3d); g->sia3d = nullptr; }
    g->sia3d_nZ = 0;
    int rc = cuda_status(cudaMalloc(&g->sia3d, (4 * nV * nZ + nV) * sizeof(double)), "sia3d work");
    if (rc) return rc;
    g->sia3d_nZ = (int)nZ;
  }
  Sia3dArgs a;
  a.nV = (int)nV; a.nZ = (int)nZ; a.ncm = m.ncm; a.nC = g->nC; a.C = g->C; a.Nx = g->Nx; a.Ny = g->Ny;
  a.dev_of_orig = m.dev_of_orig; a.slice_g = m.slice_g;
  a.Hi = AAF(ga, A_HI); a.dHs_dx = AAF(ga, A_DHS_DX); a.dHs_dy = AAF(ga, A_DHS_DY);
  a.dHi_dx = AAF(ga, A_DHI_DX); a.dHi_dy = AAF(ga, A_DHI_DY);
  a.mask_shelf = AAM(ga, M_SHELF); a.mask_sheet = AAM(ga, M_SHEET);
  double *A = g->sia3d, *dhb = A + nV * nZ;
  a.U3 = dhb + nV; a.V3 = a.U3 + nV * nZ; a.W3 = a.V3 + nV * nZ;
  a.A = A_dev ? A_dev : A; a.dHb_dt = dhb;
  const double *uv = ssa_device_UV(h);
  a.U_SSA = uv; a.V_SSA = uv ? uv + nV : nullptr;
  a.m_enh = p->m_enh_sia;
  for (size_t k = 0; k < nZ; ++k) { a.zeta[k] = p->zeta[k]; a.zeta3[k] = std::pow(p->zeta[k], 3.0); }
  int rc = A_dev ? UFE_OK : up(A, A_flow, nV * nZ, s);
  if (!rc) rc = up(dhb, dHb_dt, nV, s);
  const unsigned gv = (unsigned)((nV + 127) / 128);
  if (!rc) { k_sia3d_uv<<<gv, 128, 0, s>>>(a); rc = cuda_status(cudaGetLastError(), "k_sia3d_uv"); }
  for (double *d : {a.U3, a.V3}) {
    if (!rc) { k_neumann3d_edges<<<gv, 128, 0, s>>>(a, d); rc = cuda_status(cudaGetLastError(), "k_neumann3d_edges"); }
    if (!rc) { k_neumann3d_corners<<<1, 32, 0, s>>>(a, d); rc = cuda_status(cudaGetLastError(), "k_neumann3d_corners"); }
  }
  if (!rc) { k_sia3d_w<<<gv, 128, 0, s>>>(a); rc = cuda_status(cudaGetLastError(), "k_sia3d_w"); }
  if (!rc) { k_neumann3d_edges<<<gv, 128, 0, s>>>(a, a.W3); rc = cuda_status(cudaGetLastError(), "k_neumann3d_edges"); }
  if (!rc) { k_neumann3d_corners<<<1, 32, 0, s>>>(a, a.W3); rc = cuda_status(cudaGetLastError(), "k_neumann3d_corners"); }
  auto dn = [&](double *dst, const double *src) {
    if (!dst || rc) return;
    rc = cuda_status(cudaMemcpyAsync(dst, src, nV * nZ * sizeof(double), cudaMemcpyDeviceToHost, s), "sia3d D2H");
  };
  dn(out->U_3D, a.U3);
  dn(out->V_3D, a.V3);
  dn(out->W_3D, a.W3);
  if (!rc) rc = cuda_status(cudaStreamSynchronize(s), "sia3d solve");
  g->sia3d_done = rc == UFE_OK;
  return rc;
}

// ---------------------------------------------------------------------------------------
// Upwind derivatives for the thermodynamics: get_upwind_derivative_vertex_3D
// (mesh_derivatives_module.f90:434-483) with is_in_triangle (mesh_help_functions_module.f90:
// 646-672). One thread per (vertex, layer), vertex fastest, so the wind and the field are read
// coalesced and only the triangle search gathers. Separately rounded products (no FMA) and
// IEEE sqrt/division: the search takes the same decisions as the reference's arithmetic.
// ---------------------------------------------------------------------------------------
namespace ufe {
namespace {

struct UpwArgs {
  int nV, nZ, nTri;
  const int *nC, *C;                    // (nV), (nV, ncm), 1-based
  const double *Nx, *Ny;                // (nV, ncm + 1), home at column nC + 1
  const double *V, *R;                  // (nV, 2), (nV)
  const int *niTri, *iTri, *Tri;        // (nV), (nV, ncm), (nTri, 3), 1-based
  const double *NxTri, *NyTri;          // (nTri, 3)
  const double *U, *Vw, *d;             // (nV, nZ)
  double *ddx, *ddy;                    // (nV, nZ)
  unsigned long long *missing;
};

__device__ __forceinline__ bool in_triangle(double pax, double pay, double pbx, double pby, double pcx, double pcy,
                                            double px, double py) {
  const double tol = 1E-8;
  const double as_x = px - pax, as_y = py - pay;
  const double s1 = ((pbx - pax) * as_y - (pby - pay) * as_x);
  const double s2 = ((pcx - pax) * as_y - (pcy - pay) * as_x);
  const double s3 = ((pcx - pbx) * (py - pby) - (pcy - pby) * (px - pbx));
  return s1 > -tol && s2 < tol && s3 > -tol;
}

__global__ void k_upwind(const UpwArgs a) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const size_t n = a.nV, nt = a.nTri;
  if (i >= n * a.nZ) return;
  const int vi = (int)(i % n);
  const size_t kof = i - vi;            // k * nV
  const double u = a.U[i], v = a.Vw[i];
  double dx = 0.0, dy = 0.0;
  if (fabs(u) < 1E-10 && fabs(v) < 1E-10) {
    // get_mesh_derivatives_vertex_3D (372-392): home term first
    const int nc = a.nC[vi];
    dx = a.Nx[vi + nc * n] * a.d[i];
    dy = a.Ny[vi + nc * n] * a.d[i];
    for (int c = 0; c < nc; ++c) {
      const double dc = a.d[(a.C[vi + c * n] - 1) + kof];
      dx = dx + a.Nx[vi + c * n] * dc;
      dy = dy + a.Ny[vi + c * n] * dc;
    }
  } else {
    const double s = 4.0 * sqrt(u * u + v * v);
    const double r = a.R[vi];
    const double px = a.V[vi] - u * r / s, py = a.V[vi + n] - v * r / s;
    int tup = -1, ta = 0, tb = 0, tc = 0;
    const int ni = a.niTri[vi];
    for (int it = 0; it < ni; ++it) {
      const int ti = a.iTri[vi + it * n] - 1;
      const int qa = a.Tri[ti] - 1, qb = a.Tri[ti + nt] - 1, qc = a.Tri[ti + 2 * nt] - 1;
      if (in_triangle(a.V[qa], a.V[qa + n], a.V[qb], a.V[qb + n], a.V[qc], a.V[qc + n], px, py)) {
        tup = ti; ta = qa; tb = qb; tc = qc;
        break;
      }
    }
    if (tup < 0) {
      atomicAdd(a.missing, 1ull);
    } else {
      const double da = a.d[ta + kof], db = a.d[tb + kof], dc = a.d[tc + kof];
      dx = a.NxTri[tup] * da + a.NxTri[tup + nt] * db + a.NxTri[tup + 2 * nt] * dc;
      dy = a.NyTri[tup] * da + a.NyTri[tup + nt] * db + a.NyTri[tup + 2 * nt] * dc;
    }
  }
  a.ddx[i] = dx;
  a.ddy[i] = dy;
}

}  // namespace
}  // namespace ufe

extern "C" int ufe_triangles_attach(ufe_mesh_h h, const ufe_triangle_mesh *t) {
  if (!h || !t || !t->V || !t->R || !t->niTri || !t->iTri || !t->Tri || !t->NxTri || !t->NyTri) {
    set_error("ufe_triangles_attach: missing array");
    return UFE_BAD_ARG;
  }
  if (!h->geom) { set_error("ufe_triangles_attach: call ufe_geometry_attach first"); return UFE_BAD_ARG; }
  GeomWork *w = h->geom;
  const int nV = w->nV, ncm = w->ncm, nTri = t->nTri;
  if (nTri < 1) { set_error("ufe_triangles_attach: nTri must be positive"); return UFE_BAD_MESH; }
  // validate the index arrays on the host before any kernel reads them
  for (size_t k = 0; k < 3 * (size_t)nTri; ++k)
    if (t->Tri[k] < 1 || t->Tri[k] > nV) { set_error("ufe_triangles_attach: Tri out of range"); return UFE_BAD_MESH; }
  for (int v = 0; v < nV; ++v) {
    if (t->niTri[v] < 0 || t->niTri[v] > ncm) { set_error("ufe_triangles_attach: niTri out of range"); return UFE_BAD_MESH; }
    for (int c = 0; c < t->niTri[v]; ++c) {
      const int ti = t->iTri[v + (size_t)c * nV];
      if (ti < 1 || ti > nTri) { set_error("ufe_triangles_attach: iTri out of range"); return UFE_BAD_MESH; }
    }
  }
  void *old[] = {w->tV, w->tR, w->NxTri, w->NyTri, w->niTri, w->iTri, w->Tri};
  for (void *p : old)
    if (p) cudaFree(p);
  w->tV = w->tR = w->NxTri = w->NyTri = nullptr;
  w->niTri = w->iTri = w->Tri = nullptr;
  w->nTri = 0;
  cudaStream_t s = h->stream;
  const size_t nv = nV, nt = nTri, nc = ncm;
  int rc = cuda_status(cudaMalloc(&w->tV, 2 * nv * sizeof(double)), "triangles");
  if (!rc) rc = cuda_status(cudaMalloc(&w->tR, nv * sizeof(double)), "triangles");
  if (!rc) rc = cuda_status(cudaMalloc(&w->NxTri, 3 * nt * sizeof(double)), "triangles");
  if (!rc) rc = cuda_status(cudaMalloc(&w->NyTri, 3 * nt * sizeof(double)), "triangles");
  if (!rc) rc = cuda_status(cudaMalloc(&w->niTri, nv * sizeof(int)), "triangles");
  if (!rc) rc = cuda_status(cudaMalloc(&w->iTri, nv * nc * sizeof(int)), "triangles");
  if (!rc) rc = cuda_status(cudaMalloc(&w->Tri, 3 * nt * sizeof(int)), "triangles");
  if (!rc) rc = up(w->tV, t->V, 2 * nv, s);
  if (!rc) rc = up(w->tR, t->R, nv, s);
  if (!rc) rc = up(w->NxTri, t->NxTri, 3 * nt, s);
  if (!rc) rc = up(w->NyTri, t->NyTri, 3 * nt, s);
  if (!rc) rc = up(w->niTri, t->niTri, nv, s);
  if (!rc) rc = up(w->iTri, t->iTri, nv * nc, s);
  if (!rc) rc = up(w->Tri, t->Tri, 3 * nt, s);
  if (!rc) rc = cuda_status(cudaStreamSynchronize(s), "triangles attach");
  if (!rc) w->nTri = nTri;
  return rc;
}

extern "C" int ufe_upwind_derivatives_3d(ufe_mesh_h h, const ufe_params *p, const double *U_3D, const double *V_3D,
                                         const double *d, double *ddx, double *ddy, int64_t *no_upwind) {
  if (!h || !p || !ddx || !ddy || (!U_3D) != (!V_3D)) {
    set_error("ufe_upwind_derivatives_3d: null argument");
    return UFE_BAD_ARG;
  }
  if (p->nZ < 1) { set_error("ufe_upwind_derivatives_3d: nZ must be positive"); return UFE_BAD_ARG; }
  if (!h->geom || h->geom->nTri < 1) {
    set_error("ufe_upwind_derivatives_3d: call ufe_geometry_attach and ufe_triangles_attach first");
    return UFE_BAD_ARG;
  }
  GeomWork *w = h->geom;
  const size_t nV = w->nV, nZ = p->nZ, nf = nV * nZ;
  if (!U_3D && !(w->sia3d_done && w->sia3d_nZ == (int)nZ)) {
    set_error("ufe_upwind_derivatives_3d: no 3-D velocities on the device for this nZ (ufe_sia3d_solve first)");
    return UFE_BAD_ARG;
  }
  if (!d && !(w->props_law == UFE_FLOW_ARRHENIUS && w->props_nZ == (int)nZ)) {
    set_error("ufe_upwind_derivatives_3d: no Ti on the device for this nZ (ufe_ice_physical_properties first)");
    return UFE_BAD_ARG;
  }
  cudaStream_t s = h->stream;
  int rc = UFE_OK;
  if (w->upw_nZ != (int)nZ) {
    if (w->upw) { cudaFree(w->upw); w->upw = nullptr; }
    w->upw_nZ = 0;
    rc = cuda_status(cudaMalloc(&w->upw, 5 * nf * sizeof(double)), "upwind work");
    if (rc) return rc;
    w->upw_nZ = (int)nZ;
  }
  if (!w->upw_missing) {
    rc = cuda_status(cudaMalloc(&w->upw_missing, sizeof(unsigned long long)), "upwind work");
    if (rc) return rc;
  }
  double *Ud = w->upw, *Vd = Ud + nf, *dd = Vd + nf, *ox = dd + nf, *oy = ox + nf;
  UpwArgs a;
  a.nV = (int)nV; a.nZ = (int)nZ; a.nTri = w->nTri;
  a.nC = w->nC; a.C = w->C; a.Nx = w->Nx; a.Ny = w->Ny;
  a.V = w->tV; a.R = w->tR; a.niTri = w->niTri; a.iTri = w->iTri; a.Tri = w->Tri;
  a.NxTri = w->NxTri; a.NyTri = w->NyTri;
  if (U_3D) {
    a.U = Ud; a.Vw = Vd;
    rc = up(Ud, U_3D, nf, s);
    if (!rc) rc = up(Vd, V_3D, nf, s);
  } else {
    const double *u3 = w->sia3d + nf + nV;           // A_flow, dHb_dt, then U_3D, V_3D, W_3D
    a.U = u3; a.Vw = u3 + nf;
  }
  if (d) {
    a.d = dd;
    if (!rc) rc = up(dd, d, nf, s);
  } else {
    a.d = w->props;                                   // Ti comes first in the properties block
  }
  a.ddx = ox; a.ddy = oy; a.missing = w->upw_missing;
  if (!rc) rc = cuda_status(cudaMemsetAsync(w->upw_missing, 0, sizeof(unsigned long long), s), "upwind");
  if (!rc) {
    k_upwind<<<(unsigned)((nf + 255) / 256), 256, 0, s>>>(a);
    rc = cuda_status(cudaGetLastError(), "k_upwind");
  }
  unsigned long long missing = 0;
  if (!rc) rc = cuda_status(cudaMemcpyAsync(ddx, ox, nf * sizeof(double), cudaMemcpyDeviceToHost, s), "upwind D2H");
  if (!rc) rc = cuda_status(cudaMemcpyAsync(ddy, oy, nf * sizeof(double), cudaMemcpyDeviceToHost, s), "upwind D2H");
  if (!rc) rc = cuda_status(cudaMemcpyAsync(&missing, w->upw_missing, sizeof(missing), cudaMemcpyDeviceToHost, s), "upwind D2H");
  if (!rc) rc = cuda_status(cudaStreamSynchronize(s), "upwind derivatives");
  if (!rc && no_upwind) *no_upwind = (int64_t)missing;
  return rc;
}
