// Internal declarations shared by the translation units of libufemism_gb300.
#pragma once

#include <cstdint>
#include <string>

#include "../../include/ufemism_gb300.h"

#ifdef __CUDACC__
#include <cuda_runtime.h>
#else
#include <cuda_runtime_api.h>
#endif

namespace ufe {

constexpr int kMaxDeg = 32;    // neighbours per AaAc row the kernels accept (nconmax <= 31)
constexpr int kSlice = 32;     // rows per SELL slice (one warp, one row per lane)
constexpr int kGroups = 6;     // colours 1..5 (rows swept by SOR), then the edge rows
constexpr int kMaxPatchSlices = 1024;  // slices of 32 rows per patch
// Persistent SSA solver: CTAs of kSsaBlock threads, kCtasPerSm per SM, one spatial patch per
// CTA. Measured on the 200k-vertex dome: 1024 x 1 beats 576 x 2, 640 x 2, 384 x 3 and
// 320 x 4 for the mixed sweep (more CTAs per SM spill at the lower register cap).
#ifndef UFE_SSA_BLOCK
#define UFE_SSA_BLOCK 1024
#endif
#ifndef UFE_SSA_CTAS_PER_SM
#define UFE_SSA_CTAS_PER_SM 1
#endif
constexpr int kSsaBlock = UFE_SSA_BLOCK;
constexpr int kCtasPerSm = UFE_SSA_CTAS_PER_SM;
constexpr int kMaxSync = 64;   // patches one patch may synchronise with

// Physical constants, parameters_module.f90:9-21.
constexpr double kIceDensity = 910.0;
constexpr double kSeawaterDensity = 1028.0;
constexpr double kGrav = 9.81;
constexpr double kPi = 3.141592653589793;

void set_error(const std::string &msg);
int cuda_status(cudaError_t e, const char *what);

void neighbour_functions(double px, double py, int n, const double *qx, const double *qy,
                         bool edge, double *Nx, double *Ny, double *Nxx, double *Nxy,
                         double *Nyy);
int aaac_build(const ufe_base_mesh *b, ufe_aaac_mesh *o, std::string *msg);
// ufe_mesh_create with a chosen number of spatial patches (0: the single-solve default).
int mesh_create(const ufe_mesh_desc *d, int n_patch, ufe_mesh_h *out);

// Device re-layout of the combined AaAc mesh.
//
// Rows are cut into spatially compact patches (Morton order of the row coordinates), one
// per CTA of the persistent solver. Inside a patch they are permuted into groups: the
// non-edge rows of colour 1, ..., colour 5 (the rows the SOR sweep updates, each colour an
// independent set), then the patch's edge rows (updated by the Neumann boundary condition)
// with corners last. Inside a colour the rows are sorted by degree (descending, stable in
// Morton order) so that the sliced-ELL slices of 32 rows are nearly uniform. Every group
// starts on a multiple of 32; the gaps are padding rows (degree 0) that kernels skip.
struct DevMesh {
  int nV = 0, nAc = 0, nA = 0, ncm = 0;
  int nP = 0;                   // padded device rows
  int nSlices = 0;
  int n_patch = 0;              // spatial patches = CTAs of the persistent SSA solver
  int max_patch_slices = 0;
  int max_sync = 0;
  int n_edge_total = 0;         // edge rows including the four corners
  int bnd_total = 0;            // entries of bnd_nbr
  int64_t nE = 0;               // padded SELL entries

  // Device arrays:
  int *orig_of_dev = nullptr;   // [nP] original 0-based AaAc row, -1 = padding
  int *dev_of_orig = nullptr;   // [nA]
  uint8_t *deg = nullptr;       // [nP]
  int64_t *slice_ptr = nullptr; // [nSlices] first SELL entry of the slice
  int *slice_e0 = nullptr;      // [nSlices] the same as int32
  uint8_t *slice_w = nullptr;   // [nSlices] slice width (entries per row)
  uint8_t *slice_g = nullptr;   // [nSlices] group: colour 0..4, 5 = edge rows
  int *patch_slice = nullptr;   // [n_patch][kGroups + 1] first slice of each group of a patch
  int *patch_edge0 = nullptr;   // [n_patch + 1] first edge ordinal of a patch
  int *edge_row = nullptr;      // [n_edge_total] device row of each edge ordinal
  int *sync_ptr = nullptr;      // [n_patch + 1] CSR of the patches each patch synchronises with
  int *sync_list = nullptr;
  int *col = nullptr;           // [nE] neighbour device row, -1 = padding
  double2 *cuv = nullptr;       // [nE] (4Nxx+Nyy, 4Nyy+Nxx)
  double2 *nxy = nullptr;       // [nE] (Nx, Ny)
  float2 *cuv32 = nullptr;      // [nE]
  float2 *nxy32 = nullptr;      // [nE]
  double2 *h_nxy = nullptr;     // [nP] home (Nx, Ny)
  double2 *h_cuv = nullptr;     // [nP] home (4Nxx+Nyy, 4Nyy+Nxx)
  double *sNxy = nullptr;       // [nP] sum of Nxy over home + neighbours
  double *s3Nxy = nullptr;      // [nP] 3 * sNxy (cross-term coefficient of the fast sweeps)
  float2 *h_nxy32 = nullptr;    // [nP] (Nx, Ny) row sums (home + neighbours), for the mixed viscosity
  float *s3Nxy32 = nullptr;     // [nP] 3 * sNxy in FP32
  // Neumann boundary lists by edge ordinal: edge rows' non-edge neighbours; corners' neighbours
  // with an edge neighbour k encoded as -(k+1).
  int *bnd_ptr = nullptr;       // [n_edge_total + 1]
  int *bnd_nbr = nullptr;
  // Geometry for the po rotation and the GL flux.
  double2 *V = nullptr;         // [nV] vertex x,y
  int2 *Aci12 = nullptr;        // [nAc] (vi, vj) 0-based
  int *iAci = nullptr;          // [nV * ncm] column-major Ac ids (0-based), for map_Ac_to_Aa
  int *nC = nullptr;            // [nV]

  // Halo sweep program (single solves; batched members in the mixed mode). One SOR sweep runs
  // in seven phases: colours 1..5, then the edge rows, then the corners. A patch updates,
  // besides its own rows, the halo
  // rows whose updates its own rows read within the same sweep (the closure of "reads a row
  // of an earlier phase"), with the same arithmetic, so that a whole sweep needs the
  // neighbouring patches only once, at its start. Its working copy of the velocities
  // (shared memory) holds its own device rows [p0, p1) at local index p - p0, then its halo
  // rows. The program lists, per phase, slices of 32 (local row, device row) slots with
  // their entries as local columns and coefficients, in the reference's neighbour order.
  bool has_halo = false;
  int max_local = 0;            // largest own slots + halo rows of a patch
  int max_halo = 0;             // largest number of halo rows of a patch
  int max_hslices = 0;          // largest number of program slices of a patch
  int max_hsync = 0;
  int n_hslices = 0;
  int64_t n_hE = 0;
  int *hp_slice = nullptr;      // [n_patch * 7 + 1] first program slice of phases 0..6 of each patch, then the end
  int *hp_split = nullptr;      // [n_patch] first slice of phase 0's rows that read halo slots (the others come first)
  int *hslice_e0 = nullptr;     // [n_hslices] first entry of a program slice
  uint8_t *hslice_w = nullptr;  // [n_hslices] entries per slot
  int *hrow_l = nullptr;        // [n_hslices * 32] local row, -1 = padding
  int *hrow_g = nullptr;        // [n_hslices * 32] device row
  uint16_t *hcol = nullptr;     // [n_hE] local column, 0xffff = padding
  float2 *hcuv32 = nullptr;     // [n_hE]
  double2 *hcuv = nullptr;      // [n_hE]
  int *hload_ptr = nullptr;     // [n_patch + 1] a patch's halo rows in hload_dev
  int *hload_dev = nullptr;     // device row of each halo slot
  int *hsync_ptr = nullptr;     // [n_patch + 1] patches a patch waits for / is waited for by
  int *hsync_list = nullptr;
  float *hs3_32 = nullptr;      // [n_hslices * 32] 3 sNxy of the slot's row (FP32), 0 on padding
  double *hs3 = nullptr;        // [n_hslices * 32] the same in FP64
};

struct SsaWork;   // per-handle device buffers of the SSA solve (ufe_ssa.cu)
struct SiaWork;   // per-handle device buffers of the SIA solve (ufe_sia.cu)
struct AdjWork;   // per-handle device buffers of the SSA adjoint (ufe_ssa.cu)
struct GeomWork;  // per-handle geometry preparation (ufe_geom.cu)

}  // namespace ufe

struct ufe_mesh_s {
  int device = 0;
  cudaStream_t stream = nullptr;
  int num_sms = 0;
  ufe::DevMesh m;
  ufe::SsaWork *ssa = nullptr;
  ufe::SiaWork *sia = nullptr;
  ufe::AdjWork *adj = nullptr;
  ufe::GeomWork *geom = nullptr;
};

namespace ufe {
void ssa_free(SsaWork *w);
void sia_free(SiaWork *w);
void adj_free(AdjWork *w);
void geom_free(GeomWork *w);
// ufe_sia_solve with the mask and Ac fields of `in` on the device (A_flow_Ac on the host).
int sia_solve_impl(ufe_mesh_h h, const ufe_params *p, const ufe_sia_in *in, ufe_sia_out *out, bool fields_on_device,
                   bool A_on_device = false);
// Velocities of the last solves on a handle, on the device (caller order), or null.
const double *ssa_device_Up(ufe_mesh_h h);
const double *ssa_device_UV(ufe_mesh_h h);
const double *sia_device_Up(ufe_mesh_h h);
// ufe_ssa_upload from device arrays of this device (sheet_count: grounded-ice vertices).
int ssa_upload_impl(ufe_mesh_h h, const ufe_params *p, const ufe_ssa_in *in, const ufe_ssa_inout *io,
                    bool in_on_device, long long sheet_count);
}  // namespace ufe
