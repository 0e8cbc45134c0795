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
constexpr int kMaxRuns = 24;   // distinct slice widths per group (degrees are <= nconmax)

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

// Device re-layout of the combined AaAc mesh.
//
// Rows are permuted into groups: the non-edge rows of colour 1, ..., colour 5 (the rows
// the SOR sweep updates, each colour an independent set), then all edge rows (updated by
// the Neumann boundary condition) with the four corners last. Inside a colour the rows
// are sorted by degree (descending, stable in the reference's row order) so that the
// sliced-ELL slices of 32 rows are nearly uniform. Every group starts on a multiple of 32;
// the gaps are padding rows (degree 0) that kernels skip.
struct DevMesh {
  int nV = 0, nAc = 0, nA = 0, ncm = 0;
  int nP = 0;                   // padded device rows
  int nSlices = 0;
  int grp_off[kGroups + 1] = {};  // device row offsets of the groups (multiples of 32)
  int grp_rows[kGroups] = {};   // real rows per group
  // Runs of equal slice width inside each group (rows are sorted by degree, so widths only
  // fall): run r of group g covers slices [run_s0, next run's run_s0) of width run_w, whose
  // first SELL entry is run_e0. Kernels compute a slice's entry offset from this table
  // instead of loading it.
  int n_runs[kGroups] = {};
  int run_s0[kGroups][kMaxRuns] = {};
  int run_w[kGroups][kMaxRuns] = {};
  int64_t run_e0[kGroups][kMaxRuns] = {};
  int n_edge = 0;               // edge rows excluding the corners
  int n_corner = 0;             // 4
  int edge_first = 0;           // device row of the first edge row (== grp_off[5])
  int64_t nE = 0;               // padded SELL entries

  // Host copies kept for scatter bookkeeping.
  // Device arrays:
  int *orig_of_dev = nullptr;   // [nP] original 0-based AaAc row, -1 = padding
  int *dev_of_orig = nullptr;   // [nA]
  uint8_t *deg = nullptr;       // [nP]
  int64_t *slice_ptr = nullptr; // [nSlices] first SELL entry of the slice
  int *col = nullptr;           // [nE] neighbour device row
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
  // Neumann boundary: edge rows' non-edge neighbours, corners' neighbours.
  int *bnd_ptr = nullptr;       // [n_edge + n_corner + 1]
  int *bnd_nbr = nullptr;       // device rows; for corners an edge neighbour is -(k+1), k = edge list index
  // Geometry for the po rotation and the GL flux.
  double2 *V = nullptr;         // [nV] vertex x,y
  int2 *Aci12 = nullptr;        // [nAc] (vi, vj) 0-based
  int *iAci = nullptr;          // [nV * ncm] column-major Ac ids (0-based), for map_Ac_to_Aa
  int *nC = nullptr;            // [nV]
};

struct SsaWork;   // per-handle device buffers of the SSA solve (ufe_ssa.cu)
struct SiaWork;   // per-handle device buffers of the SIA solve (ufe_sia.cu)

}  // namespace ufe

struct ufe_mesh_s {
  int device = 0;
  cudaStream_t stream = nullptr;
  int num_sms = 0;
  ufe::DevMesh m;
  ufe::SsaWork *ssa = nullptr;
  ufe::SiaWork *sia = nullptr;
};

namespace ufe {
void ssa_free(SsaWork *w);
void sia_free(SiaWork *w);
}  // namespace ufe
