/*
 * ufemism_gb300 -- C-ABI of the GB300 (sm_103a) ice-velocity solver for UFEMISM.
 *
 * Drop-in boundary for the two Fortran call sites of the reference model:
 *   CALL solve_SIA( region%mesh, region%ice)   UFEMISM_main_model.f90:124
 *   CALL solve_SSA( region%mesh, region%ice)   UFEMISM_main_model.f90:132
 * A Fortran wrapper with the same names and signatures (ice_dynamics_module.f90:240-249 and
 * 408-417) passes raw pointers of the type_mesh / type_ice_model components
 * (data_types_module.f90:15-345) to the functions below through ISO_C_BINDING.
 *
 * Conventions
 *  - Every array is in the reference's own layout: 2-D arrays column-major (Fortran order)
 *    with their allocated leading dimension, index VALUES 1-based, unused neighbour slots 0.
 *    Floating point is double (REAL(dp)), integers int32_t (default INTEGER).
 *  - The library copies host arrays in and out during each call and keeps no host pointer
 *    after it returns. Device buffers live in the opaque mesh handle; the handle must be
 *    destroyed and re-created after a mesh update (run_model_update_mesh,
 *    UFEMISM_main_model.f90:240-315).
 *  - Calls on one handle are not re-entrant; each handle owns one CUDA stream and the host
 *    thread blocks until results are back. The Fortran wrapper calls from the master rank
 *    only, then CALL sync (all ranks see the results in the shared windows).
 *  - Return value: 0 = UFE_OK, > 0 a warning, < 0 an error. ufe_last_error_string() gives a
 *    thread-local message for the last non-zero status.
 *  - There is no CPU fallback: without a usable sm_103a device every solve returns
 *    UFE_NO_DEVICE.
 */
#ifndef UFEMISM_GB300_H
#define UFEMISM_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define UFE_ABI_VERSION 1

/* Status codes. The warnings and errors mirror the reference's failure handling:
 *   UFE_NOT_CONVERGED  SOR hit SSA_max_inner_loops: WRITE(0,*) warning, ice_dynamics_module.f90:685-689
 *   UFE_RESET_ONCE     velocities reset to zero once after max residual > 1e6, 676-684
 *   UFE_DIVERGED       second reset: the reference calls MPI_ABORT, 532-540
 *   UFE_BAD_MESH       make_combined_AaAc_mesh / check_solution aborts
 *   UFE_COLOUR_IDENTIFY the five-colouring reached 'identify', where the reference aborts
 *                      unconditionally (mesh_five_colour_module.f90:452)
 *   UFE_TIMEOUT        a bounded device-side wait (inter-CTA colour barrier) ran out */
enum {
  UFE_OK = 0,
  UFE_NOT_CONVERGED = 1,
  UFE_RESET_ONCE = 2,
  UFE_DIVERGED = -1,
  UFE_BAD_MESH = -2,
  UFE_COLOUR_IDENTIFY = -3,
  UFE_TIMEOUT = -4,
  UFE_CUDA_ERROR = -5,
  UFE_BAD_ARG = -6,
  UFE_NO_DEVICE = -7,
  UFE_OUT_OF_MEMORY = -8,
};

enum { UFE_FP64 = 0, UFE_MIXED = 1 };
enum { UFE_SLIDING_COULOMB_REGULARISED = 0, UFE_SLIDING_LINEAR = 1 };

/* Mesh as held by the reference's type_mesh (data_types_module.f90:216-345), after
 * make_Ac_mesh (mesh_ArakawaC_module.f90:24-241), make_combined_AaAc_mesh (286-540) and
 * calculate_five_colouring_AaAc (mesh_five_colour_module.f90:18-137). */
typedef struct ufe_mesh_desc {
  int32_t nV, nAc, nVAaAc, nC_mem;
  const double *V;             /* (nV,2) vertex x,y */
  const int32_t *nC;           /* (nV) */
  const int32_t *iAci;         /* (nV,nC_mem) Aa->Ac map */
  const int32_t *Aci;          /* (nAc,4) [vi,vj,vl,vr] */
  const int32_t *edge_index;   /* (nV) */
  const int32_t *edge_index_Ac;/* (nAc) */
  const int32_t *nCAaAc;       /* (nVAaAc) */
  const int32_t *CAaAc;        /* (nVAaAc,nC_mem) */
  const double *Nx_AaAc, *Ny_AaAc, *Nxx_AaAc, *Nxy_AaAc, *Nyy_AaAc; /* (nVAaAc,nC_mem+1) */
  const int32_t *colour;       /* (nVAaAc) 1..5 */
  const int32_t *colour_vi;    /* (nVAaAc,5) */
  const int32_t *colour_nV;    /* (5) */
} ufe_mesh_desc;

/* SSA/SIA knobs (configuration_module.f90:124-126, 169-184) as a POD struct. */
typedef struct ufe_params {
  double SSA_RN_tol;
  int32_t SSA_max_outer_loops;
  double SSA_max_residual_UV;
  double SSA_SOR_omega;
  int32_t SSA_max_inner_loops;
  double m_enh_ssa, m_enh_sia;
  int32_t sliding_law;            /* UFE_SLIDING_* ; linear is this library's extension */
  double beta_sq;                 /* linear law, used when ufe_ssa_in.beta_sq_AaAc is NULL */
  int32_t use_analytical_GL_flux;
  int32_t zero_velocities;        /* benchmark experiments that skip the SSA (431-449) */
  int32_t nZ;
  const double *zeta;             /* (nZ) */
  int32_t precision;              /* UFE_FP64 or UFE_MIXED */
  int32_t mixed_refold_sweeps;    /* mixed: FP64 defect recomputed every this many sweeps (0 = default 256) */
  int32_t fp64_exact;             /* FP64: 1 = the reference's expression order, separately rounded
                                     multiplies and adds and IEEE divisions (bit-level parity mode);
                                     0 = fused multiply-adds and a reciprocal of the centre
                                     coefficient per Picard iteration (results differ in the last bits) */
  int32_t mixed_fp32_viscosity;   /* mixed: 1 = effective viscosity in FP32 as well (default 0: FP64) */
} ufe_params;

/* Inputs of solve_SSA (type_ice_model fields). Aa arrays have nV entries, Ac arrays nAc. */
typedef struct ufe_ssa_in {
  const double *Hi, *Hb, *SL, *dHs_dx_shelf, *dHs_dy_shelf, *A_flow_mean;
  const int32_t *mask_sheet;
  const double *Hi_Ac, *Hb_Ac, *SL_Ac, *dHs_dx_shelf_Ac, *dHs_dy_shelf_Ac, *A_flow_mean_Ac;
  const double *beta_sq_AaAc;     /* (nVAaAc) linear law field, or NULL */
  /* only with use_analytical_GL_flux */
  const int32_t *mask_gl_Ac;
  const double *dHi_dx_Ac, *dHi_dy_Ac, *dSL_dx_Ac, *dSL_dy_Ac, *dHb_dx_Ac, *dHb_dy_Ac;
} ufe_ssa_in;

/* Warm start in, solution out (INTENT(INOUT) in the reference). N_AaAc is the Picard state
 * that persists in the ice model between calls; NULL means zeros and no write-back. */
typedef struct ufe_ssa_inout {
  double *U_SSA, *V_SSA;          /* (nV) */
  double *Ux_SSA_Ac, *Uy_SSA_Ac;  /* (nAc) */
  double *N_AaAc;                 /* (nVAaAc) or NULL */
} ufe_ssa_inout;

/* Optional outputs; any pointer may be NULL. */
typedef struct ufe_ssa_out {
  double *Up_SSA_Ac, *Uo_SSA_Ac;  /* (nAc) rotate_xy_to_po, mesh_ArakawaC_module.f90:815-844 */
  double *eta_AaAc, *S_AaAc, *tau_c_AaAc, *phi_fric_AaAc; /* (nVAaAc) */
} ufe_ssa_out;

typedef struct ufe_ssa_stats {
  int32_t status;
  int32_t picard_iterations;
  int32_t linear_solves;
  int32_t resets;
  int32_t not_converged;
  int64_t total_sweeps;
  double last_RN;
  double last_max_residual;
  int32_t sweeps[64];             /* SOR sweeps of the first 64 linear solves */
  double device_ms;               /* device time of the solve (CUDA events) */
} ufe_ssa_stats;

/* Inputs and outputs of solve_SIA (ice_dynamics_module.f90:240-314). */
typedef struct ufe_sia_in {
  const int32_t *mask_sheet_Ac;   /* (nAc) */
  const double *Hi_Ac, *dHs_dx_Ac, *dHs_dy_Ac, *dHs_dp_Ac, *dHs_do_Ac; /* (nAc) */
  const double *A_flow_Ac;        /* (nAc,nZ) */
} ufe_sia_in;

typedef struct ufe_sia_out {
  double *D_SIA_3D_Ac;            /* (nAc,nZ) or NULL */
  double *D_SIA_Ac, *Ux_SIA_Ac, *Uy_SIA_Ac, *Up_SIA_Ac, *Uo_SIA_Ac; /* (nAc) */
  double *U_SIA, *V_SIA, *D_SIA;  /* (nV) map_Ac_to_Aa */
} ufe_sia_out;

typedef struct ufe_mesh_s *ufe_mesh_h;

/* Library version / device probe. Returns UFE_OK when an sm_103 device is usable. */
int ufe_init(int device);
const char *ufe_last_error_string(void);

/* Upload a mesh: the colour-sorted device re-layout is built here (once per mesh).
 * Replaces the per-call use of the mesh arrays by solve_SSA / solve_SIA. */
int ufe_mesh_create(const ufe_mesh_desc *desc, ufe_mesh_h *out);
int ufe_mesh_destroy(ufe_mesh_h mesh);
/* The handle's CUDA stream (cudaStream_t), for callers that time on it. */
void *ufe_mesh_stream(ufe_mesh_h mesh);

/* solve_SSA, ice_dynamics_module.f90:408-557, including basal_yield_stress (780-844) and,
 * with use_analytical_GL_flux, calculate_GL_flux (848-949). */
int ufe_ssa_solve(ufe_mesh_h mesh, const ufe_params *params, const ufe_ssa_in *in,
                  ufe_ssa_inout *inout, ufe_ssa_out *out, ufe_ssa_stats *stats);

/* The same solve split into its transfer and compute parts: ufe_ssa_upload copies the
 * inputs and warm start into the handle's device buffers, ufe_ssa_run solves from them
 * (device-resident in, device-resident out, may be called repeatedly on the same
 * uploaded inputs) and ufe_ssa_download copies the results back. */
int ufe_ssa_upload(ufe_mesh_h mesh, const ufe_params *params, const ufe_ssa_in *in,
                   const ufe_ssa_inout *inout);
int ufe_ssa_run(ufe_mesh_h mesh, const ufe_params *params, ufe_ssa_stats *stats);
int ufe_ssa_download(ufe_mesh_h mesh, ufe_ssa_inout *inout, ufe_ssa_out *out);

/* bottom_frictional_heating (thermodynamics_module.f90:281-311) from the last solve on this
 * handle: on vertices with mask_sheet == 1, tau_c (U^2 + V^2) (delta_v^2 + U^2 + V^2)^((q-1)/2)
 * / u_threshold^q with the solve's own U_SSA, V_SSA and tau_c_AaAc; 0 elsewhere. (nV) arrays. */
int ufe_ssa_frictional_heating(ufe_mesh_h mesh, const int32_t *mask_sheet, double *frictional_heating);

/* solve_SIA, ice_dynamics_module.f90:240-314 with map_Ac_to_Aa (mesh_ArakawaC_module.f90:770-791). */
int ufe_sia_solve(ufe_mesh_h mesh, const ufe_params *params, const ufe_sia_in *in,
                  ufe_sia_out *out);

/* No counterpart in the reference. ufe_sia_solve for callers that cannot allocate device
 * memory (a model that reserves the device's memory for its own pool; a time loop that cannot
 * afford the device-wide synchronisation of cudaMalloc/cudaFree): every array of `in` and `out`
 * is DEVICE memory of the mesh's device (the mesh's device must be current), nothing is
 * allocated, and the Ac intermediates the caller leaves NULL live in a fixed scratch array of
 * the library (at most UFE_SIA_NOALLOC_MAX_AC Ac edges; larger meshes return UFE_BAD_ARG).
 * Up to 64 devices. The scratch is shared by every call on a device: calls that overlap in
 * time (several threads, or several meshes of the same device) race on it and must be
 * serialised by the caller. Synchronous like ufe_sia_solve. The results stay in the caller's
 * arrays only, not on the handle: the call drops the SIA velocities an earlier ufe_sia_solve
 * left there, so a later ufe_thickness_update must be given Up_SIA_Ac (with NULL it returns
 * UFE_BAD_ARG). */
#define UFE_SIA_NOALLOC_MAX_AC 262144
int ufe_sia_solve_noalloc(ufe_mesh_h mesh, const ufe_params *params, const ufe_sia_in *in,
                          ufe_sia_out *out);

/* Geometry preparation on the device: the fields update_general_ice_model_data
 * (general_ice_model_data_module.f90:23-96) derives from Hi, Hb and SL for the velocity
 * solve — Aa-to-Ac maps, Hs, ocean/ice/sheet/shelf masks on Aa and Ac, the grounding-line
 * mask on Ac, the Aa slopes of Hi and Hs, the Ac slopes of Hi, Hb, Hs and SL, and the shelf
 * slopes — bit-identical to the reference's. ufe_geometry_attach uploads the derivative
 * stencils once per mesh; ufe_ssa_upload_geometry then replaces ufe_ssa_upload with only
 * Hi, Hb, SL, the flow factor and the optional friction field crossing from the host. */
typedef struct ufe_geometry_mesh {
  const int32_t *nC, *C;                /* (nV), (nV,nC_mem) */
  const double *Nx, *Ny;                /* (nV,nC_mem+1) Aa neighbour functions */
  const int32_t *Aci;                   /* (nAc,4) */
  const double *Nx_Ac, *Ny_Ac, *No_Ac;  /* (nAc,4) */
  const double *Np_Ac;                  /* (nAc) */
} ufe_geometry_mesh;
typedef struct ufe_geometry_out {       /* host arrays, each may be NULL */
  double *Hs, *dHi_dx, *dHi_dy, *dHs_dx, *dHs_dy, *dHs_dx_shelf, *dHs_dy_shelf;     /* (nV) */
  int32_t *mask_ocean, *mask_ice, *mask_sheet, *mask_shelf;                        /* (nV) */
  double *Hi_Ac, *Hb_Ac, *SL_Ac, *Hs_Ac;                                            /* (nAc) */
  double *dHi_dx_Ac, *dHi_dy_Ac, *dHi_dp_Ac, *dHi_do_Ac, *dHb_dx_Ac, *dHb_dy_Ac, *dHb_dp_Ac, *dHb_do_Ac;
  double *dHs_dx_Ac, *dHs_dy_Ac, *dHs_dp_Ac, *dHs_do_Ac, *dSL_dx_Ac, *dSL_dy_Ac, *dSL_dp_Ac, *dSL_do_Ac;
  double *dHs_dx_shelf_Ac, *dHs_dy_shelf_Ac;                                        /* (nAc) */
  int32_t *mask_ocean_Ac, *mask_ice_Ac, *mask_sheet_Ac, *mask_shelf_Ac, *mask_gl_Ac; /* (nAc) */
} ufe_geometry_out;
int ufe_geometry_attach(ufe_mesh_h mesh, const ufe_geometry_mesh *geometry);
int ufe_geometry_update(ufe_mesh_h mesh, const double *Hi, const double *Hb, const double *SL,
                        ufe_geometry_out *out);

/* Every mask of determine_masks (general_ice_model_data_module.f90:97-297) from the device
 * geometry of the last ufe_geometry_update / ufe_ssa_upload_geometry, where they are computed
 * beside the others and stay: land, ocean, lake (never set by the routine: all 0), ice, sheet,
 * shelf, coast, margin, grounding line, calving front, and the type mask `mask` (type_land 0,
 * ocean 1, lake 2, sheet 3, shelf 4, coast 5, margin 6, groundingline 7, calvingfront 8: the
 * last type the routine assigns), on the Aa vertices (nV) and the Ac edges (nAc). Host arrays,
 * each may be NULL. */
typedef struct ufe_mask_out {
  int32_t *mask_land, *mask_ocean, *mask_lake, *mask_ice, *mask_sheet, *mask_shelf, *mask_coast, *mask_margin,
      *mask_gl, *mask_cf, *mask;                                                    /* (nV) */
  int32_t *mask_land_Ac, *mask_ocean_Ac, *mask_lake_Ac, *mask_ice_Ac, *mask_sheet_Ac, *mask_shelf_Ac,
      *mask_coast_Ac, *mask_margin_Ac, *mask_gl_Ac, *mask_cf_Ac, *mask_Ac;           /* (nAc) */
} ufe_mask_out;
int ufe_geometry_masks(ufe_mesh_h mesh, ufe_mask_out *out);
int ufe_ssa_upload_geometry(ufe_mesh_h mesh, const ufe_params *params, const double *Hi, const double *Hb,
                            const double *SL, const double *A_flow_mean, const double *A_flow_mean_Ac,
                            const double *beta_sq_AaAc, const ufe_ssa_inout *inout);
/* solve_SIA on the device geometry of the last ufe_geometry_update / ufe_ssa_upload_geometry
 * (mask_sheet_Ac, Hi_Ac and the Ac surface slopes never leave the device); A_flow_Ac (nAc,nZ)
 * from the host. */
int ufe_sia_solve_geometry(ufe_mesh_h mesh, const ufe_params *params, const double *A_flow_Ac, ufe_sia_out *out);

/* solve_SIA_3D (ice_dynamics_module.f90:317-405) on the device geometry of the last
 * ufe_geometry_update / ufe_ssa_upload_geometry and the U_SSA, V_SSA of the last solve on the
 * handle (zero without one): U_3D, V_3D = SIA deformation velocities plus the SSA basal ones on
 * grounded vertices, Neumann rule on the domain edge, W_3D by vertical integration of the
 * divergence. A_flow (nV,nZ), dHb_dt (nV) host arrays; outputs (nV,nZ), each may be NULL. */
typedef struct ufe_sia3d_out {
  double *U_3D, *V_3D, *W_3D;
} ufe_sia3d_out;
int ufe_sia3d_solve(ufe_mesh_h mesh, const ufe_params *params, const double *A_flow, const double *dHb_dt,
                    ufe_sia3d_out *out);

/* ice_physical_properties (general_ice_model_data_module.f90:298-462) on the device, the last
 * step of update_general_ice_model_data: from the ice temperature Ti (nV,nZ) and the Hi,
 * mask_sheet, mask_sheet_Ac of the last ufe_geometry_update / ufe_ssa_upload_geometry.
 *   UFE_FLOW_ARRHENIUS: Ti_Ac = map_Aa_to_Ac_3D(Ti); Ti_pmp, A_flow (Arrhenius law, two
 *     branches at 263.15 K), Cpi, Ki on Aa; A_flow_Ac on Ac; A_flow_mean(_Ac) = the vertical
 *     average under grounded ice, else the Arrhenius law at (Ti(:,1) + SMT) / 2.
 *   UFE_FLOW_EISMINT (the EISMINT_1..6, Halfar, Bueler, mesh_generation_test benchmarks):
 *     A = 1e-16 everywhere, Ki = 2.1 sec_per_year, Cpi = 2009, Ti_pmp from Hi; Ti not read,
 *     Ti_Ac not written.
 *   UFE_FLOW_MISMIP_MOD: A = 1e-16, 1e-17 or 1e-16 for time < 25,000, < 50,000, < 75,000
 *     years, else 1e-16; only the four A fields are written.
 * The results stay on the device: ufe_ssa_upload_geometry with both A_flow_mean arrays NULL,
 * ufe_sia_solve_geometry with A_flow_Ac NULL and ufe_sia3d_solve with A_flow NULL take them
 * from there. Each output host array may be NULL. */
enum { UFE_FLOW_ARRHENIUS = 0, UFE_FLOW_EISMINT = 1, UFE_FLOW_MISMIP_MOD = 2 };
typedef struct ufe_physprop_out {
  double *A_flow, *Ti_pmp, *Cpi, *Ki;   /* (nV,nZ) */
  double *A_flow_mean;                  /* (nV) */
  double *A_flow_Ac, *Ti_Ac;            /* (nAc,nZ) */
  double *A_flow_mean_Ac;               /* (nAc) */
} ufe_physprop_out;
int ufe_ice_physical_properties(ufe_mesh_h mesh, const ufe_params *params, int flow_law, double time,
                                const double *Ti, ufe_physprop_out *out);

/* Upwind derivatives for the thermodynamics: get_upwind_derivative_vertex_3D
 * (mesh_derivatives_module.f90:434-483) for every vertex and layer on the device. Where the
 * wind (U_3D, V_3D) is below 1e-10 in both components, the Aa neighbour-function derivative;
 * otherwise the derivative on the first triangle around the vertex (iTri order) that holds the
 * point V(vi) - (U,V) R(vi) / (4 |(U,V)|) (is_in_triangle, mesh_help_functions_module.f90:646-672,
 * tolerance 1e-8). ufe_triangles_attach (after ufe_geometry_attach) uploads the reference's
 * triangle data once per mesh. U_3D and V_3D both NULL: those of the last ufe_sia3d_solve on the
 * device; d NULL: the Ti of the last ufe_ice_physical_properties (UFE_FLOW_ARRHENIUS). All 2-D
 * arrays are (nV,nZ). A pair (vertex, layer) with no upwind triangle gets 0 and is counted in
 * *no_upwind (may be NULL); the reference reports it and reads outside NxTri there. */
typedef struct ufe_triangle_mesh {
  int32_t nTri;
  const double *V;                      /* (nV,2) vertex coordinates */
  const double *R;                      /* (nV) mesh%R, the distance to the nearest neighbour */
  const int32_t *niTri, *iTri;          /* (nV), (nV,nC_mem) */
  const int32_t *Tri;                   /* (nTri,3) */
  const double *NxTri, *NyTri;          /* (nTri,3) */
} ufe_triangle_mesh;
int ufe_triangles_attach(ufe_mesh_h mesh, const ufe_triangle_mesh *triangles);
int ufe_upwind_derivatives_3d(ufe_mesh_h mesh, const ufe_params *params, const double *U_3D, const double *V_3D,
                              const double *d, double *ddx, double *ddy, int64_t *no_upwind);

/* calculate_ice_thickness_change (ice_dynamics_module.f90:31-237) on the device: upwind ice
 * volume fluxes across every Aa connection from Up_SIA_Ac + Up_SSA_Ac, the outflux rescale
 * against the available ice plus SMB and BMB, dHi/dt, the update of Hi (in place), the
 * domain-edge rule and the no-ice mask. NULL velocity arrays take the handle's last SSA / SIA
 * solution from the device (the velocities never leave it). Needs ufe_geometry_attach (the
 * mesh's C and Aci). */
typedef struct ufe_thickness_in {
  const double *A;                      /* (nV) Voronoi cell areas */
  const double *Cw;                     /* (nV,nC_mem) connection widths */
  const double *Up_SIA_Ac, *Up_SSA_Ac;  /* (nAc), or NULL: the handle's last solves */
  const double *SMB_year, *BMB;         /* (nV) */
  const int32_t *mask_noice;            /* (nV) or NULL */
  double dt;
  int32_t zero_edges;                   /* 1: Hi = 0 on domain-edge vertices (all configurations but SSA_icestream) */
} ufe_thickness_in;
typedef struct ufe_thickness_out {      /* host arrays, each may be NULL */
  double *Hi_prev, *dHi_dt;             /* (nV) */
  double *dVi_in;                       /* (nV,nC_mem) the rescaled fluxes */
} ufe_thickness_out;
int ufe_thickness_update(ufe_mesh_h mesh, const ufe_thickness_in *in, double *Hi, ufe_thickness_out *out);

/* VJP of the converged solve (no counterpart in the reference): for a misfit J(u) of the
 * velocities of the last ufe_ssa_solve / ufe_ssa_run on this handle, solves the adjoint
 * system (dF/du)^T mu = dJ/du of the discrete fixed point F(u) = 0 the Picard/SOR loop
 * converged to (viscosity and friction linearised at the converged state, Neumann rows as
 * averaging constraints, masks frozen) by a transposed coloured SOR on the device, and
 * returns dJ/d(log beta^2) on AaAc, the sensitivities to the gathered driving-stress slopes
 * and Hi_AaAc and, given the Aa and Ac derivative stencils, dJ/dHi on Aa. Both sliding laws:
 * the linear law (this library's extension, S = beta^2), and the reference's
 * Coulomb_regularised law (SSA_sliding_term, ice_dynamics_module.f90:745-751), whose S(u)
 * adds a 2x2 block per grounded row to the transposed sweep; under it dJ_dlogbeta_sq_AaAc
 * holds dJ/d(log tau_c) (tau_c the basal yield stress of basal_yield_stress, 780-844: S is
 * proportional to it), dJ_dphi_fric_AaAc dJ/d(phi_fric) in degrees, and the friction term
 * does not depend on Hi (tau_c and the friction denominator both carry max(0.1, Hi)). The
 * params' sliding law must be the last solve's. The grounding-line flux option is not
 * differentiated. Output arrays may be NULL.
 * The forward solve should be converged well below the tolerances the gradient is wanted
 * to (the VJP differentiates the fixed point, not the truncated iteration). */
enum { UFE_VJP_GMRES = 0, UFE_VJP_SOR = 1 };
typedef struct ufe_vjp_params {
  double tol;          /* GMRES: relative residual of the sweep-preconditioned system (0: 1e-12);
                          SOR: stop when max |update| < tol * max |mu| (0: 1e-13) */
  int32_t max_sweeps;  /* GMRES: iterations (0: 50000); SOR: sweeps (0: 2000000) */
  double omega;        /* 0: SSA_SOR_omega */
  int32_t method;      /* UFE_VJP_GMRES (default): restarted GMRES on the fixed-point map of
                          sweeps_per_iteration transposed sweeps (stops when a restart cycle
                          gains less than 5 %); UFE_VJP_SOR: plain sweeps */
  int32_t restart;     /* GMRES restart length (0: 100, at most 1000) */
  int32_t sweeps_per_iteration;  /* GMRES: transposed sweeps per Krylov iteration (0: 8) */
} ufe_vjp_params;
typedef struct ufe_vjp_in {
  const double *dJ_dU, *dJ_dV;          /* (nV) */
  const double *dJ_dUx_Ac, *dJ_dUy_Ac;  /* (nAc) */
} ufe_vjp_in;
typedef struct ufe_vjp_geom {           /* the type_mesh arrays of get_mesh_derivatives and _Ac */
  const int32_t *nC, *C;                /* (nV), (nV,nC_mem) */
  const double *Nx, *Ny;                /* (nV,nC_mem+1) Aa neighbour functions */
  const int32_t *Aci;                   /* (nAc,4) */
  const double *Nx_Ac, *Ny_Ac;          /* (nAc,4) */
} ufe_vjp_geom;
typedef struct ufe_vjp_out {
  double *dJ_dlogbeta_sq_AaAc;          /* (nVAaAc) */
  double *dJ_dHi;                       /* (nV), needs geom */
  double *dJ_dhx_AaAc, *dJ_dhy_AaAc, *dJ_dHi_AaAc;  /* (nVAaAc) sensitivities to the gathered fields */
  double *lambda_U_AaAc, *lambda_V_AaAc;            /* (nVAaAc) adjoint state */
  double *dJ_dphi_fric_AaAc;                        /* (nVAaAc) Coulomb law only */
} ufe_vjp_out;
typedef struct ufe_vjp_stats {
  int32_t status, sweeps;
  double last_rel_update, device_ms;
} ufe_vjp_stats;
int ufe_ssa_vjp(ufe_mesh_h mesh, const ufe_params *params, const ufe_vjp_params *vjp_params,
                const ufe_vjp_in *in, const ufe_vjp_geom *geom, ufe_vjp_out *out, ufe_vjp_stats *stats);

/* Batched ensemble (no counterpart in the reference, whose model runs one solve_SSA per
 * time step): many independent solves on meshes of uneven size (friction or rheology
 * ensembles) in one persistent cooperative launch. The grid is cut into teams of CTAs; a
 * member whose mesh is laid out in T spatial patches is solved by a team of T CTAs. Teams
 * of one size form a class with its own device queue (largest expected cost first), and
 * each class gets CTAs in proportion to its estimated work. With use_graph the whole batch
 * (gathers, the persistent solve, scatters) is captured once per parameter set and upload
 * state and replayed as a CUDA graph. Members share one ufe_params; their inputs are
 * uploaded one by one (the arrays of ufe_ssa_upload). In the mixed precision the members run
 * the halo sweeps of the single solves when the largest member's working copy fits beside the
 * CTAs the plan keeps resident (else the phased sweeps); either gives each member the result of
 * its single solve. */
typedef struct ufe_batch_s *ufe_batch_h;
typedef struct ufe_batch_config {
  int32_t team_ctas;     /* > 0: every member solved by a team of this many CTAs */
  int32_t rows_per_cta;  /* team_ctas == 0: member team = the power of two nearest above
                            rows / rows_per_cta (0: 8192 rows) - the per-CTA packing */
  int32_t block;         /* threads per CTA: 1024, 512 or 256 (0: 1024); 512 and 256 run 2 and 4 CTAs per SM */
  int32_t use_graph;     /* 1: capture and replay the batch as a CUDA graph */
} ufe_batch_config;
typedef struct ufe_batch_plan_out {
  int32_t n_classes;
  int32_t class_team_ctas[16];  /* team size of each class, largest first */
  int32_t class_teams[16];      /* teams of each class */
  int32_t grid_ctas;            /* CTAs of the persistent launch */
} ufe_batch_plan_out;
typedef struct ufe_batch_timing {
  double device_ms;      /* the whole batch on the device (CUDA events) */
  double solve_ms;       /* first member start to last member end inside the persistent kernel */
  double member_p50_ms, member_p99_ms, member_max_ms;  /* per-member solve time (team start to end) */
  double *member_ms;     /* (n_members) per-member solve time, or NULL */
  int32_t n_active, n_teams, n_classes, grid_ctas, max_team_ctas, block;
} ufe_batch_timing;
/* The planner alone (host only): team size of every member from its row count (nVAaAc)
 * and the classes' teams for `resident_ctas` co-resident CTAs. */
int ufe_batch_plan(const int32_t *rows, int32_t n_members, const ufe_batch_config *config,
                   int32_t resident_ctas, int32_t *team_ctas_of_member, ufe_batch_plan_out *plan);
int ufe_batch_create(const ufe_mesh_desc *descs, int32_t n_members, const ufe_batch_config *config,
                     ufe_batch_h *out);
int ufe_batch_destroy(ufe_batch_h batch);
int ufe_batch_upload(ufe_batch_h batch, int32_t member, const ufe_params *params, const ufe_ssa_in *in,
                     const ufe_ssa_inout *inout);
/* stats: (n_members) or NULL. Returns the most severe member status. */
int ufe_batch_run(ufe_batch_h batch, const ufe_params *params, ufe_ssa_stats *stats, ufe_batch_timing *timing);
int ufe_batch_download(ufe_batch_h batch, int32_t member, ufe_ssa_inout *inout, ufe_ssa_out *out);
/* Autotuner: times real batches of the given members over the per-CTA packing
 * (rows_per_cta 4096..24576 at 1024-thread CTAs), then the CTA size (512, 256) at the best
 * packing, then the neighbouring packings at the best CTA size, and returns the fastest
 * configuration. log (capacity entries) receives one entry
 * per candidate tried. Candidates that cannot hold the members are skipped. */
typedef struct ufe_batch_tune_entry {
  int32_t rows_per_cta, block, grid_ctas, n_classes;
  double device_ms, member_p99_ms;
} ufe_batch_tune_entry;
int ufe_batch_autotune(int32_t n_members, const ufe_mesh_desc *descs, const ufe_params *params,
                       const ufe_ssa_in *in, const ufe_ssa_inout *inout, ufe_batch_config *best,
                       ufe_batch_tune_entry *log, int32_t log_capacity, int32_t *log_count);
/* One call for a Fortran caller: create, upload, run, download and destroy. in, inout,
 * out and stats are arrays of n_members (out and stats may be NULL). */
int ufe_ssa_solve_batched(int32_t n_members, const ufe_mesh_desc *descs, const ufe_batch_config *config,
                          const ufe_params *params, const ufe_ssa_in *in, ufe_ssa_inout *inout,
                          ufe_ssa_out *out, ufe_ssa_stats *stats);

/* Host-side mesh substrate: builds the Ac and combined AaAc mesh, the AaAc and Aa
 * neighbour functions and the five-colouring from a base triangulation, exactly as
 * make_Ac_mesh (mesh_ArakawaC_module.f90:24-540), get_neighbour_functions
 * (mesh_derivatives_module.f90:14-313) and calculate_five_colouring_AaAc
 * (mesh_five_colour_module.f90:18-735) do. For callers that do not run the reference's
 * Fortran mesh code. Output arrays are caller-allocated with nAc = nV + nTri - 1 and
 * nVAaAc = nV + nAc; any output pointer may be NULL except those the later steps need. */
typedef struct ufe_base_mesh {
  int32_t nV, nTri, nC_mem;
  const double *V;             /* (nV,2) */
  const int32_t *nC, *C;       /* (nV), (nV,nC_mem) */
  const int32_t *niTri, *iTri; /* (nV), (nV,nC_mem) */
  const int32_t *Tri;          /* (nTri,3) */
  const int32_t *edge_index;   /* (nV) */
} ufe_base_mesh;

typedef struct ufe_aaac_mesh {
  int32_t nAc, nVAaAc;
  double *Nx, *Ny, *Nxx, *Nxy, *Nyy;   /* (nV,nC_mem+1) Aa neighbour functions */
  int32_t *iAci, *Aci;                 /* (nV,nC_mem), (nAc,4) */
  double *VAc;                         /* (nAc,2) */
  double *Nx_Ac, *Ny_Ac, *No_Ac;       /* (nAc,4) */
  double *Np_Ac;                       /* (nAc) */
  int32_t *edge_index_Ac;              /* (nAc) */
  double *VAaAc;                       /* (nVAaAc,2) */
  int32_t *nCAaAc, *CAaAc;             /* (nVAaAc), (nVAaAc,nC_mem) */
  double *Nx_AaAc, *Ny_AaAc, *Nxx_AaAc, *Nxy_AaAc, *Nyy_AaAc; /* (nVAaAc,nC_mem+1) */
  int32_t *colour, *colour_vi, *colour_nV; /* (nVAaAc), (nVAaAc,5), (5) */
} ufe_aaac_mesh;

int ufe_aaac_build(const ufe_base_mesh *base, ufe_aaac_mesh *out);

#ifdef __cplusplus
}
#endif
#endif /* UFEMISM_GB300_H */
